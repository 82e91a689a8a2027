"""gm_close_noalloc: the closing for callers that are not allowed to call
cudaMalloc (a host application that owns the GPU memory budget, or a
latency-bound loop that cannot take cudaMalloc's implicit synchronisation).

Called through the C ABI, it must give the same grids as gm_close (bit for
bit: the closing is integer work) on two calls in a row, which also checks
that the shared scratch array left over from the previous call does not leak
into the next one.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from broxy_gb300 import _lib as L
from broxy_gb300 import api, synth

pytestmark = pytest.mark.gpu


def _noalloc(desc, X, R, r, mode, se, out, D, S):
    import torch
    st = L.load().gm_close_noalloc(C.byref(desc), C.c_void_p(X.data_ptr()),
                                   C.c_void_p(R.data_ptr()) if R is not None else None, r, mode, se,
                                   C.c_void_p(out.data_ptr()), C.c_void_p(D.data_ptr()), C.c_void_p(S.data_ptr()),
                                   C.c_void_p(torch.cuda.current_stream().cuda_stream))
    return st


@pytest.mark.parametrize("res,variable,mode", [(32, True, L.GM_REF), (64, False, L.GM_REF), (64, True, L.GM_EXACT)])
def test_noalloc_matches_gm_close_twice(res, variable, mode):
    import torch
    ctx = api.Context(0)
    desc = api.make_desc(res)
    for call in range(2):  # two calls in a row, different inputs
        X = torch.as_tensor(synth.random_grid(res, 900 + 10 * call + res)).cuda()
        R = None
        if variable:
            rng = np.random.default_rng(call + res)
            R = torch.as_tensor(rng.integers(-2, 9, size=(2 * res) ** 3).astype(np.int8)).cuda()
        ref_D, ref_S = torch.empty_like(X), torch.empty_like(X)
        ref = ctx.close(desc, X, R, 5, mode, L.GM_SE_SPHERE, D=ref_D, S=ref_S)
        out, D, S = torch.full_like(X, 7), torch.full_like(X, 7), torch.full_like(X, 7)
        assert _noalloc(desc, X, R, 5, mode, L.GM_SE_SPHERE, out, D, S) == L.GM_OK
        torch.cuda.synchronize()
        assert torch.equal(out, ref)
        assert torch.equal(D, ref_D)
        assert torch.equal(S, ref_S)
    ctx.close_ctx()


def test_noalloc_rejects_grids_beyond_its_scratch():
    import torch
    res = 128
    desc = api.make_desc(res)
    X = torch.zeros(res ** 3, dtype=torch.uint8, device="cuda")
    out = torch.empty_like(X)
    assert _noalloc(desc, X, None, 4, L.GM_REF, L.GM_SE_SPHERE, out, out, out) == L.GM_ERR_CAPACITY
