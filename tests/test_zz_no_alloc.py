"""gm_close_noalloc: the closing for callers that are not allowed to call
cudaMalloc (a host application that owns the GPU memory budget, or a
latency-bound loop that cannot take cudaMalloc's implicit synchronisation).

Called through the C ABI, it must give the same grids as gm_close (bit for
bit: the closing is integer work) on two calls in a row, which also checks
that the shared scratch array left over from the previous call does not leak
into the next one.  A repeated call must leave the device's free memory and
torch's allocation count unchanged.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from broxy_gb300 import _lib as L
from broxy_gb300 import api, synth

pytestmark = pytest.mark.gpu


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _noalloc(desc, X, R, r, mode, se, out, D, S):
    import torch
    return L.load().gm_close_noalloc(C.byref(desc), _ptr(X), _ptr(R), r, mode, se, _ptr(out), _ptr(D), _ptr(S),
                                     C.c_void_p(torch.cuda.current_stream().cuda_stream))


def _inputs(res, call, variable):
    import torch
    X = torch.as_tensor(synth.random_grid(res, 900 + 10 * call + res)).cuda()
    R = None
    if variable:
        rng = np.random.default_rng(call + res)
        R = torch.as_tensor(rng.integers(-2, 9, size=(2 * res) ** 3).astype(np.int8)).cuda()
    return X, R


@pytest.mark.parametrize("res,variable,mode,se,outs", [
    (32, True, L.GM_REF, L.GM_SE_SPHERE, True),
    (64, False, L.GM_REF, L.GM_SE_SPHERE, True),
    (64, True, L.GM_EXACT, L.GM_SE_SPHERE, True),
    (32, True, L.GM_REF, L.GM_SE_CUBE, True),
    (16, False, L.GM_REF, L.GM_SE_SPHERE, False),
    (64, True, L.GM_REF, L.GM_SE_CUBE, False),
])
def test_noalloc_matches_gm_close_twice(res, variable, mode, se, outs):
    import torch
    ctx = api.Context(0)
    desc = api.make_desc(res)
    for call in range(2):  # two calls in a row, different inputs
        X, R = _inputs(res, call, variable)
        ref_D, ref_S = torch.empty_like(X), torch.empty_like(X)
        ref = ctx.close(desc, X, R, 5, mode, se, D=ref_D, S=ref_S)
        out = torch.full_like(X, 7)
        D = torch.full_like(X, 7) if outs else None
        S = torch.full_like(X, 7) if outs else None
        assert _noalloc(desc, X, R, 5, mode, se, out, D, S) == L.GM_OK
        torch.cuda.synchronize()
        assert torch.equal(out, ref)
        if outs:
            assert torch.equal(D, ref_D)
            assert torch.equal(S, ref_S)
    ctx.close_ctx()


@pytest.mark.parametrize("variable", [False, True])
def test_noalloc_allocates_nothing(variable):
    import torch
    res = 64
    desc = api.make_desc(res)
    X0, R0 = _inputs(res, 0, variable)
    X1, R1 = _inputs(res, 1, variable)
    out = torch.empty_like(X0)
    # warm-up: the first call of a configuration loads its kernels
    assert _noalloc(desc, X0, R0, 6, L.GM_REF, L.GM_SE_SPHERE, out, None, None) == L.GM_OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    alloc0 = torch.cuda.memory_allocated()
    assert _noalloc(desc, X1, R1, 6, L.GM_REF, L.GM_SE_SPHERE, out, None, None) == L.GM_OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert torch.cuda.memory_allocated() == alloc0


def test_noalloc_rejects_grids_beyond_its_scratch():
    import torch
    res = 128
    desc = api.make_desc(res)
    X = torch.zeros(res ** 3, dtype=torch.uint8, device="cuda")
    out = torch.empty_like(X)
    assert _noalloc(desc, X, None, 4, L.GM_REF, L.GM_SE_SPHERE, out, out, out) == L.GM_ERR_CAPACITY
