"""Runs the reference GMorpho build (oracle/_ref/libgmref.so) on one input,
in a process of its own, so that a fault of the reference code stays out of
the test session.  TEST INFRASTRUCTURE ONLY.

    python run_ref.py in.npz out.npz

in.npz: X (uint8 res^3), R (int8 (2 res)^3), res, data_res (3), se (0 sphere,
1 cube), cap_v, cap_t.  out.npz: rc, err, D, S, C, V, N, T.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(os.path.dirname(HERE), "_ref", "libgmref.so")


def _ptr(a):
    return C.c_void_p(a.ctypes.data)


def run(inp, out):
    d = np.load(inp)
    X = np.ascontiguousarray(d["X"], np.uint8)
    R = np.ascontiguousarray(d["R"], np.int8)
    res, se = int(d["res"]), int(d["se"])
    dr = np.ascontiguousarray(d["data_res"], np.int32)
    cap_v, cap_t = int(d["cap_v"]), int(d["cap_t"])
    lib = C.CDLL(LIB, mode=os.RTLD_NOW)
    P = C.c_void_p
    lib.gmref_update.argtypes = [P, P, C.c_int, P, C.c_int, C.c_int, P, P, P, P, P, P, C.c_int64, C.c_int64, P, P,
                                 C.c_char_p, C.c_int]
    lib.gmref_update.restype = C.c_int
    n = res ** 3
    D, S, Cg = np.zeros(n, np.uint8), np.zeros(n, np.uint8), np.zeros(n, np.uint8)
    V, N = np.zeros((cap_v, 3), np.float32), np.zeros((cap_v, 3), np.float32)
    T = np.zeros((cap_t, 3), np.uint32)
    nv, nt = C.c_int64(0), C.c_int64(0)
    err = C.create_string_buffer(512)
    rc = lib.gmref_update(_ptr(X), _ptr(R), res, _ptr(dr), se, 1, _ptr(D), _ptr(S), _ptr(Cg), _ptr(V), _ptr(N),
                          _ptr(T), cap_v, cap_t, C.byref(nv), C.byref(nt), err, 512)
    nv, nt = nv.value, nt.value
    ok = rc == 0 and nv <= cap_v and nt <= cap_t
    np.savez(out, rc=rc, err=err.value.decode(errors="replace"), nv=nv, nt=nt, D=D, S=S, C=Cg,
             V=V[:nv] if ok else V[:0], N=N[:nv] if ok else N[:0], T=T[:nt] if ok else T[:0])
    return rc


if __name__ == "__main__":
    sys.exit(0 if run(sys.argv[1], sys.argv[2]) == 0 else 1)
