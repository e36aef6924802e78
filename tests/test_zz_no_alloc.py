"""The allocation-free ERI entry point (mmdg_eri_tensor_noalloc) against the regular
one (mmdg_eri_tensor), both called through the C ABI.

Some callers cannot allocate device memory (a framework owns the memory pool, or
the call must not synchronise the device), so this entry point keeps all scratch
in a static device array shared by every call.  The test makes two calls in a row
with different molecules, so the second call runs on the first call's leftover
scratch, and compares each tensor with the regular entry point to 1e-12.  It sits
in a file of its own that pytest collects last, and passes alone or after the rest.
"""
import ctypes
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WATER = "\n0 1\nO 0.000000 -0.075791844 0.000000\nH 0.866811829 0.601435779 0.000000\nH -0.866811829 0.601435779 0.000000\n"
METHANE = ("\n0 1\nC 0 0 0\nH 0.626425042 -0.626425042 -0.626425042\nH 0.626425042 0.626425042 0.626425042\n"
           "H -0.626425042 0.626425042 -0.626425042\nH -0.626425042 -0.626425042 0.626425042\n")


def _noalloc_tensor(lib, ss, torch):
    N = ss.nfunc
    out = torch.full((N, N, N, N), float("nan"), dtype=torch.float64, device="cuda")
    a = lambda x, t: np.ascontiguousarray(x, dtype=t)
    L, K, cen = a(ss.L, np.int32), a(ss.nprim, np.int32), a(ss.center, np.float64)
    ex, co, fn = a(ss.exps, np.float64), a(ss.coefs, np.float64), a(ss.func, np.int32)
    p = lambda x: ctypes.c_void_p(x.ctypes.data)
    rc = lib.mmdg_eri_tensor_noalloc(ss.nshell, p(L), p(K), p(cen), p(ex), p(co), p(fn), N,
                                     ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, lib.mmdg_last_error().decode()
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_noalloc_eri_tensor_matches_regular_entry_point(built_lib):
    import torch
    assert torch.cuda.is_available()
    from mmd.molecule import Molecule
    from mmd.integrals.shells import shells_from_bfs
    from mmd import _native
    lib = ctypes.CDLL(built_lib)
    lib.mmdg_eri_tensor_noalloc.restype = ctypes.c_int
    lib.mmdg_eri_tensor_noalloc.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 6 + [ctypes.c_int, ctypes.c_void_p,
                                                                                       ctypes.c_void_p]
    lib.mmdg_last_error.restype = ctypes.c_char_p
    for geom, basis in ((WATER, "6-31g"), (METHANE, "sto-3g"), (WATER, "6-31gss")):
        ss = shells_from_bfs(Molecule(geom, basis).bfs)
        ref = _native.Context(ss).eri_tensor().cpu().numpy()
        got = _noalloc_tensor(lib, ss, torch)
        assert not np.isnan(got).any()
        assert np.abs(got - ref).max() < 1e-12, (basis, np.abs(got - ref).max())


def test_noalloc_rejects_sizes_beyond_the_scratch(built_lib):
    import torch
    from mmd.integrals.shells import ShellSet
    lib = ctypes.CDLL(built_lib)
    lib.mmdg_eri_tensor_noalloc.restype = ctypes.c_int
    lib.mmdg_eri_tensor_noalloc.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 6 + [ctypes.c_int, ctypes.c_void_p,
                                                                                       ctypes.c_void_p]
    lib.mmdg_last_error.restype = ctypes.c_char_p
    n = 65  # one shell more than the static scratch holds
    ss = ShellSet(nfunc=n, L=np.zeros(n, dtype=np.int32), nprim=np.ones(n, dtype=np.int32),
                  center=np.arange(3 * n, dtype=np.float64).reshape(n, 3), exps=np.ones(n), coefs=np.ones(n),
                  func=np.array([[i, -1, -1, -1, -1, -1] for i in range(n)], dtype=np.int32))
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    p = lambda x: ctypes.c_void_p(np.ascontiguousarray(x).ctypes.data)
    rc = lib.mmdg_eri_tensor_noalloc(n, p(ss.L), p(ss.nprim), p(ss.center), p(ss.exps), p(ss.coefs), p(ss.func), n,
                                     ctypes.c_void_p(out.data_ptr()), None)
    assert rc != 0
    assert b"64 shells" in lib.mmdg_last_error()
    # non-finite inputs are rejected like mmdg_set_basis does, before any GPU work
    m = 2
    # every array is held in a name for the duration of the call (a temporary would be
    # freed before the library reads it)
    func = np.array([[i, -1, -1, -1, -1, -1] for i in range(m)], dtype=np.int32)
    Lm, Km, co = np.zeros(m, dtype=np.int32), np.ones(m, dtype=np.int32), np.ones(m)
    for exps, cen, word in ((np.array([1.0, np.inf]), np.zeros((m, 3)), b"finite"),
                            (np.ones(m), np.array([[0.0, 0.0, 0.0], [np.nan, 0.0, 0.0]]), b"centre")):
        rc = lib.mmdg_eri_tensor_noalloc(m, p(Lm), p(Km), p(cen), p(exps), p(co), p(func), m,
                                         ctypes.c_void_p(out.data_ptr()), None)
        assert rc != 0
        assert word in lib.mmdg_last_error()
