"""Python face of the oracle (TEST INFRASTRUCTURE ONLY).

The oracle checks the GPU path: ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU-baseline leg may import it; the product package never does.

Two backends live here, both restating / running the reference's hot path:

* ``port``      -- ``oracle/mmd_oracle.c`` (``liboracle.so``): a plain-C restatement
                   of cython/util.pxi, cython/twoe.pyx, cython/basis.pxi and
                   cython/fock.pyx, function by function.
* ``reference`` -- the reference's own Cython modules compiled by
                   ``oracle/build_ref.py`` into ``oracle/_ref`` (when present).

Both expose the reference's call signatures: ``Basis(origin, shell, num_exps,
exps, coefs)``, ``ERI(a, b, c, d)``, ``doERIs(N, TwoE, bfs)``, ``formPT(P, P_old,
bfs, nbasis, screen, tol)`` and ``boys(m, T)``.
"""
from __future__ import annotations

import ctypes
import importlib
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def build() -> str:
    """Compile liboracle.so (gcc) if it is missing or stale."""
    so = os.path.join(HERE, "liboracle.so")
    src = os.path.join(HERE, "mmd_oracle.c")
    if not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", HERE, "liboracle.so"])
    return so


def lib():
    global _LIB
    if _LIB is None:
        L = ctypes.CDLL(build())
        d, l, p = ctypes.c_double, ctypes.c_long, ctypes.c_void_p
        L.oracle_boys.restype = d
        L.oracle_boys.argtypes = [d, d]
        L.oracle_E.restype = d
        L.oracle_E.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, d, d, d]
        L.oracle_normalize.restype = None
        L.oracle_normalize.argtypes = [p, l, p, p, p]
        L.oracle_eri_flat.restype = d
        L.oracle_eri_flat.argtypes = [p, l, l, l, l]
        L.oracle_doERIs.restype = None
        L.oracle_doERIs.argtypes = [l, p, p]
        L.oracle_screen.restype = None
        L.oracle_screen.argtypes = [l, p, p]
        L.oracle_formPT.restype = l
        L.oracle_formPT.argtypes = [l, p, p, p, p, d, p]
        _LIB = L
    return _LIB


class _Flat(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("origin", "shell", "nprim", "off", "exps", "coefs", "norm")]


class Basis:
    """Contracted Cartesian Gaussian, normalised as cython/basis.pxi:87-120."""

    def __init__(self, origin, shell, num_exps, exps, coefs):
        self.origin = np.ascontiguousarray(origin, dtype=np.float64).reshape(3).copy()
        self.shell = np.ascontiguousarray(shell, dtype=np.int64).reshape(3).copy()
        self.num_exps = int(num_exps)
        self.exps = np.ascontiguousarray(exps, dtype=np.float64)[: self.num_exps].copy()
        self.coefs = np.ascontiguousarray(coefs, dtype=np.float64)[: self.num_exps].copy()
        self.norm = np.zeros(self.num_exps)
        lib().oracle_normalize(self.shell.ctypes.data, self.num_exps, self.exps.ctypes.data,
                               self.coefs.ctypes.data, self.norm.ctypes.data)


class _Pack:
    """Flat arrays for a list of Basis-like objects (anything with the reference's attributes)."""

    def __init__(self, bfs):
        n = len(bfs)
        self.origin = np.zeros((n, 3))
        self.shell = np.zeros((n, 3), dtype=np.int64)
        self.nprim = np.zeros(n, dtype=np.int64)
        self.off = np.zeros(n, dtype=np.int64)
        exps, coefs, norm = [], [], []
        o = 0
        for f, b in enumerate(bfs):
            self.origin[f] = np.asarray(b.origin, dtype=np.float64)
            self.shell[f] = np.asarray(b.shell, dtype=np.int64)
            k = int(b.num_exps)
            self.nprim[f] = k
            self.off[f] = o
            o += k
            exps.append(np.asarray(b.exps, dtype=np.float64)[:k])
            coefs.append(np.asarray(b.coefs, dtype=np.float64)[:k])
            norm.append(np.asarray(b.norm, dtype=np.float64)[:k])
        self.exps = np.ascontiguousarray(np.concatenate(exps)) if exps else np.zeros(1)
        self.coefs = np.ascontiguousarray(np.concatenate(coefs)) if coefs else np.zeros(1)
        self.norm = np.ascontiguousarray(np.concatenate(norm)) if norm else np.zeros(1)
        self.flat = _Flat(*(a.ctypes.data for a in (self.origin, self.shell, self.nprim, self.off,
                                                      self.exps, self.coefs, self.norm)))

    @property
    def ptr(self):
        return ctypes.addressof(self.flat)


def boys(m, T) -> float:
    return lib().oracle_boys(float(m), float(T))


def ERI(a, b, c, d) -> float:
    pk = _Pack([a, b, c, d])
    return lib().oracle_eri_flat(pk.ptr, 0, 1, 2, 3)


def doERIs(N, TwoE, bfs):
    pk = _Pack(bfs)
    out = np.zeros((N, N, N, N))
    lib().oracle_doERIs(int(N), out.ctypes.data, pk.ptr)
    TwoE[...] = out
    return TwoE


def screen_table(bfs) -> np.ndarray:
    """Flat Schwarz table screen[p(p+1)/2+q] = (pq|pq) (mmd/molecule.py:95-99)."""
    pk = _Pack(bfs)
    N = len(bfs)
    out = np.zeros(N * (N + 1) // 2)
    lib().oracle_screen(N, pk.ptr, out.ctypes.data)
    return out


def formPT(P, P_old, bfs, nbasis, screen, tol):
    """formPT (cython/fock.pyx:13-87) for a real density; returns complex G like the reference."""
    N = int(nbasis)
    P = np.asarray(P)
    P_old = np.asarray(P_old)
    assert np.all(np.imag(P) == 0) and np.all(np.imag(P_old) == 0), "oracle formPT handles real densities"
    Pr = np.ascontiguousarray(np.real(P), dtype=np.float64)
    Po = np.ascontiguousarray(np.real(P_old), dtype=np.float64)
    if isinstance(screen, dict):
        scr = np.array([screen[i] for i in range(N * (N + 1) // 2)], dtype=np.float64)
    else:
        scr = np.ascontiguousarray(screen, dtype=np.float64)
    G = np.zeros((N, N))
    pk = _Pack(bfs)
    lib().oracle_formPT(N, pk.ptr, Pr.ctypes.data, Po.ctypes.data, scr.ctypes.data, float(tol), G.ctypes.data)
    return G.astype(complex)


def reference_modules():
    """Import the compiled reference modules from oracle/_ref (None if not built)."""
    ref = os.path.join(HERE, "_ref")
    if not os.path.isdir(os.path.join(ref, "mmd", "integrals")):
        return None
    if ref not in sys.path:
        sys.path.insert(0, ref)
    try:
        twoe = importlib.import_module("mmd.integrals.twoe")
        fock = importlib.import_module("mmd.integrals.fock")
    except ImportError:
        return None
    return twoe, fock
