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
        L.oracle_formPT_part.restype = l
        L.oracle_formPT_part.argtypes = [l, p, p, p, p, d, p, l, l, p, p, ctypes.c_int]
        L.oracle_formPT_table.restype = l
        L.oracle_formPT_table.argtypes = [l, p, p, p, p, d, p]
        L.oracle_eri_unique.restype = None
        L.oracle_eri_unique.argtypes = [l, p, l, l, p]
        L.oracle_eri_shell.restype = None
        L.oracle_eri_shell.argtypes = [p, p, l, p, l, p, l, p, l, p]
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


# ------------------------------------------------------------------ partial / parallel forms
def formPT_part(P, P_old, bfs, nbasis, screen, tol, ij_lo=0, ij_hi=None, func_shell=None, owner=None, part=0):
    """formPT restricted to canonical bra pairs ij in [ij_lo, ij_hi) and, with
    ``owner`` (per canonical shell-pair index s1(s1+1)/2+s2) and ``func_shell`` (shell
    of every function), to the shell quartets owned by ``part`` (the owner of the
    quartet's pair with the larger canonical index).  Returns the real partial G."""
    N = int(nbasis)
    npair = N * (N + 1) // 2
    ij_hi = npair if ij_hi is None else int(ij_hi)
    Pr = np.ascontiguousarray(np.real(np.asarray(P)), dtype=np.float64)
    Po = np.ascontiguousarray(np.real(np.asarray(P_old)), dtype=np.float64)
    if isinstance(screen, dict):
        scr = np.array([screen[i] for i in range(npair)], dtype=np.float64)
    else:
        scr = np.ascontiguousarray(screen, dtype=np.float64)
    G = np.zeros((N, N))
    pk = _Pack(bfs)
    fs = ow = None
    if owner is not None:
        fs = np.ascontiguousarray(func_shell, dtype=np.int64)
        ow = np.ascontiguousarray(owner, dtype=np.int32)
    lib().oracle_formPT_part(N, pk.ptr, Pr.ctypes.data, Po.ctypes.data, scr.ctypes.data, float(tol), G.ctypes.data,
                             int(ij_lo), ij_hi, None if fs is None else fs.ctypes.data,
                             None if ow is None else ow.ctypes.data, int(part))
    return G


def formPT_table(P, P_old, eri_table, nbasis, screen, tol):
    """formPT (cython/fock.pyx:13-87) reading the ERIs from ``eri_table``, the unique
    quartets in doERIs loop order (``eri_unique`` / ``parallel_eri_unique``); real G."""
    N = int(nbasis)
    npair = N * (N + 1) // 2
    tab = np.ascontiguousarray(eri_table, dtype=np.float64)
    assert tab.size == npair * (npair + 1) // 2
    Pr = np.ascontiguousarray(np.real(np.asarray(P)), dtype=np.float64)
    Po = np.ascontiguousarray(np.real(np.asarray(P_old)), dtype=np.float64)
    scr = np.ascontiguousarray([screen[i] for i in range(npair)] if isinstance(screen, dict) else screen,
                               dtype=np.float64)
    G = np.zeros((N, N))
    lib().oracle_formPT_table(N, tab.ctypes.data, Pr.ctypes.data, Po.ctypes.data, scr.ctypes.data, float(tol),
                              G.ctypes.data)
    return G


def eri_unique(bfs, ij_lo, ij_hi):
    """The unique ERIs (ij|kl), kl <= ij, for canonical ij in [ij_lo, ij_hi), in doERIs
    loop order (twoe.pyx:12-31)."""
    N = len(bfs)
    n = sum(ij + 1 for ij in range(int(ij_lo), int(ij_hi)))
    out = np.zeros(max(n, 1))
    pk = _Pack(bfs)
    lib().oracle_eri_unique(N, pk.ptr, int(ij_lo), int(ij_hi), out.ctypes.data)
    return out[:n]


def eri_shell(bfs, fa, fb, fc, fd, pack=None):
    """All component ERIs of four shells given as function-index lists (each list one
    Cartesian shell: same origin and exponents); array [len(fa), len(fb), len(fc), len(fd)],
    equal bit for bit to ERI() per function quartet.  ``pack`` (a _Pack of ``bfs``)
    saves re-packing the basis on every call."""
    arrs = [np.ascontiguousarray(x, dtype=np.int64) for x in (fa, fb, fc, fd)]
    out = np.zeros(tuple(len(a) for a in arrs))
    pk = pack if pack is not None else _Pack(bfs)
    lib().oracle_eri_shell(pk.ptr, arrs[0].ctypes.data, len(arrs[0]), arrs[1].ctypes.data, len(arrs[1]),
                           arrs[2].ctypes.data, len(arrs[2]), arrs[3].ctypes.data, len(arrs[3]), out.ctypes.data)
    return out


class _Plain:
    """A Basis-like record carrying already-normalised data (no renormalisation)."""

    def __init__(self, origin, shell, num_exps, exps, coefs, norm):
        self.origin, self.shell, self.num_exps = origin, shell, num_exps
        self.exps, self.coefs, self.norm = exps, coefs, norm


def _plain(bfs):
    return [(list(map(float, b.origin)), [int(x) for x in b.shell], int(b.num_exps),
             list(map(float, np.asarray(b.exps)[: int(b.num_exps)])),
             list(map(float, np.asarray(b.coefs)[: int(b.num_exps)])),
             list(map(float, np.asarray(b.norm)[: int(b.num_exps)]))) for b in bfs]


_WB = None


def _w_init(data):
    global _WB
    _WB = [_Plain(*t) for t in data]


def _w_formPT(args):
    P, Po, N, scr, tol, lo, hi = args
    return formPT_part(P, Po, _WB, N, scr, tol, lo, hi)


def _w_unique(args):
    lo, hi = args
    return eri_unique(_WB, lo, hi)


def _w_shell(args):
    pk = _Pack(_WB)
    return [eri_shell(_WB, *q, pack=pk) for q in args]


def _w_shell_unique(args):
    """Unique-ERI positions (doERIs loop order) and values of a chunk of shell
    quartets: every component of each block, mapped to its canonical (ij|kl)."""
    quartets, shells = args
    pk = _Pack(_WB)
    pos, val = [], []
    for q in quartets:
        fl = [shells[s] for s in q]
        blk = eri_shell(_WB, *fl, pack=pk)
        i, j, k, l = (x.ravel() for x in np.meshgrid(*[np.asarray(f, dtype=np.int64) for f in fl], indexing="ij"))
        ij = np.where(i >= j, i * (i + 1) // 2 + j, j * (j + 1) // 2 + i)
        kl = np.where(k >= l, k * (k + 1) // 2 + l, l * (l + 1) // 2 + k)
        hi, lo = np.maximum(ij, kl), np.minimum(ij, kl)
        pos.append(hi * (hi + 1) // 2 + lo)
        val.append(blk.ravel())
    return np.concatenate(pos), np.concatenate(val)


def _ij_ranges(N, parts):
    """Contiguous canonical-ij ranges holding about equal numbers of quartets (ij+1 each)."""
    npair = N * (N + 1) // 2
    cum = np.cumsum(np.arange(1, npair + 1, dtype=np.float64))
    cuts = [0] + [int(np.searchsorted(cum, cum[-1] * k / parts)) for k in range(1, parts)] + [npair]
    return [(a, b) for a, b in zip(cuts[:-1], cuts[1:]) if b > a]


def _pool(bfs, nproc):
    import multiprocessing as mp
    nproc = int(nproc or os.cpu_count() or 1)
    # spawn: safe after CUDA has been initialised in the parent
    return mp.get_context("spawn").Pool(nproc, initializer=_w_init, initargs=(_plain(bfs),)), nproc


def parallel_formPT(P, P_old, bfs, nbasis, screen, tol, nproc=None):
    """formPT over every function quartet, split into ij ranges over processes; real G."""
    N = int(nbasis)
    scr = np.array([screen[i] for i in range(N * (N + 1) // 2)]) if isinstance(screen, dict) else np.asarray(screen)
    pool, n = _pool(bfs, nproc)
    with pool:
        parts = pool.map(_w_formPT, [(np.real(P), np.real(P_old), N, scr, tol, lo, hi)
                                     for lo, hi in _ij_ranges(N, 4 * n)])
    return np.sum(parts, axis=0)


def parallel_eri_unique(bfs, nproc=None):
    """All unique ERIs of doERIs in loop order, computed over processes."""
    N = len(bfs)
    pool, n = _pool(bfs, nproc)
    with pool:
        parts = pool.map(_w_unique, _ij_ranges(N, 4 * n))
    return np.concatenate(parts)


def parallel_eri_unique_shells(bfs, shells, nproc=None):
    """The vector of parallel_eri_unique (every unique ERI in doERIs loop order) from
    shell blocks: ``shells`` lists each shell's function indices (contiguous, in
    function order); every shell quartet with the larger shell pair first is
    evaluated once by eri_shell (memoised E and R, equal bit for bit to ERI for the
    block's own function order) and each component lands at its canonical position.
    A canonical quartet whose block holds it in another function order (the same
    integral by permutational symmetry) may differ from ERI in the last bits."""
    N = len(bfs)
    shells = [[int(f) for f in sh] for sh in shells]
    pairs = [(a, b) for a in range(len(shells)) for b in range(a + 1)]
    quartets = [pairs[p] + pairs[r] for p in range(len(pairs)) for r in range(p + 1)]
    pool, n = _pool(bfs, nproc)
    chunks = [(quartets[k::8 * n], shells) for k in range(8 * n)]
    with pool:
        res = pool.map(_w_shell_unique, chunks)
    npair = N * (N + 1) // 2
    out = np.full(npair * (npair + 1) // 2, np.nan)
    for pos, val in res:
        out[pos] = val
    if np.isnan(out).any():
        raise ValueError("parallel_eri_unique_shells: the shells do not cover every function")
    return out


def parallel_eri_shells(bfs, quartets, nproc=None):
    """eri_shell for a list of (fa, fb, fc, fd) function-index lists, over processes."""
    pool, n = _pool(bfs, nproc)
    chunks = [quartets[k::4 * n] for k in range(4 * n)]
    with pool:
        res = pool.map(_w_shell, chunks)
    out = [None] * len(quartets)
    for k, r in enumerate(res):
        for m, v in enumerate(r):
            out[k + m * 4 * n] = v
    return out


def unique_index(N):
    """(i, j, k, l) arrays of the unique quartets in doERIs loop order (ij ascending,
    then kl = 0..ij), matching eri_unique / parallel_eri_unique."""
    ii, jj = np.tril_indices(N)
    order = np.argsort(ii * (ii + 1) // 2 + jj, kind="stable")
    ii, jj = ii[order], jj[order]
    npair = len(ii)
    a, b = np.tril_indices(npair)  # a = ij (row), b = kl <= ij, row-major: ij ascending then kl
    return ii[a], jj[a], ii[b], jj[b]
