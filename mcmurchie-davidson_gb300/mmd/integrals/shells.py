"""Shells from the reference's per-function basis lists.

The reference keeps one ``Basis`` object per Cartesian function
(cython/basis.pxi:6-44), emitted by ``Molecule.formBasis`` atom by atom, shell by
shell, component by component in the order of ``momentum2shell``
(mmd/molecule.py:63-73,108-114).  The GPU kernels work on shells, so consecutive
functions that share origin, angular momentum, exponents and (component-free)
contraction weights are grouped back into one shell.  Any list works: a function
that cannot join a shell becomes a shell of its own whose other components are
marked absent (-1) and never digested.

Per-primitive weights: the reference's weight of primitive k of function
(l,m,n) is ``norm[k] * coefs[k]`` with
    norm[k] = sqrt(2^(2L+1.5) a^(L+1.5) / ((2l-1)!!(2m-1)!!(2n-1)!! pi^1.5))
(basis.pxi:101-105) and the contracted normalisation folded into coefs
(basis.pxi:109-120).  The double factorials only enter through the component
factor n(l,m,n) = 1/sqrt((2l-1)!!(2m-1)!!(2n-1)!!), which the pair kernel applies;
the shell stores ``norm[k]*coefs[k] / n(l,m,n)``, identical for all components.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

LMAX = 2
MAX_COMP = 6


def components(l: int):
    """Cartesian components in the reference's order (mmd/molecule.py:108-114)."""
    return [(x, y, l - x - y) for x in range(l, -1, -1) for y in range(l - x, -1, -1)]


_COMP_INDEX = {l: {c: k for k, c in enumerate(components(l))} for l in range(4)}


def _fact2_odd(k: int) -> float:
    r = 1.0
    while k > 1:
        r *= k
        k -= 2
    return r


def comp_norm(lmn) -> float:
    l, m, n = (int(x) for x in lmn)
    return 1.0 / np.sqrt(_fact2_odd(2 * l - 1) * _fact2_odd(2 * m - 1) * _fact2_odd(2 * n - 1))


@dataclass
class ShellSet:
    """The shells of one molecule's basis, in the flat layout mmdg_set_basis takes."""
    nfunc: int
    L: np.ndarray        # [S] int32
    nprim: np.ndarray    # [S] int32
    center: np.ndarray   # [S,3] bohr
    exps: np.ndarray     # [sum K]
    coefs: np.ndarray    # [sum K] component-free weights
    func: np.ndarray     # [S,6] function index per component or -1
    atom: np.ndarray | None = None

    @property
    def nshell(self) -> int:
        return int(self.L.shape[0])


def shells_from_bfs(bfs) -> ShellSet:
    """Groups a reference basis list (one ``Basis`` per Cartesian function,
    mmd/molecule.py:57-88) into shells: consecutive functions with the same origin,
    angular momentum, exponents and component-free weights form one shell; any
    function that does not fit starts a new shell (its other components absent)."""
    L_, K_, cen_, ex_, co_, fn_ = [], [], [], [], [], []
    cur = None  # (origin, L, exps, weights, last component index)
    for f, b in enumerate(bfs):
        lmn = tuple(int(x) for x in np.asarray(b.shell))
        L = sum(lmn)
        if L > LMAX:
            raise ValueError(f"basis function {f} has angular momentum {L}; the GPU path supports up to {LMAX} (d)")
        c = _COMP_INDEX[L][lmn]
        k = int(b.num_exps)
        origin = np.asarray(b.origin, dtype=np.float64).reshape(3)
        exps = np.asarray(b.exps, dtype=np.float64)[:k]
        w = np.asarray(b.norm, dtype=np.float64)[:k] * np.asarray(b.coefs, dtype=np.float64)[:k] / comp_norm(lmn)
        # (the weights test is np.allclose(cur_w, w, rtol=1e-12, atol=0) written out)
        join = (cur is not None and cur[1] == L and c > cur[4] and cur[2].shape == exps.shape
                and bool((cur[0] == origin).all()) and bool((cur[2] == exps).all())
                and bool((np.abs(cur[3] - w) <= 1e-12 * np.abs(w)).all()))
        if join:
            fn_[-1][c] = f
            cur = (cur[0], cur[1], cur[2], cur[3], c)
        else:
            L_.append(L)
            K_.append(k)
            cen_.append(origin)
            ex_.append(exps)
            co_.append(w)
            row = np.full(MAX_COMP, -1, dtype=np.int32)
            row[c] = f
            fn_.append(row)
            cur = (origin, L, exps, w, c)
    return ShellSet(nfunc=len(bfs), L=np.array(L_, dtype=np.int32), nprim=np.array(K_, dtype=np.int32),
                    center=np.array(cen_, dtype=np.float64).reshape(-1, 3),
                    exps=np.concatenate(ex_) if ex_ else np.zeros(0),
                    coefs=np.concatenate(co_) if co_ else np.zeros(0),
                    func=np.array(fn_, dtype=np.int32).reshape(-1, MAX_COMP))


def fingerprint(bfs) -> tuple:
    """Cheap identity of a basis list (origins, shells, exponents, weights)."""
    return tuple((tuple(np.asarray(b.origin, dtype=np.float64).tolist()), tuple(int(x) for x in b.shell),
                  tuple(np.asarray(b.exps, dtype=np.float64).tolist()),
                  tuple(np.asarray(b.coefs, dtype=np.float64).tolist())) for b in bfs)
