"""Two-electron integrals on the GPU, behind the reference's ``mmd.integrals.twoe`` API.

``Basis``, ``ERI`` and ``doERIs`` keep the signatures and semantics of
cython/basis.pxi:6-121 and cython/twoe.pyx:12-50.  The integrals themselves are
evaluated by the sm_103a McMurchie-Davidson kernels of libmmdg.so; there is no
CPU path.
"""
from __future__ import annotations

import os
from collections import OrderedDict

import numpy as np

from .. import _native
from .shells import fingerprint, shells_from_bfs

PI = 3.141592653589793238462643383279  # cython/util.pxi:7


def _fact2(k: int) -> float:
    """(2n-1)!! with (-1)!! = 1, the value the reference's normalisation assumes."""
    r = 1.0
    while k > 1:
        r *= k
        k -= 2
    return r


# (shell, raw exponents, raw coefficients) -> (norm, normalised coefficients): every
# function of an element's shell type shares them, so a molecule normalises each once
_NORMALISED: dict = {}
_NORMALISED_MAX = 4096


class Basis:
    """Contracted Cartesian Gaussian function (cython/basis.pxi:6-121).

    Same constructor and attributes as the reference's extension class:
    ``Basis(origin, shell, num_exps, exps, coefs)`` with ``origin``, ``shell``,
    ``num_exps``, ``exps``, ``coefs`` (contraction-normalised in place) and
    ``norm`` (primitive normalisation)."""

    __slots__ = ("origin", "shell", "num_exps", "exps", "coefs", "norm")

    def __init__(self, origin, shell, num_exps, exps, coefs):
        self.origin = np.array(origin, dtype=np.float64).reshape(3)
        self.shell = np.array(shell, dtype=np.int64).reshape(3)
        self.num_exps = int(num_exps)
        if self.num_exps < 1:
            raise ValueError("a basis function needs at least one primitive")
        self.exps = np.array(exps, dtype=np.float64)[: self.num_exps].copy()
        self.coefs = np.array(coefs, dtype=np.float64)[: self.num_exps].copy()
        key = (self.shell.tobytes(), self.exps.tobytes(), self.coefs.tobytes())
        done = _NORMALISED.get(key)
        if done is None:
            self.norm = np.zeros(self.num_exps)
            self.normalize()
            if len(_NORMALISED) < _NORMALISED_MAX:
                _NORMALISED[key] = (self.norm.copy(), self.coefs.copy())
        else:  # the same arithmetic on the same inputs: bit-identical results
            self.norm = done[0].copy()
            self.coefs = done[1].copy()

    def normalize(self):
        """Primitive then contracted normalisation (basis.pxi:87-120)."""
        l, m, n = (int(x) for x in self.shell)
        L = l + m + n
        f2 = _fact2(2 * l - 1) * _fact2(2 * m - 1) * _fact2(2 * n - 1)
        self.norm = np.sqrt(np.power(2, 2 * L + 1.5) * np.power(self.exps, L + 1.5) / f2 / np.power(np.pi, 1.5))
        prefactor = np.power(np.pi, 1.5) * f2 / np.power(2.0, L)
        # the double sum over primitive pairs, each term formed in the reference's
        # operation order and accumulated left to right in its (ia, ib) order
        nm, c, e = self.norm, self.coefs, self.exps
        terms = nm[:, None] * nm[None, :] * c[:, None] * c[None, :] / np.power(e[:, None] + e[None, :], L + 1.5)
        N = 0.0 + np.add.accumulate(terms.ravel())[-1]
        N *= prefactor
        N = np.power(N, -0.5)
        self.coefs *= N
        return self.norm


# Device contexts by basis fingerprint, least recently used first.  The cache is
# bounded by the device bytes its contexts hold (a context's quartet lists grow as
# S^4/8 in the number of shells: 1.4 GB for (H2O)16 6-31G**, 22 GB for (H2O)32) and
# by a count; the oldest entries are dropped first.  Dropping an entry releases only
# the cache's reference: a context still held by a Molecule stays valid and frees its
# device memory when its last holder lets go.  MMD_CONTEXT_CACHE_BYTES overrides the
# byte budget.
_ctx_cache: "OrderedDict" = OrderedDict()
CONTEXT_CACHE_MAX = 16
CONTEXT_CACHE_BYTES = int(float(os.environ.get("MMD_CONTEXT_CACHE_BYTES", 48e9)))


def _trim_cache(keep=None):
    total = 0
    sizes = {}
    for k, c in _ctx_cache.items():
        sizes[k] = c.device_bytes()
        total += sizes[k]
    while _ctx_cache and (len(_ctx_cache) > CONTEXT_CACHE_MAX or total > CONTEXT_CACHE_BYTES):
        k = next(iter(_ctx_cache))
        if k == keep:
            if len(_ctx_cache) == 1:
                break
            _ctx_cache.move_to_end(k)
            continue
        _ctx_cache.pop(k)
        total -= sizes.pop(k)


def context_for(bfs):
    """Device context (primitive pairs + Schwarz table) for a basis list, cached."""
    key = fingerprint(bfs)
    ctx = _ctx_cache.get(key)
    if ctx is None:
        ctx = _native.Context(shells_from_bfs(bfs))
        _ctx_cache[key] = ctx
        _trim_cache(keep=key)
    else:
        _ctx_cache.move_to_end(key)
    return ctx


def clear_context_cache():
    """Drop every cached device context (contexts still held elsewhere stay valid)."""
    _ctx_cache.clear()


def ERI(a, b, c, d) -> float:
    """Contracted ERI (ab|cd) of four basis functions (twoe.pyx:36-50): one shell
    quartet evaluated by the class kernels (``mmdg_eri_quartets``) in the cached
    context of the four functions."""
    ctx = context_for([a, b, c, d])
    v = ctx.function_quartets(np.array([[0, 1, 2, 3]], dtype=np.int32))
    return float(v[0])


def doERIs(N, TwoE, bfs):
    """Fill ``TwoE`` (N^4, C order) with all ERIs and return it (twoe.pyx:12-31)."""
    N = int(N)
    if len(bfs) != N:
        raise ValueError("doERIs: N must equal len(bfs)")
    ctx = context_for(bfs)
    T = ctx.eri_tensor()
    out = T.cpu().numpy()
    TwoE[...] = out
    return TwoE


def eri_tensor_device(bfs):
    """The ERI tensor as a CUDA tensor (kept on the device for the conventional SCF)."""
    return context_for(bfs).eri_tensor()
