"""Algorithmic FLOP model of the McMurchie-Davidson ERI + Fock digestion.

Per primitive quartet of class (la lb|lc ld), with Lp = la+lb, Lq = lc+ld,
L = Lp+Lq, H(n) = (n+1)(n+2)(n+3)/6 Hermite functions of order <= n and
C(l) = (l+1)(l+2)/2 Cartesian components (one FMA = 2 FLOPs):

  F_boys = 2(L+1) + 10                    Boys interpolation and recursion
  F_R    = 3 sum_{k<=L} H(k) = (L+1)(L+2)(L+3)(L+4)/8   Hermite Coulomb recursion
  F_ket  = 2 C(lc)C(ld) H(Lp) H(Lq)       ket Hermite -> Cartesian transform
  F_bra  = 2 C(la)C(lb)C(lc)C(ld) H(Lp)   bra transform
  F_acc  = 2 C(la)C(lb)C(lc)C(ld)         contraction accumulate

and F_JK = 12 per digested function quartet (two Coulomb and four exchange
multiply-adds).  ``model`` is this dense count, the yardstick of the roofline.

``executed`` counts what the generated kernels actually perform: the ket transform
over the non-zero Hermite terms only (sum over ket function pairs of
(xc+xd+1)(yc+yd+1)(zc+zd+1), times H(Lp)), the bra transform once per bra
primitive pair and contracted ket (not per primitive quartet), and the R recursion
and Boys evaluation once per primitive quartet and ket chunk.
"""
from __future__ import annotations

from functools import lru_cache

CLASSES = [(la, lb, lc, ld) for la in range(3) for lb in range(la + 1) for lc in range(3) for ld in range(lc + 1)
           if (la, lb) >= (lc, ld)]


def H(n: int) -> int:
    return (n + 1) * (n + 2) * (n + 3) // 6


def C(l: int) -> int:
    return (l + 1) * (l + 2) // 2


def _comps(l):
    return [(x, y, l - x - y) for x in range(l, -1, -1) for y in range(l - x, -1, -1)]


@lru_cache(maxsize=None)
def nnz(la: int, lb: int) -> int:
    return sum((a[0] + b[0] + 1) * (a[1] + b[1] + 1) * (a[2] + b[2] + 1) for a in _comps(la) for b in _comps(lb))


def prim_quartet_flops(la, lb, lc, ld) -> int:
    """Model FLOPs per primitive quartet (dense Hermite transforms)."""
    Lp, Lq = la + lb, lc + ld
    L = Lp + Lq
    f_boys = 2 * (L + 1) + 10
    f_r = (L + 1) * (L + 2) * (L + 3) * (L + 4) // 8
    f_ket = 2 * C(lc) * C(ld) * H(Lp) * H(Lq)
    f_bra = 2 * C(la) * C(lb) * C(lc) * C(ld) * H(Lp)
    f_acc = 2 * C(la) * C(lb) * C(lc) * C(ld)
    return f_boys + f_r + f_ket + f_bra + f_acc


def class_flops(cls, n_prim_quartets, n_function_quartets, n_shell_quartets=0) -> float:
    """Model FLOPs of a class given its computed primitive / function quartet counts."""
    return prim_quartet_flops(*cls) * float(n_prim_quartets) + 12.0 * float(n_function_quartets)


def executed_flops_per_prim_quartet(la, lb, lc, ld, chunk_passes: int = 1) -> float:
    """FLOPs the generated code performs per primitive quartet, excluding the bra
    transform (counted per bra primitive by ``executed_bra_flops``)."""
    Lp, Lq = la + lb, lc + ld
    L = Lp + Lq
    f_boys = 2 * (L + 1) + 10
    f_r = (L + 1) * (L + 2) * (L + 3) * (L + 4) // 8
    f_ket = 2 * nnz(lc, ld) * H(Lp)
    return chunk_passes * (f_boys + f_r + 16) + f_ket


def executed_bra_flops(la, lb, lc, ld) -> int:
    return 2 * nnz(la, lb) * C(lc) * C(ld)


def build_flops(counts, kind: str = "model") -> float:
    """Total FLOPs of one Fock build from the per-class counters of ``mmdg_fock``
    (rows: classes in CLASSES order; columns: function quartets, shell quartets,
    primitive quartets)."""
    tot = 0.0
    for cls, row in zip(CLASSES, counts):
        nfq, nsq, npq = (float(x) for x in row)
        if kind == "model":
            tot += class_flops(cls, npq, nfq, nsq)
        else:
            tot += executed_flops_per_prim_quartet(*cls) * npq + 12.0 * nfq
    return tot
