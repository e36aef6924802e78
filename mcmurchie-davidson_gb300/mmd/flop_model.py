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


# ------------------------------------------------------------------ issued / useful FP64 FLOPs
# What the Fock kernels really issue, counted from the structure of the generated
# code (csrc/gen_md.py, csrc/md_device.cuh, csrc/md_warp.cuh), lane by lane, with an
# FMA as 2 FLOPs and a multiply or add as 1 -- the quantity that ncu's
# smsp__sass_thread_inst_executed_op_{dfma,dmul,dadd}_pred_on counters measure as
# 2 DFMA + DMUL + DADD.  Not counted: the FP64 instructions inside CUDA's exp
# (library code, called only by the asymptotic Boys branch of L >= 5), conversions
# and compares (the ncu summary gives their share).  Per-class inputs are the Fock build's counters: digested
# function quartets, shell quartets, primitive quartets, bra-primitive passes and
# asymptotic-branch Boys evaluations.

def _gen_md():
    import importlib.util
    import os
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "csrc", "gen_md.py")
    spec = importlib.util.spec_from_file_location("_gen_md_for_flops", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@lru_cache(maxsize=None)
def _gm():
    return _gen_md()


RSQRT_FLOPS = 7  # rsqrt_dd: y0^2 and three FMAs (md_device.cuh; 3e/4 and y0/2 from FP32)


def boys_flops(L: int, asymptotic: bool) -> int:
    """boys_eval<L> (md_device.cuh).  Taylor branch: y = T_k - T (1), the F_L row (6
    FMAs); for L = 1 the F_0 row (6 FMAs); for L > 1 the exp row (7 FMAs), 2T and the
    downward recursion (an FMA and a product per order).  Asymptotic branch (T >= 48):
    rsqrt_dd(T), F_0, 1/T and the upward recursion (exp(-T) terms from L = 5)."""
    if not asymptotic:
        if L == 0:
            return 13
        if L == 1:
            return 25
        return 13 + 14 + 1 + 3 * L
    if L == 0:
        return RSQRT_FLOPS + 1
    return RSQRT_FLOPS + 2 + (1 + 3 * L if L > 4 else 2 * L)


def boys_df_flops(L: int) -> int:
    """FP64 FLOPs of boys_eval_df<L> (md_device.cuh), the near branch of L <= 4: y =
    T_k - T (1), per Taylor row a conversion sum (1) and the last Horner step as an FMA
    (2) -- the other steps run as float pairs on the FP32 pipe -- and for L > 1 the exp
    row likewise, 2T and the downward recursion (an FMA and a product per order)."""
    if L == 0:
        return 1 + 3
    if L == 1:
        return 1 + 3 + 3
    return 1 + 3 + 3 + 1 + 3 * L


def r0_flops(L: int, asymptotic: bool) -> int:
    """hermite_r0_pp<L> (md_device.cuh).  L <= 4: P - Q (3), |PQ|^2 (5), pq, p + q and
    pq |PQ|^2 (3), one rsqrt_dd, then the chain R^(n) = rr M^n B_n shared by both sides:
    R^(0) (1) and two products per order n >= 1; M = -2 pq rr^2 or -pq rr^2 needs pq rr^2
    (2; sign and factor 2 on the integer pipe), which for L = 0 only the near side
    computes; near (T < 48) adds T (1) and the Boys rows by boys_eval_df, far lanes take
    constant B_n.  L >= 5 (the warp kernel): P - Q, |PQ|^2, p + q, rsqrt_dd(p + q),
    alpha (3), T, Boys (either branch of boys_eval), the prefactor powers."""
    pref = 1 if L == 0 else 1 + (2 * L + 1)
    if L <= 4:
        common = 3 + 5 + 3 + RSQRT_FLOPS
        chain = 1 + 2 * L
        if asymptotic:
            return common + (0 if L == 0 else 2) + chain
        return common + 2 + 1 + boys_df_flops(L) + chain
    return 3 + 5 + 1 + RSQRT_FLOPS + 3 + 1 + boys_flops(L, asymptotic) + pref


@lru_cache(maxsize=None)
def recursion_flops(L: int) -> int:
    """The in-place Hermite Coulomb recursion of the per-thread code: X R1 (1 FLOP) when
    the stepped index m is 1, fma(X, R1, R2) (2 FLOPs) when m = 2 (the factor m - 1 = 1
    is folded), fma(X, R1, (m-1) R2) (3 FLOPs) when m > 2."""
    g = _gm()
    tot = 0
    for s in range(1, L + 1):
        for (t, u, v) in g.herm(s):
            if (t, u, v) == (0, 0, 0):
                continue
            m = t if t > 0 else (u if u > 0 else v)
            tot += 3 if m > 2 else (2 if m == 2 else 1)
    return tot


@lru_cache(maxsize=None)
def _thread_config(cls):
    """(chunk passes, ket FLOPs per primitive quartet, bra FLOPs per bra pass) of the
    per-thread Fock kernel of a class."""
    g = _gm()
    la, lb, lc, ld = cls
    chunk, _ = g.choose(la, lb, lc, ld)
    ncd = C(lc) * C(ld)
    nch = -(-ncd // chunk)
    hp = H(la + lb)
    return nch, 2 * hp * nnz(lc, ld), 2 * nnz(la, lb) * ncd


@lru_cache(maxsize=None)
def _warp_config(cls):
    """(ket FLOPs per primitive quartet, bra FLOPs per bra pass, R-level FLOPs) issued by
    the warp-cooperative kernel: every lane of a pass runs the pass's longest term loop."""
    g = _gm()
    la, lb, lc, ld = cls
    L, hp = la + lb + lc + ld, H(la + lb)
    kcd = [((r >> 8) & 15) * ((r >> 12) & 15) * ((r >> 16) & 15) for r in g._pair_records(lc, ld)]
    kab = [((r >> 8) & 15) * ((r >> 12) & 15) * ((r >> 16) & 15) for r in g._pair_records(la, lb)]
    ncd, nab = len(kcd), len(kab)
    ket = 0
    for m in range(-(-ncd * hp // 32)):
        ket += max(kcd[o // hp] for o in range(32 * m, min(32 * m + 32, ncd * hp)))
    bra = 0
    for m in range(-(-nab * ncd // 32)):
        bra += max(kab[o // ncd] for o in range(32 * m, min(32 * m + 32, nab * ncd)))
    rlev = 3 * sum(H(s) for s in range(1, L + 1))
    return 64 * ket, 64 * bra, rlev


def fock_kernel(cls) -> str:
    return "warp" if _gm().is_warp_class(tuple(cls)) else "thread"


def issued_flops(cls, row) -> float:
    """FP64 FLOPs the Fock kernel of class ``cls`` issues for the counters ``row``."""
    nfq, nsq, npq, nbp, nas = (float(x) for x in list(row) + [0.0] * (5 - len(row)))
    L = sum(cls)
    r0 = (npq - nas) * r0_flops(L, False) + nas * r0_flops(L, True)
    if fock_kernel(cls) == "warp":
        ket, bra, rlev = _warp_config(tuple(cls))
        return r0 + npq * (rlev + ket) + nbp * bra + 6.0 * nfq
    nch, ket, bra = _thread_config(tuple(cls))
    return nch * (r0 + npq * recursion_flops(L)) + npq * ket + nbp * bra + 6.0 * nfq


def useful_flops(cls, row) -> float:
    """The algorithm's own FP64 FLOPs for the counters ``row``: Boys and R once per
    primitive quartet, the ket transform over the non-zero Hermite terms once per
    primitive quartet, the bra transform once per bra primitive, six products per
    digested function quartet -- no recomputation, no padded lanes."""
    nfq, nsq, npq, nbp, nas = (float(x) for x in list(row) + [0.0] * (5 - len(row)))
    la, lb, lc, ld = cls
    L = la + lb + lc + ld
    r0 = (npq - nas) * r0_flops(L, False) + nas * r0_flops(L, True)
    ket = 2 * H(la + lb) * nnz(lc, ld)
    bra = 2 * nnz(la, lb) * C(lc) * C(ld)
    return r0 + npq * (recursion_flops(L) + ket) + nbp * bra + 6.0 * nfq
