#!/usr/bin/env python3
"""Generator of the per-class McMurchie-Davidson shell-quartet device code.

For every angular class (la lb|lc ld) with la>=lb, lc>=ld, (la,lb)>=(lc,ld)
(lmax = 2: 21 classes) it emits one ``struct MD_<la><lb><lc><ld>`` whose
``run()`` evaluates one contracted shell quartet in straight-line code:

    for each chunk of ket Cartesian function pairs (compile-time unrolled; a Fock
    kernel thread evaluates one chunk of one quartet, ``c.chunk``; -1 = all):
      acc[ab][cd in chunk] = 0
      for each bra primitive pair i:
        W[cd in chunk][tuv] = 0                         (tuv: bra Hermite, t+u+v <= la+lb)
        for each ket primitive pair j:
          R^(n)_000 = pref (-2 alpha)^n F_n(T)          (Boys: md_device.cuh)
          R_tuv    <- Hermite Coulomb recursion         (in place, registers or shared memory)
          W[cd][tuv] += sum_{tau nu phi} (-1)^(tau+nu+phi) E'_cd[tau nu phi] R_{t+tau,u+nu,v+phi}
        acc[ab][cd] += sum_{tuv} E'_ab[tuv] W[cd][tuv]
      digest(acc)                                       (Fock / tensor / Schwarz consumer)

This is the algorithm of the reference's ``electron_repulsion`` + ``ERI``
(cython/twoe.pyx:36-94) with its loops reordered: the E products are formed once
per primitive pair (E' tables, built by the pair kernel with the contraction
coefficients, normalisation and 1/p folded in), the R recursion (cython/util.pxi:33-50)
is evaluated once per primitive quartet for all (t,u,v) instead of recursively per
term, and the six-fold Hermite sum is factorised into a ket transform (per
primitive quartet) and a bra transform (per bra primitive).

Chunking trades R recomputation for registers: W and acc of one chunk live in
registers; R lives in registers when its table is small, otherwise in a
per-thread slice of shared memory.  The chunk size per class is a tunable.

The E' table layout (shared with pairs.cu): for fa in comps(la), fb in comps(lb)
(row-major), for t <= xa+xb, u <= ya+yb, v <= za+zb (t outermost):
    E'[fa fb][t u v] = c K_ab / p * norm_a norm_b * Ex_t Ey_u Ez_v.
"""
from __future__ import annotations

import argparse
import os

LMAX = 2


def comps(l):
    return [(x, y, l - x - y) for x in range(l, -1, -1) for y in range(l - x, -1, -1)]


def herm(L):
    """Hermite (t,u,v), t+u+v <= L, ordered by order n, then t desc, u desc."""
    out = []
    for n in range(L + 1):
        for t in range(n, -1, -1):
            for u in range(n - t, -1, -1):
                out.append((t, u, n - t - u))
    return out


def hidx_map(L):
    return {h: k for k, h in enumerate(herm(L))}


def pair_terms(la, lb):
    """List over function pairs (fa,fb) of lists of (t,u,v) with their E' offset."""
    res = []
    off = 0
    for a in comps(la):
        for b in comps(lb):
            terms = []
            for t in range(a[0] + b[0] + 1):
                for u in range(a[1] + b[1] + 1):
                    for v in range(a[2] + b[2] + 1):
                        terms.append(((t, u, v), off))
                        off += 1
            res.append(terms)
    return res, off


def H(n):
    return (n + 1) * (n + 2) * (n + 3) // 6


def C(l):
    return (l + 1) * (l + 2) // 2


def classes():
    out = []
    for la in range(LMAX + 1):
        for lb in range(la + 1):
            for lc in range(LMAX + 1):
                for ld in range(lc + 1):
                    if (la, lb) >= (lc, ld):
                        out.append((la, lb, lc, ld))
    return out


# register budget (doubles) for W + acc (+ R when register-resident)
REG_BUDGET = 96


def choose(la, lb, lc, ld):
    """(chunk, r_in_smem) minimising a DP-instruction estimate under the register budget."""
    Lp, Lq = la + lb, lc + ld
    L = Lp + Lq
    nab, ncd = C(la) * C(lb), C(lc) * C(ld)
    cost_R = (L + 1) * (L + 2) * (L + 3) * (L + 4) / 8 + 2 * (L + 1) + 40
    best = None
    for smem in (0, 1):
        for c in range(1, ncd + 1):
            state = c * H(Lp) + nab * c + (0 if smem else H(L))
            if state > REG_BUDGET:
                continue
            nch = -(-ncd // c)
            cost = nch * cost_R * (1.05 if smem else 1.0)
            if best is None or cost < best[0]:
                best = (cost, c, smem)
    return best[1], best[2]


def emit_r_recursion(L, rvar, out, ind):
    """In-place Hermite Coulomb recursion: R^(n) for t+u+v<=s from R^(n+1), s=1..L.

    ``rvar(k)`` gives the lvalue of Hermite slot k (of the order-L table).  Slot 0
    holds R^(L)_000 on entry of step 1 ... the caller writes Rn[] into slot 0 at
    each level.  Order within a level: t desc, then u desc, then v desc, so every
    source is read before it is overwritten.
    """
    hm = hidx_map(L)
    for s in range(1, L + 1):
        n = L - s
        ents = [h for h in herm(s)]
        # process (t,u,v) != 0 in the safe order
        def key(h):
            return (-h[0], -h[1], -h[2])
        for (t, u, v) in sorted([h for h in ents if h != (0, 0, 0)], key=key):
            if t > 0:
                src1 = hm[(t - 1, u, v)]
                expr = f"X * {rvar(src1)}"
                if t > 1:
                    expr = f"fma(X, {rvar(src1)}, Real({t - 1}) * {rvar(hm[(t - 2, u, v)])})"
            elif u > 0:
                src1 = hm[(0, u - 1, v)]
                expr = f"Y * {rvar(src1)}"
                if u > 1:
                    expr = f"fma(Y, {rvar(src1)}, Real({u - 1}) * {rvar(hm[(0, u - 2, v)])})"
            else:
                src1 = hm[(0, 0, v - 1)]
                expr = f"Z * {rvar(src1)}"
                if v > 1:
                    expr = f"fma(Z, {rvar(src1)}, Real({v - 1}) * {rvar(hm[(0, 0, v - 2)])})"
            out.append(f"{ind}{rvar(hm[(t, u, v)])} = {expr};")
        out.append(f"{ind}{rvar(0)} = Rn[{n}];")


def gen_class(la, lb, lc, ld, chunk=None, smem=None, compact=None):
    Lp, Lq = la + lb, lc + ld
    L = Lp + Lq
    if compact is None:
        compact = L > COMPACT_ABOVE_L
    if compact:
        return gen_class_compact(la, lb, lc, ld)
    c_auto, s_auto = choose(la, lb, lc, ld)
    chunk = c_auto if chunk is None else chunk
    smem = s_auto if smem is None else smem
    if L == 0:
        smem = 0
    bra_terms, nnz_ab = pair_terms(la, lb)
    ket_terms, nnz_cd = pair_terms(lc, ld)
    nab, ncd = len(bra_terms), len(ket_terms)
    hp = herm(Lp)
    hpm = hidx_map(Lp)
    hm = hidx_map(L)
    name = f"MD_{la}{lb}{lc}{ld}"
    o = []
    o.append(f"template <typename Real>")
    o.append(f"struct {name} {{")
    o.append(f"  static constexpr int LA = {la}, LB = {lb}, LC = {lc}, LD = {ld}, L = {L};")
    o.append(f"  static constexpr int NAB = {nab}, NCD = {ncd}, NNZ_AB = {nnz_ab}, NNZ_CD = {nnz_cd};")
    nchunk = -(-ncd // chunk)
    o.append(f"  static constexpr int HL = {H(L)}, HP = {H(Lp)}, CHUNK = {chunk}, NCHUNK = {nchunk}, RSMEM = {smem};")
    o.append(f"  template <class Ctx, class Digest>")
    o.append(f"  static __device__ __forceinline__ void run(const Ctx& c, Digest& dg) {{")
    if smem:
        o.append(f"    Real* __restrict__ Rs = c.template rsmem<Real>();")
        o.append(f"    const int RS = c.rstride();")
        rvar = lambda k: f"Rs[{k} * RS]"
    else:
        o.append(f"    Real Rr[{H(L)}];")
        rvar = lambda k: f"Rr[{k}]"
    chunks = [list(range(s, min(s + chunk, ncd))) for s in range(0, ncd, chunk)]
    for ci, ch in enumerate(chunks):
        o.append(f"    if (c.chunk < 0 || c.chunk == {ci}) {{ // ket function pairs {ch[0]}..{ch[-1]}")
        for fab in range(nab):
            o.append("      Real " + ", ".join(f"a{fab}_{fcd} = 0" for fcd in ch) + ";")
        o.append(f"      for (int i = c.bra_begin; i < c.bra_end; ++i) {{")
        for fcd in ch:
            o.append("        Real " + ", ".join(f"w{fcd}_{k} = 0" for k in range(len(hp))) + ";")
        o.append(f"        const auto ap = c.pp(i);")
        o.append(f"        auto bq = c.pp(c.ket_begin);")
        if not smem and L <= UNROLL_KET_MAX_L:
            # two independent primitive quartets in flight: hides the Boys/rsqrt chains
            o.append(f"#pragma unroll 2")
        o.append(f"        for (int j = c.ket_begin; j < c.ket_end; ++j) {{")
        o.append(f"          const auto bp = bq;")
        o.append(f"          if (j + 1 < c.ket_end) bq = c.pp(j + 1);  // next ket primitive pair, one iteration ahead")
        o.append(f"          Real Rn[{L + 1}], X, Y, Z;")
        o.append(f"          c.template hermite_r0_pp<{L}>(ap, bp, Rn, X, Y, Z);")
        if L == 0:
            o.append(f"          {rvar(0)} = Rn[0];")
        else:
            o.append(f"          {rvar(0)} = Rn[{L}];")
            emit_r_recursion(L, rvar, o, "          ")
        o.append(f"          const Real* __restrict__ ek = c.ket_E(j);")
        for fcd in ch:
            for (tq, uq, vq), eoff in ket_terms[fcd]:
                sgn = -1 if (tq + uq + vq) % 2 else 1
                o.append(f"          {{ const Real e = {'-' if sgn < 0 else ''}ek[{eoff}];")
                parts = []
                for k, (t, u, v) in enumerate(hp):
                    parts.append(f"w{fcd}_{k} = fma(e, {rvar(hm[(t + tq, u + uq, v + vq)])}, w{fcd}_{k});")
                o.append("            " + " ".join(parts) + " }")
        o.append(f"        }}")
        o.append(f"        const Real* __restrict__ eb = c.bra_E(i);")
        for fab in range(nab):
            for (t, u, v), eoff in bra_terms[fab]:
                k = hpm[(t, u, v)]
                o.append(f"        {{ const Real e = eb[{eoff}]; " +
                         " ".join(f"a{fab}_{fcd} = fma(e, w{fcd}_{k}, a{fab}_{fcd});" for fcd in ch) + " }")
        o.append(f"      }}")
        nb_, nd_ = C(lb), C(ld)
        for fab in range(nab):
            for fcd in ch:
                o.append(f"      dg.put({fab // nb_}, {fab % nb_}, {fcd // nd_}, {fcd % nd_}, a{fab}_{fcd});")
        o.append(f"    }}")
    o.append(f"  }}")
    o.append(f"}};")
    return "\n".join(o)


def gen_class_compact(la, lb, lc, ld):
    """Compact form for high L: runtime loop over ket function pairs (one per
    pass, R recomputed per pass), ket transform driven by a constant-memory term
    table, bra transform straight-line.  R lives in shared memory."""
    Lp, Lq = la + lb, lc + ld
    L = Lp + Lq
    bra_terms, nnz_ab = pair_terms(la, lb)
    ket_terms, nnz_cd = pair_terms(lc, ld)
    nab, ncd = len(bra_terms), len(ket_terms)
    hp = herm(Lp)
    hpm = hidx_map(Lp)
    hq = herm(Lq)
    hqm = hidx_map(Lq)
    hm = hidx_map(L)
    s = f"{la}{lb}{lc}{ld}"
    name = f"MD_{s}"
    o = []
    # constant tables: term ranges per ket function pair, E' offset, Hermite index, sign;
    # comb[hq][k] = slot of (t+tau, u+nu, v+phi) in the order-L table
    tb, toff, th = [0], [], []
    for fcd in range(ncd):
        for (tq, uq, vq), eoff in ket_terms[fcd]:
            toff.append(eoff)
            th.append(hqm[(tq, uq, vq)] | ((tq + uq + vq) % 2) << 15)
        tb.append(len(toff))
    comb = [hm[(t + a, u + b, v + c)] for (a, b, c) in hq for (t, u, v) in hp]
    o.append(f"static __constant__ unsigned short kTB_{s}[{len(tb)}] = {{{', '.join(map(str, tb))}}};")
    o.append(f"static __constant__ unsigned short kTO_{s}[{len(toff)}] = {{{', '.join(map(str, toff))}}};")
    o.append(f"static __constant__ unsigned short kTH_{s}[{len(th)}] = {{{', '.join(map(str, th))}}};")
    o.append(f"static __constant__ unsigned short kCB_{s}[{len(comb)}] = {{{', '.join(map(str, comb))}}};")
    o.append(f"template <typename Real>")
    o.append(f"struct {name} {{")
    o.append(f"  static constexpr int LA = {la}, LB = {lb}, LC = {lc}, LD = {ld}, L = {L};")
    o.append(f"  static constexpr int NAB = {nab}, NCD = {ncd}, NNZ_AB = {nnz_ab}, NNZ_CD = {nnz_cd};")
    o.append(f"  static constexpr int HL = {H(L)}, HP = {H(Lp)}, CHUNK = 1, NCHUNK = {ncd}, RSMEM = 1;")
    o.append(f"  template <class Ctx, class Digest>")
    o.append(f"  static __device__ __forceinline__ void run(const Ctx& c, Digest& dg) {{")
    o.append(f"    Real* __restrict__ Rs = c.template rsmem<Real>();")
    o.append(f"    const int RS = c.rstride();")
    rvar = lambda k: f"Rs[{k} * RS]"
    o.append(f"    const int f0 = c.chunk < 0 ? 0 : c.chunk, f1 = c.chunk < 0 ? NCD : c.chunk + 1;")
    o.append(f"#pragma unroll 1")
    o.append(f"    for (int fcd = f0; fcd < f1; ++fcd) {{")
    o.append(f"      const int t0 = kTB_{s}[fcd], t1 = kTB_{s}[fcd + 1];")
    o.append("      Real " + ", ".join(f"a{fab} = 0" for fab in range(nab)) + ";")
    o.append(f"      for (int i = c.bra_begin; i < c.bra_end; ++i) {{")
    o.append("        Real " + ", ".join(f"w{k} = 0" for k in range(len(hp))) + ";")
    o.append(f"        const auto ap = c.pp(i);")
    o.append(f"        auto bq = c.pp(c.ket_begin);")
    o.append(f"        for (int j = c.ket_begin; j < c.ket_end; ++j) {{")
    o.append(f"          const auto bp = bq;")
    o.append(f"          if (j + 1 < c.ket_end) bq = c.pp(j + 1);")
    o.append(f"          Real Rn[{L + 1}], X, Y, Z;")
    o.append(f"          c.template hermite_r0_pp<{L}>(ap, bp, Rn, X, Y, Z);")
    o.append(f"          {rvar(0)} = Rn[{L}];")
    emit_r_recursion(L, rvar, o, "          ")
    o.append(f"          const Real* __restrict__ ek = c.ket_E(j);")
    o.append(f"#pragma unroll 1")
    o.append(f"          for (int t = t0; t < t1; ++t) {{")
    o.append(f"            const unsigned h = kTH_{s}[t];")
    o.append(f"            const Real e = mmdg::flip_sign(ek[kTO_{s}[t]], (int)(h >> 15));  // sign on the integer pipe")
    o.append(f"            const unsigned short* __restrict__ cb = kCB_{s} + (h & 0x7fffu) * {len(hp)};")
    o.append("            " + " ".join(f"w{k} = fma(e, Rs[cb[{k}] * RS], w{k});" for k in range(len(hp))))
    o.append(f"          }}")
    o.append(f"        }}")
    o.append(f"        const Real* __restrict__ eb = c.bra_E(i);")
    for fab in range(nab):
        parts = []
        for (t, u, v), eoff in bra_terms[fab]:
            parts.append(f"a{fab} = fma(eb[{eoff}], w{hpm[(t, u, v)]}, a{fab});")
        o.append("        " + " ".join(parts))
    o.append(f"      }}")
    nb_, nd_ = C(lb), C(ld)
    o.append(f"      const int cc = fcd / {nd_}, cd = fcd - cc * {nd_};")
    for fab in range(nab):
        o.append(f"      dg.put({fab // nb_}, {fab % nb_}, cc, cd, a{fab});")
    o.append(f"    }}")
    o.append(f"  }}")
    o.append(f"}};")
    return "\n".join(o)


def _pair_records(la, lb):
    """Packed records of the function pairs of (la lb), sorted by their number of
    Hermite terms: real index | n_tau << 8 | n_nu << 12 | n_phi << 16 | E' offset << 20."""
    terms, _ = pair_terms(la, lb)
    recs = []
    for idx, (a, b) in enumerate((a, b) for a in comps(la) for b in comps(lb)):
        nt, nu, nph = a[0] + b[0] + 1, a[1] + b[1] + 1, a[2] + b[2] + 1
        off = terms[idx][0][1]
        assert len(terms[idx]) == nt * nu * nph and off < 4096
        recs.append((nt * nu * nph, idx | nt << 8 | nu << 12 | nph << 16 | off << 20))
    recs.sort(key=lambda r: r[0])
    return [r[1] for r in recs]


def gen_class_warp(la, lb, lc, ld):
    """Tables and constants of the warp-cooperative Fock kernel (md_warp.cuh) of one
    high-L class: function pairs sorted by Hermite term count."""
    Lp, Lq = la + lb, lc + ld
    L = Lp + Lq
    s = f"{la}{lb}{lc}{ld}"
    kab = _pair_records(la, lb)
    kcd = _pair_records(lc, ld)
    _, nnz_ab = pair_terms(la, lb)
    _, nnz_cd = pair_terms(lc, ld)
    o = []
    o.append(f"static __constant__ unsigned kWB_{s}[{len(kab)}] = {{{', '.join(f'{x}u' for x in kab)}}};")
    o.append(f"static __constant__ unsigned kWK_{s}[{len(kcd)}] = {{{', '.join(f'{x}u' for x in kcd)}}};")
    o.append(f"template <typename Real>")
    o.append(f"struct MDW_{s} {{")
    o.append(f"  static constexpr int LA = {la}, LB = {lb}, LC = {lc}, LD = {ld}, L = {L};")
    o.append(f"  static constexpr int NAB = {len(kab)}, NCD = {len(kcd)}, NNZ_AB = {nnz_ab}, NNZ_CD = {nnz_cd};")
    o.append(f"  static constexpr int HL = {H(L)}, HP = {H(Lp)};")
    o.append(f"  static __device__ __forceinline__ unsigned bra_pair(int x) {{ return kWB_{s}[x]; }}")
    o.append(f"  static __device__ __forceinline__ unsigned ket_pair(int x) {{ return kWK_{s}[x]; }}")
    o.append(f"  static __device__ __forceinline__ short herm(int x) {{ return kWH_{L}[x]; }}")
    o.append(f"}};")
    return "\n".join(o)


def gen_herm_tables():
    """Packed (t | u << 5 | v << 10) of every Hermite index, for each total L of the
    warp-cooperative classes."""
    out = []
    for L in sorted({sum(c) for c in classes() if is_warp_class(c)}):
        vals = [t | u << 5 | v << 10 for (t, u, v) in herm(L)]
        out.append(f"static __constant__ short kWH_{L}[{len(vals)}] = {{{', '.join(map(str, vals))}}};")
    return "\n".join(out)


def is_warp_class(cl):
    return sum(cl) > WARP_FOCK_ABOVE_L


# classes with la+lb+lc+ld above this use the compact form (k_tensor, k_quartets,
# k_schwarz)
COMPACT_ABOVE_L = 4
# classes with la+lb+lc+ld above this run Fock builds in the warp-cooperative kernel
# of md_warp.cuh, the others in the per-thread kernel k_fock.  Measured on (H2O)16
# 6-31G** (ms per build, per-thread -> warp form): L = 4 (pp|pp) 2.31 -> 3.32,
# (dp|pp) 3.30 -> 4.62, (dd|ss) 0.51 -> 1.16; L = 3 (pp|ps) 3.85 -> 7.69: below L = 5
# the warp form's lane padding and recursion passes cost more than they save.
WARP_FOCK_ABOVE_L = 4
# register-resident classes up to this total L unroll the ket primitive loop by two
UNROLL_KET_MAX_L = 2


def generate(path, overrides=None):
    overrides = overrides or {}
    parts = ["// Generated by gen_md.py -- do not edit.", "#pragma once", ""]
    for cl in classes():
        ch, sm = overrides.get(cl, (None, None))
        parts.append(gen_class(*cl, chunk=ch, smem=sm))
        parts.append("")
    parts.append(gen_herm_tables())
    for cl in classes():
        if is_warp_class(cl):
            parts.append(gen_class_warp(*cl))
            parts.append("")
    # class table for the host: smem doubles per thread
    parts.append("#define MMDG_FOR_EACH_CLASS(X) \\")
    cls = classes()
    for k, (la, lb, lc, ld) in enumerate(cls):
        parts.append(f"  X({la}, {lb}, {lc}, {ld}){' \\' if k + 1 < len(cls) else ''}")
    text = "\n".join(parts) + "\n"
    if os.path.exists(path):
        with open(path) as f:
            if f.read() == text:
                return path
    with open(path, "w") as f:
        f.write(text)
    return path


def generate_instances(outdir, ngroups=6):
    """Instantiation TUs (parallel compilation) and the dispatch table."""
    cls = classes()
    # balance groups by generated code size
    sizes = [(len(gen_class(*c)), c) for c in cls]
    sizes.sort(reverse=True)
    groups = [[] for _ in range(ngroups)]
    load = [0] * ngroups
    for sz, c in sizes:
        k = load.index(min(load))
        groups[k].append(c)
        load[k] += sz
    files = []
    decl = ["// Generated by gen_md.py -- do not edit.", "#pragma once", '#include "md_kernels.cuh"',
            '#include "md_warp.cuh"', "namespace mmdg {",
            "typedef cudaError_t (*fock_fn)(int, const Geometry&, const FockArgs&, const ClassLaunch&, const int2*, const unsigned*, const long long*, int, int, int, int, cudaStream_t);",
            "typedef cudaError_t (*tensor_fn)(const Geometry&, const TensorArgs&, const ClassLaunch&, cudaStream_t);",
            "typedef cudaError_t (*schwarz_fn)(const Geometry&, const SchwarzArgs&, const int*, int, cudaStream_t);",
            "typedef cudaError_t (*quartets_fn)(int, const Geometry&, const QuartetArgs&, const QuartetItem*, int, cudaStream_t);",
            "struct ClassEntry { int la, lb, lc, ld; fock_fn fock; tensor_fn tensor; schwarz_fn schwarz; quartets_fn quartets; };"]
    for g in range(ngroups):
        decl.append(f"cudaError_t init_group{g}();")
    for c in cls:
        s = "".join(map(str, c))
        decl.append(f"cudaError_t launch_fock_{s}(int, const Geometry&, const FockArgs&, const ClassLaunch&, const int2*, const unsigned*, const long long*, int, int, int, int, cudaStream_t);")
        decl.append(f"cudaError_t launch_tensor_{s}(const Geometry&, const TensorArgs&, const ClassLaunch&, cudaStream_t);")
        decl.append(f"cudaError_t launch_quartets_{s}(int, const Geometry&, const QuartetArgs&, const QuartetItem*, int, cudaStream_t);")
        if c[:2] == c[2:]:
            decl.append(f"cudaError_t launch_schwarz_{s}(const Geometry&, const SchwarzArgs&, const int*, int, cudaStream_t);")
    decl.append("static const ClassEntry kClasses[] = {")
    for c in cls:
        s = "".join(map(str, c))
        sch = f"launch_schwarz_{s}" if c[:2] == c[2:] else "nullptr"
        decl.append(f"  {{{c[0]}, {c[1]}, {c[2]}, {c[3]}, launch_fock_{s}, launch_tensor_{s}, {sch}, launch_quartets_{s}}},")
    decl.append("};")
    decl.append(f"static const int kNumGroups = {ngroups};")
    decl.append("static cudaError_t (*const kGroupInit[])() = {" + ", ".join(f"init_group{g}" for g in range(ngroups)) + "};")
    decl.append("}  // namespace mmdg")
    _write(os.path.join(outdir, "md_dispatch.cuh"), "\n".join(decl) + "\n")
    for g, grp in enumerate(groups):
        t = ["// Generated by gen_md.py -- do not edit.", '#include "md_dispatch.cuh"', "namespace mmdg {"]
        inits = []
        for c in grp:
            s = "".join(map(str, c))
            md = f"MD_{s}"
            t.append(f"cudaError_t launch_fock_{s}(int prec, const Geometry& g, const FockArgs& f, const ClassLaunch& cl, const int2* list, const unsigned* count, const long long* koff, int nkeys, int grid, int block, int item, cudaStream_t st) {{")
            if is_warp_class(c):
                mw = f"MDW_{s}"
                t.append("  (void)block;")
                for real, cond in (("float", "if (prec)"), ("double", "else")):
                    k = f"k_fock_warp<{mw}<{real}>, {real}>"
                    sm = f"WarpSmem<{mw}<{real}>, {real}>::bytes()"
                    t.append(f"  {cond} {k}<<<persistent_blocks({k}, {sm}, grid), kThreads, {sm}, st>>>(g, f, cl, list, count, koff, nkeys, item);")
            else:
                t.append("  (void)item;")
                t.append(f"  if ({md}<double>::RSMEM || block <= 0) block = kThreads;  // shared-memory R tables are sized for kThreads")
                for real, cond in (("float", "if (prec)"), ("double", "else")):
                    k = f"k_fock<{md}<{real}>, {real}>"
                    sm = f"smem_bytes<{md}<{real}>, {real}>()"
                    t.append(f"  {cond} {k}<<<persistent_blocks({k}, {sm}, grid, block), block, {sm}, st>>>(g, f, cl, list, count, koff, nkeys);")
            t.append(f"  return cudaGetLastError();")
            t.append("}")
            t.append(f"cudaError_t launch_tensor_{s}(const Geometry& g, const TensorArgs& a, const ClassLaunch& cl, cudaStream_t st) {{")
            t.append(f"  dim3 grid(cl.nbra, (cl.nket + kThreads - 1) / kThreads, {md}<double>::NCHUNK);")
            t.append(f"  k_tensor<{md}<double>><<<grid, kThreads, smem_bytes<{md}<double>, double>(), st>>>(g, a, cl);")
            t.append(f"  return cudaGetLastError();")
            t.append("}")
            t.append(f"cudaError_t launch_quartets_{s}(int prec, const Geometry& g, const QuartetArgs& a, const QuartetItem* items, int n, cudaStream_t st) {{")
            t.append(f"  const unsigned nb = (unsigned)(((long long)n * {md}<double>::NCHUNK + kThreads - 1) / kThreads);")
            t.append(f"  if (prec) k_quartets<{md}<float>, float><<<nb, kThreads, smem_bytes<{md}<float>, float>(), st>>>(g, a, items, n);")
            t.append(f"  else k_quartets<{md}<double>, double><<<nb, kThreads, smem_bytes<{md}<double>, double>(), st>>>(g, a, items, n);")
            t.append(f"  return cudaGetLastError();")
            t.append("}")
            for real in ("double", "float"):
                inits.append(f"  if ((e = cudaFuncSetAttribute(k_quartets<{md}<{real}>, {real}>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes<{md}<{real}>, {real}>()))) return e;")
            if is_warp_class(c):
                for real in ("double", "float"):
                    mw = f"MDW_{s}<{real}>"
                    inits.append(f"  if ((e = cudaFuncSetAttribute(k_fock_warp<{mw}, {real}>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)WarpSmem<{mw}, {real}>::bytes()))) return e;")
            else:
                inits.append(f"  if ((e = cudaFuncSetAttribute(k_fock<{md}<double>, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes<{md}<double>, double>()))) return e;")
                inits.append(f"  if ((e = cudaFuncSetAttribute(k_fock<{md}<float>, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes<{md}<float>, float>()))) return e;")
            inits.append(f"  if ((e = cudaFuncSetAttribute(k_tensor<{md}<double>>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes<{md}<double>, double>()))) return e;")
            if c[:2] == c[2:]:
                t.append(f"cudaError_t launch_schwarz_{s}(const Geometry& g, const SchwarzArgs& a, const int* list, int n, cudaStream_t st) {{")
                t.append(f"  k_schwarz<{md}<double>><<<(unsigned)(((long long)n * {md}<double>::NCHUNK + kThreads - 1) / kThreads), kThreads, smem_bytes<{md}<double>, double>(), st>>>(g, a, list, n);")
                t.append(f"  return cudaGetLastError();")
                t.append("}")
                inits.append(f"  if ((e = cudaFuncSetAttribute(k_schwarz<{md}<double>>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes<{md}<double>, double>()))) return e;")
        t.append(f"cudaError_t init_group{g}() {{")
        t.append("  cudaError_t e = cudaSuccess;")
        t.extend(inits)
        t.append("  return e;")
        t.append("}")
        t.append("}  // namespace mmdg")
        fn = os.path.join(outdir, f"md_inst{g}.cu")
        _write(fn, "\n".join(t) + "\n")
        files.append(fn)
    return files


def _write(path, text):
    if os.path.exists(path):
        with open(path) as f:
            if f.read() == text:
                return
    with open(path, "w") as f:
        f.write(text)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("out")
    args = ap.parse_args()
    generate(args.out)
    for cl in classes():
        print(cl, choose(*cl))
