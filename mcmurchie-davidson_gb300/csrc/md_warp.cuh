// md_warp.cuh -- warp-cooperative Fock kernel of the high-L angular classes.
//
// One warp evaluates one contracted shell quartet (ab|cd) and digests it into G
// (formPT semantics, cython/fock.pyx:38-85), with the work of the reference's
// electron_repulsion / ERI (cython/twoe.pyx:36-94) spread over the 32 lanes:
//
//   1. Boys function and R^(n)_000 = pref (-2 alpha)^n F_n(T) (cython/util.pxi:37-38,
//      54-55) for up to 32 primitive quartets at once, one per lane, into shared memory;
//   2. per primitive quartet, the Hermite Coulomb recursion (cython/util.pxi:33-50)
//      level by level: level s holds R^(L-s)_tuv for t+u+v <= s, its entries computed
//      by the lanes in parallel from level s-1 (two shared-memory buffers);
//   3. ket transform  W[cd][h] += sum_{tau nu phi} (-1)^(tau+nu+phi) E'_cd[tau nu phi] R[h + (tau nu phi)]
//      over the flattened outputs (cd, h), h a bra Hermite index, W in shared memory;
//   4. per bra primitive, bra transform  acc[ab][cd] += sum_{tuv} E'_ab[tuv] W[cd][tuv]
//      over the flattened outputs (ab, cd), acc in registers;
//   5. every lane digests its function quartets (FockDigest).
//
// The R table is computed once per primitive quartet and shared by every ket
// function pair (the one-thread-per-(quartet, ket pair) form recomputed it up to 36
// times), and the shared memory holds one R table per warp rather than per thread.
// On this GPU an FP64 warp instruction occupies the FP64 pipe for ~64 cycles of its
// sub-partition, so the integer index arithmetic and shared-memory traffic around
// each FMA are nearly free: what counts is FP64 instructions and their lane use.
// Function pairs are sorted by their number of Hermite terms (generated tables), so
// the 32 lanes of a pass run loops of nearly equal length; the remaining padding
// issues FMAs with a zero coefficient.
//
// Hermite index of (t, u, v) in the order of gen_md.herm(): by n = t+u+v, then t
// descending, then u descending:  n(n+1)(n+2)/6 + (n-t)(n-t+1)/2 + (n-t-u).
#pragma once
#include "md_kernels.cuh"

namespace mmdg {

constexpr int kWarps = kThreads / 32;
constexpr int kItem = 8;  // most list quartets per warp work item (k_fock_warp)

__device__ __forceinline__ int herm_index(int t, int u, int v) {
  const int n = t + u + v, m = n - t;
  return n * (n + 1) * (n + 2) / 6 + m * (m + 1) / 2 + (m - u);
}

// packed function-pair record of the generated tables:
//   bits 0-7 real function-pair index, 8-11 n_tau, 12-15 n_nu, 16-19 n_phi,
//   20-31 E' offset of the pair's first term within one primitive pair's E' block
__device__ __forceinline__ int fp_index(unsigned r) { return r & 0xff; }
__device__ __forceinline__ int fp_nt(unsigned r) { return (r >> 8) & 15; }
__device__ __forceinline__ int fp_nu(unsigned r) { return (r >> 12) & 15; }
__device__ __forceinline__ int fp_np(unsigned r) { return (r >> 16) & 15; }
__device__ __forceinline__ int fp_eoff(unsigned r) { return (int)(r >> 20); }

template <class MD, typename Real>
struct WarpSmem {
  static constexpr int BQ = MD::L + 4;  // R^(n)_000 for n = 0..L, then X, Y, Z
  static constexpr int W = MD::NCD * MD::HP;
  static constexpr int PER_WARP = W + 2 * MD::HL + 32 * BQ;
  static constexpr size_t bytes() { return size_t(PER_WARP) * kWarps * sizeof(Real); }
};

template <class MD, typename Real>
__global__ void __launch_bounds__(kThreads) k_fock_warp(Geometry g, FockArgs f, ClassLaunch cl, const int2* list,
                                                        const unsigned* count, const long long* key_off,
                                                        int nkeys, int max_item) {
  constexpr int L = MD::L, HL = MD::HL, HP = MD::HP, NAB = MD::NAB, NCD = MD::NCD;
  constexpr int NB = ncart(MD::LB), ND = ncart(MD::LD);
  constexpr int NKO = (NCD * HP + 31) / 32;  // ket-transform passes
  constexpr int NBO = (NAB * NCD + 31) / 32; // bra-transform passes (accumulators per lane)
  using SM = WarpSmem<MD, Real>;
  __shared__ unsigned s_pre[kMaxKeys + 1];
  __shared__ long long s_off[kMaxKeys];
  __shared__ unsigned s_ket[NCD], s_bra[NAB];
  __shared__ short s_herm[HL];  // packed (t | u << 5 | v << 10) of every Hermite index
  if (threadIdx.x == 0) {
    unsigned acc = 0;
    for (int k = 0; k < nkeys; ++k) {
      s_pre[k] = acc;
      s_off[k] = key_off[k];
      acc += count[k];
    }
    s_pre[nkeys] = acc;
  }
  for (int x = threadIdx.x; x < NCD; x += kThreads) s_ket[x] = MD::ket_pair(x);
  for (int x = threadIdx.x; x < NAB; x += kThreads) s_bra[x] = MD::bra_pair(x);
  for (int x = threadIdx.x; x < HL; x += kThreads) s_herm[x] = MD::herm(x);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  extern __shared__ double smem_d[];
  Real* const Ws = reinterpret_cast<Real*>(smem_d) + warp * SM::PER_WARP;
  Real* const R0 = Ws + SM::W;
  Real* const R1 = R0 + HL;
  Real* const Bq = R1 + HL;
  Real* const Rfin = (L & 1) ? R1 : R0;  // level L lands in buffer L % 2
  const unsigned n = s_pre[nkeys];
  constexpr unsigned kFull = 0xffffffffu;
  unsigned nfq = 0, nsq = 0, npq = 0, nbp = 0, nas = 0;
  // Work item: kItem consecutive list quartets (one bucket, mostly: equal primitive
  // counts).  Their primitive quartets are grouped into batches of at most 32, whose
  // Boys functions the lanes evaluate together; a quartet with more than 32 primitive
  // quartets is evaluated alone, 32 at a time.
  // quartets per work item: up to kItem, fewer when the class has too few quartets
  // to give every warp of the grid several items
  // Items are claimed dynamically from the launch's work counter (one atomic per item).
  const unsigned nwarps = gridDim.x * kWarps;
  const unsigned cap = max_item > 0 ? (unsigned)max_item : (unsigned)kItem;  // autotuned, or kItem
  const int item = (int)max(1u, min(cap, n / (4u * nwarps)));
  // (claimed one at a time: claiming the next item ahead, as k_fock does, was slower
  // here -- (dp|pp) 2.55 against 3.2 ms per (H2O)16 build -- since a warp then holds
  // two items of up to 8 quartets each when the list runs out)
  for (;;) {
    unsigned long long claim = 0;
    if (lane == 0) claim = atomicAdd(f.work, (unsigned long long)item);
    claim = __shfl_sync(kFull, claim, 0);
    if (claim >= (unsigned long long)n) break;
    const unsigned q0 = (unsigned)claim;
    const int nq = (int)min((unsigned)item, n - q0);
    int qbp = 0, qkp = 0, qnp = 0;  // lane x < nq: quartet x of the item
    if (lane < nq) {
      const unsigned qi = n - 1u - (q0 + lane);  // heaviest buckets (stored last) first
      int key = 0;
      while (qi >= s_pre[key + 1]) ++key;
      const int2 e = list[s_off[key] + (qi - s_pre[key])];
      qbp = __ldg(cl.bra + e.x);
      qkp = __ldg(cl.ket + e.y);
      qnp = __ldg(g.pr_count + qbp) * __ldg(g.pr_count + qkp);
    }
    int qend = qnp;  // inclusive prefix sum of the primitive-quartet counts
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int t = __shfl_up_sync(kFull, qend, d);
      if (lane >= d) qend += t;
    }
    int qs = 0;
    while (qs < nq) {
      const int prev = __shfl_sync(kFull, qend, qs > 0 ? qs - 1 : 0);
      const int base = qs > 0 ? prev : 0;
      const bool fits = lane >= qs && lane < nq && qend - base <= 32;
      int qe = qs + __popc(__ballot_sync(kFull, fits));
      const bool batched = qe > qs;
      if (!batched) qe = qs + 1;
      if (batched) {  // Boys and R^(n)_000 of every primitive quartet of quartets qs..qe-1
        __syncwarp();
        const int tot = __shfl_sync(kFull, qend, qe - 1) - base;
        int myq = qs;
        for (int x = qs; x < qe - 1; ++x)
          if (lane >= __shfl_sync(kFull, qend, x) - base) myq = x + 1;
        const int mbp = __shfl_sync(kFull, qbp, myq), mkp = __shfl_sync(kFull, qkp, myq);
        const int mprev = __shfl_sync(kFull, qend, myq > 0 ? myq - 1 : 0);  // every lane shuffles
        const int mstart = (myq > qs ? mprev : base) - base;
        if (lane < tot) {
          Ctx<Real> cq = make_ctx<MD, Real>(g, mbp, mkp, nullptr);
          const int nk = cq.ket_end - cq.ket_begin;
          const int pp = lane - mstart, ii = pp / nk, jj = pp - ii * nk;
          Real Rn[L + 1], X, Y, Z;
          cq.template hermite_r0_pp<L>(cq.pp(cq.bra_begin + ii), cq.pp(cq.ket_begin + jj), Rn, X, Y, Z);
          Real* b = Bq + lane * SM::BQ;
#pragma unroll
          for (int k = 0; k <= L; ++k) b[k] = Rn[k];
          b[L + 1] = X;
          b[L + 2] = Y;
          b[L + 3] = Z;
          nas += cq.nasym;
        }
        __syncwarp();
      }
      for (int x = qs; x < qe; ++x) {
        const int bp = __shfl_sync(kFull, qbp, x), kp = __shfl_sync(kFull, qkp, x);
        const int xprev = __shfl_sync(kFull, qend, x > 0 ? x - 1 : 0);
        const int boff = batched ? (x > qs ? xprev : base) - base : 0;  // Bq slot of its first primitive quartet
        const int sa = __ldg(g.pa + bp), sb = __ldg(g.pb + bp), sc = __ldg(g.pa + kp), sd = __ldg(g.pb + kp);
        Ctx<Real> c = make_ctx<MD, Real>(g, bp, kp, nullptr);
        const int nbra = c.bra_end - c.bra_begin, nket = c.ket_end - c.ket_begin, nprim = nbra * nket;
        Real acc[NBO];
#pragma unroll
        for (int m = 0; m < NBO; ++m) acc[m] = Real(0);
        for (int o = lane; o < NCD * HP; o += 32) Ws[o] = Real(0);
        for (int i = 0; i < nbra; ++i) {
          for (int j = 0; j < nket; ++j) {
            const int p = i * nket + j;
            if (!batched && (p & 31) == 0) {  // a large quartet: 32 primitive quartets at a time
              __syncwarp();
              const int pp = p + lane;
              if (pp < nprim) {
                const int ii = pp / nket, jj = pp - ii * nket;
                Real Rn[L + 1], X, Y, Z;
                c.template hermite_r0_pp<L>(c.pp(c.bra_begin + ii), c.pp(c.ket_begin + jj), Rn, X, Y, Z);
                Real* b = Bq + lane * SM::BQ;
#pragma unroll
                for (int k = 0; k <= L; ++k) b[k] = Rn[k];
                b[L + 1] = X;
                b[L + 2] = Y;
                b[L + 3] = Z;
              }
              __syncwarp();
            }
            // ---- Hermite Coulomb recursion, level by level
            const Real* b = Bq + (batched ? boff + p : (p & 31)) * SM::BQ;
            const Real X = b[L + 1], Y = b[L + 2], Z = b[L + 3];
            if (lane == 0) R0[0] = b[L];
            __syncwarp();
#pragma unroll
            for (int s = 1; s <= L; ++s) {
              const Real* src = (s & 1) ? R0 : R1;
              Real* dst = (s & 1) ? R1 : R0;
              const int hs = (s + 1) * (s + 2) * (s + 3) / 6;
              for (int x2 = lane; x2 < hs; x2 += 32) {
                const int tuv = s_herm[x2];
                const int t = tuv & 31, u = (tuv >> 5) & 31, v = tuv >> 10;
                // the first non-zero index steps down: (t-1) with X, else (u-1) with Y, else (v-1) with Z
                const int d = t > 0 ? 0 : (u > 0 ? 1 : 2);
                const int m1 = d == 0 ? t : (d == 1 ? u : v);
                const Real C = d == 0 ? X : (d == 1 ? Y : Z);
                const int i1 = herm_index(t - (d == 0), u - (d == 1), v - (d == 2));
                const int i2 = m1 > 1 ? herm_index(t - 2 * (d == 0), u - 2 * (d == 1), v - 2 * (d == 2)) : 0;
                Real val = C * src[x2 == 0 ? 0 : i1];
                val = fma(Real(m1 > 1 ? m1 - 1 : 0), src[i2], val);
                dst[x2] = x2 == 0 ? b[L - s] : val;
              }
              __syncwarp();
            }
            // ---- ket transform into W[cd][h]
            const Real* __restrict__ ek = c.ket_E(c.ket_begin + j);
            for (int m = 0; m < NKO; ++m) {
              const int o = m * 32 + lane;
              const bool act = o < NCD * HP;
              const int cd = act ? o / HP : 0, h = act ? o - cd * HP : 0;
              const unsigned rec = s_ket[cd];
              const int nt = fp_nt(rec), nu = fp_nu(rec), np = fp_np(rec);
              const int cnt = act ? nt * nu * np : 0;
              const int maxc = __reduce_max_sync(kFull, cnt);
              const int ht = s_herm[h];
              const int th = ht & 31, uh = (ht >> 5) & 31, vh = ht >> 10;
              const Real* __restrict__ ep = ek + fp_eoff(rec);
              Real w = act ? Ws[o] : Real(0);
              int ta = 0, nv = 0, ph = 0;
              for (int k = 0; k < maxc; ++k) {
                const bool in = k < cnt;
                const Real ev = in ? ep[k] : Real(0);
                const Real r = Rfin[in ? herm_index(th + ta, uh + nv, vh + ph) : 0];
                w = fma(flip_sign(ev, (ta + nv + ph) & 1), r, w);
                if (++ph == np) {
                  ph = 0;
                  if (++nv == nu) {
                    nv = 0;
                    ++ta;
                  }
                }
              }
              if (act) Ws[o] = w;
            }
            __syncwarp();
          }
          // ---- bra transform of this bra primitive: acc[ab][cd] += E'_ab . W[cd]
          const Real* __restrict__ eb = c.bra_E(c.bra_begin + i);
#pragma unroll
          for (int m = 0; m < NBO; ++m) {
            const int o = m * 32 + lane;
            const bool act = o < NAB * NCD;
            const int ab = act ? o / NCD : 0, cd = act ? o - ab * NCD : 0;
            const unsigned rec = s_bra[ab];
            const int nt = fp_nt(rec), nu = fp_nu(rec), np = fp_np(rec);
            const int cnt = act ? nt * nu * np : 0;
            const int maxc = __reduce_max_sync(kFull, cnt);
            const Real* __restrict__ ep = eb + fp_eoff(rec);
            const Real* __restrict__ wr = Ws + cd * HP;
            Real a = acc[m];
            int ta = 0, nv = 0, ph = 0;
            for (int k = 0; k < maxc; ++k) {
              const bool in = k < cnt;
              const Real ev = in ? ep[k] : Real(0);
              a = fma(ev, wr[in ? herm_index(ta, nv, ph) : 0], a);
              if (++ph == np) {
                ph = 0;
                if (++nv == nu) {
                  nv = 0;
                  ++ta;
                }
              }
            }
            acc[m] = a;
          }
          __syncwarp();
          for (int o = lane; o < NCD * HP; o += 32) Ws[o] = Real(0);
          __syncwarp();
        }
        if (!batched) nas += c.nasym;
        // ---- digestion: every lane its function quartets
        QuartetInfo q{sa, sb, sc, sd, sa == sb, sc == sd, bp == kp, __ldg(g.sh_mol + sa)};
        FockDigest<NB, ND> dg(g, f, q);
#pragma unroll
        for (int m = 0; m < NBO; ++m) {
          const int o = m * 32 + lane;
          if (o < NAB * NCD) {
            const int ab = fp_index(s_bra[o / NCD]), cd = fp_index(s_ket[o % NCD]);
            dg.put(ab / NB, ab % NB, cd / ND, cd % ND, acc[m]);
          }
        }
        nfq += dg.nfq;
        if (lane == 0) {
          ++nsq;
          npq += unsigned(nprim);
          nbp += unsigned(nbra);
        }
      }
      qs = qe;
    }
  }
  if (f.counters) {
    const unsigned s0 = __reduce_add_sync(0xffffffffu, nfq), s1 = __reduce_add_sync(0xffffffffu, nsq),
                   s2 = __reduce_add_sync(0xffffffffu, npq), s3 = __reduce_add_sync(0xffffffffu, nbp),
                   s4 = __reduce_add_sync(0xffffffffu, nas);
    if (lane == 0 && (s0 | s1 | s2)) {
      atomicAdd(f.counters + 0, (unsigned long long)s0);
      atomicAdd(f.counters + 1, (unsigned long long)s1);
      atomicAdd(f.counters + 2, (unsigned long long)s2);
      atomicAdd(f.counters + 3, (unsigned long long)s3);
      atomicAdd(f.counters + 4, (unsigned long long)s4);
    }
  }
}

}  // namespace mmdg
