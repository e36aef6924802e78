// md_kernels.cuh -- the shell-quartet kernels (one instantiation per angular class).
//
// Fock builds (formPT semantics) run in two launches per angular class: k_screen
// walks every candidate (bra shell pair, ket shell pair) of the class and appends
// the survivors of the Schwarz x density bound to bucketed quartet lists (buckets
// keyed by the primitive-count groups of the two pairs, FP64 and FP32 lists); then
// k_fock, a persistent kernel, evaluates the list, one thread per (quartet, ket
// chunk), chunk-major, so a warp shares its code path and, inside a bucket, its
// primitive trip counts.  Short lists and FP32 lists are split by grid stride; long
// FP64 lists are handed out 32 quartets per warp from an atomic counter, so the SMs
// finish together.  The classes above L = 4 have a warp-cooperative Fock kernel of
// their own (md_warp.cuh).  The ERI tensor, the Schwarz table and listed quartets
// use one thread per shell quartet.
#pragma once
#include "md_device.cuh"
#include "md_gen.cuh"

namespace mmdg {

constexpr int kThreads = 128;     // threads per block (shared-memory R tables are sized for it)
constexpr int kMaxFockBlock = 256; // largest block a k_fock launch may use (autotuned tile)

struct ClassLaunch {
  const int* bra;   // shell-pair indices of the bra class list
  const int* ket;   // shell-pair indices of the ket class list
  int nbra, nket;
  int same;         // bra class == ket class: only ket slot <= bra slot
  float qmin, qmax; // screening pass: quartets with Q_bra*Q_ket < qmax go to the FP32 list
  const int* kmoff; // ket list: slot offset of every molecule (lists are molecule-major)
};

__host__ __device__ constexpr int ncart(int l) { return (l + 1) * (l + 2) / 2; }

template <class MD, typename Real>
__device__ __forceinline__ Ctx<Real> make_ctx(const Geometry& g, int bp, int kp, Real* rs) {
  Ctx<Real> c;
  c.g = &g;
  c.chunk = -1;
  c.nasym = 0;
  c.bra_begin = __ldg(g.pr_begin + bp);
  c.bra_end = c.bra_begin + __ldg(g.pr_count + bp);
  c.ket_begin = __ldg(g.pr_begin + kp);
  c.ket_end = c.ket_begin + __ldg(g.pr_count + kp);
  c.ebra = __ldg(g.e_off + bp);
  c.eket = __ldg(g.e_off + kp);
  c.nnz_ab = MD::NNZ_AB;
  c.nnz_cd = MD::NNZ_CD;
  c.rs = rs;
  c.rstr = kThreads;
  return c;
}

// Screening pass of one class pair: every candidate (bra slot, ket slot) is tested
// against the shell-level bound Q_ab Q_cd max(4D_ab, 4D_cd, D_ac, D_ad, D_bc, D_bd)
// (an upper bound of formPT's function-level test, fock.pyx:46-57) and appended to
// the FP64 or the FP32 list of the class.  Each list is split into buckets keyed by
// (bra primitive-count group, ket primitive-count group), so that the 32 quartets a
// warp evaluates together have the same primitive loop trip counts.
struct QuartetLists {
  int2* q64;                  // class region (FP64)
  int2* q32;                  // class region (FP32) or null
  unsigned* n64;              // bucket lengths [nkeys]
  unsigned* n32;
  const long long* key_off;   // bucket offsets within the class region [nkeys]
  const int* gbra;            // slot -> primitive-count group, bra class list
  const int* gket;            // same for the ket class list
  int nkg;                    // groups of the ket class list
  int nkeys;
};

__device__ __forceinline__ void bucket_append(bool keep, int key, int2 v, int2* out, unsigned* n,
                                              const long long* key_off) {
  const unsigned act = __activemask();
  const unsigned peers = __match_any_sync(act, keep ? key : -1);
  if (!keep) return;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(peers) - 1;
  unsigned base = 0;
  if (lane == leader) base = atomicAdd(n + key, (unsigned)__popc(peers));
  base = __shfl_sync(peers, base, leader);
  out[key_off[key] + base + __popc(peers & ((1u << lane) - 1u))] = v;
}

// One block per bra slot; its threads walk the ket slots of the same molecule (the
// lists are molecule-major), so a batch of molecules never forms cross-molecule
// candidates.
static __global__ void __launch_bounds__(kThreads) k_screen(Geometry g, FockArgs f, ClassLaunch cl, QuartetLists ql) {
  const int ib = blockIdx.x;
  if (ib >= cl.nbra) return;
  const int bp = __ldg(cl.bra + ib);
  const int sa = __ldg(g.pa + bp), sb = __ldg(g.pb + bp);
  const int mol = __ldg(g.sh_mol + sa);
  const float qb = __ldg(g.Q + bp);
  const int gb = __ldg(ql.gbra + ib);
  const float* D = f.Dsh + g.mol_sbase[mol];
  const int S = g.mol_ns[mol];
  const int a = __ldg(g.sh_local + sa), b = __ldg(g.sh_local + sb);
  const float dab = 4.0f * __ldg(D + a * S + b);
  const int k0 = __ldg(cl.kmoff + mol);
  int k1 = __ldg(cl.kmoff + mol + 1);
  if (cl.same) k1 = min(k1, ib + 1);
  for (int base = k0; base < k1; base += kThreads) {
    const int jk = base + threadIdx.x;
    bool keep = jk < k1;
    float qq = 0.f;
    int key = 0;
    if (keep) {
      const int kp = __ldg(cl.ket + jk);
      const int sc = __ldg(g.pa + kp), sd = __ldg(g.pb + kp);
      qq = qb * __ldg(g.Q + kp);
      const int c = __ldg(g.sh_local + sc), d = __ldg(g.sh_local + sd);
      const float dm = fmaxf(fmaxf(dab, 4.0f * __ldg(D + c * S + d)),
                             fmaxf(fmaxf(__ldg(D + a * S + c), __ldg(D + a * S + d)),
                                   fmaxf(__ldg(D + b * S + c), __ldg(D + b * S + d))));
      keep = qq * dm >= f.tolf_lo;
      if (f.pair_owner) {
        const int own = __ldg(f.pair_canon + bp) >= __ldg(f.pair_canon + kp) ? __ldg(f.pair_owner + bp)
                                                                              : __ldg(f.pair_owner + kp);
        keep = keep && own == f.part;
      }
      key = gb * ql.nkg + __ldg(ql.gket + jk);
    }
    const bool lo = qq < cl.qmax;  // qmax carries the FP32 split (0: none)
    const int2 v = make_int2(ib, jk);
    bucket_append(keep && !lo, key, v, ql.q64, ql.n64, ql.key_off);
    if (ql.q32) bucket_append(keep && lo, key, v, ql.q32, ql.n32, ql.key_off);
  }
}

constexpr int kMaxKeys = 256;

// Evaluation of a bucketed quartet list: persistent loop over (chunk, bucket,
// quartet), chunk-major, so that a warp shares its chunk (code path) and, inside a
// bucket, its primitive trip counts; heaviest buckets first.
//
// FP64 lists of at least 8 items per thread claim their work dynamically: each warp
// takes the next 32 items from the launch's counter (one atomic per claim, issued one
// claim ahead so its round trip overlaps the work), lane l the item base + l.  With
// the static grid-stride split the average SM sat idle for 20 % of a (ps|ss) launch
// while the slowest finished (ncu: sm__cycles_active avg 9.9M, max 12.4M cycles of
// 12.4M); with the warp kernel's claims (md_warp.cuh) it cut the (H2O)16 class kernels
// run one after another from 44.9 to 38.6 ms and the 4-stream build from 36.4 to
// 34.9 ms (same GPU, two repeats each).  Claims of 128 or 256 items were 1.8-2.7x
// slower (the warps' working set of pairs and E' rows spreads over that many more
// quartets); short lists (a few items per thread: the near quartets of a mixed
// build) and the memory-latency-bound FP32 lists ran 5-35 % slower with claims, so
// they keep the static split.
template <class MD, typename Real>
__global__ void __launch_bounds__(kMaxFockBlock) k_fock(Geometry g, FockArgs f, ClassLaunch cl, const int2* list,
                                                   const unsigned* count, const long long* key_off, int nkeys) {
  __shared__ unsigned s_pre[kMaxKeys + 1];
  __shared__ long long s_off[kMaxKeys];
  if (threadIdx.x == 0) {
    unsigned acc = 0;
    for (int k = 0; k < nkeys; ++k) {
      s_pre[k] = acc;
      s_off[k] = key_off[k];
      acc += count[k];
    }
    s_pre[nkeys] = acc;
  }
  __syncthreads();
  const unsigned n = s_pre[nkeys];
  const long long total = (long long)n * MD::NCHUNK;
  extern __shared__ double smem_d[];
  Real* rs = reinterpret_cast<Real*>(smem_d) + threadIdx.x;
  unsigned nfq = 0, nsq = 0, npq = 0, nbp = 0, nas = 0;
  int key = 0;
  // block size: kThreads for classes with shared-memory R tables, else 64..256 (tile),
  // a multiple of 32 either way, so every warp is full
  const long long nthreads = (long long)gridDim.x * blockDim.x;
  const bool dynamic = sizeof(Real) == 8 && total >= 8 * nthreads;
  const unsigned lane = threadIdx.x & 31u;
  unsigned long long base = 0, next = 0;
  long long sidx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (dynamic) {
    if (lane == 0) base = atomicAdd(f.work, 32ull);
    base = __shfl_sync(0xffffffffu, base, 0);
  }
  for (;;) {
    long long idx;
    if (dynamic) {
      if (base >= (unsigned long long)total) break;  // warp-uniform
      if (lane == 0) next = atomicAdd(f.work, 32ull);  // the next claim, in flight during this one
      idx = (long long)base + lane;
    } else {
      if (sidx >= total) break;
      idx = sidx;
    }
    if (idx < total) {
      const int chunk = (int)(idx / n);
      // buckets run from the heaviest (most primitive pairs, stored last) to the
      // lightest, so the loop's last rounds hold the cheapest quartets
      const unsigned r = n - 1u - (unsigned)(idx - (long long)chunk * n);
      if (r < s_pre[key]) key = 0;
      while (r >= s_pre[key + 1]) ++key;
      const int2 e = list[s_off[key] + (r - s_pre[key])];
      const int bp = __ldg(cl.bra + e.x), kp = __ldg(cl.ket + e.y);
      const int sa = __ldg(g.pa + bp), sb = __ldg(g.pb + bp), sc = __ldg(g.pa + kp), sd = __ldg(g.pb + kp);
      Ctx<Real> c = make_ctx<MD, Real>(g, bp, kp, rs);
      c.chunk = MD::NCHUNK > 1 ? chunk : -1;
      QuartetInfo q{sa, sb, sc, sd, sa == sb, sc == sd, bp == kp, __ldg(g.sh_mol + sa)};
      FockDigest<ncart(MD::LB), ncart(MD::LD)> dg(g, f, q);
      MD::run(c, dg);
      nfq += dg.nfq;
      if (chunk == 0) {
        ++nsq;
        npq += unsigned((c.bra_end - c.bra_begin) * (c.ket_end - c.ket_begin));
        nbp += unsigned(c.bra_end - c.bra_begin);
        nas += c.nasym;
      }
    }
    if (dynamic) base = __shfl_sync(0xffffffffu, next, 0);
    else sidx += nthreads;
  }
  if (f.counters) {
    const unsigned mask = __activemask();
    const unsigned s0 = __reduce_add_sync(mask, nfq), s1 = __reduce_add_sync(mask, nsq),
                   s2 = __reduce_add_sync(mask, npq), s3 = __reduce_add_sync(mask, nbp),
                   s4 = __reduce_add_sync(mask, nas);
    if ((threadIdx.x & 31) == __ffs(mask) - 1 && (s0 | s1 | s2)) {
      atomicAdd(f.counters + 0, (unsigned long long)s0);
      atomicAdd(f.counters + 1, (unsigned long long)s1);
      atomicAdd(f.counters + 2, (unsigned long long)s2);
      atomicAdd(f.counters + 3, (unsigned long long)s3);
      atomicAdd(f.counters + 4, (unsigned long long)s4);
    }
  }
}

template <class MD>
__global__ void __launch_bounds__(kThreads) k_tensor(Geometry g, TensorArgs t, ClassLaunch cl) {
  const int ib = blockIdx.x;
  const int jk = blockIdx.y * kThreads + threadIdx.x;
  if (ib >= cl.nbra || jk >= cl.nket) return;
  if (cl.same && jk > ib) return;
  const int bp = __ldg(cl.bra + ib), kp = __ldg(cl.ket + jk);
  const int sa = __ldg(g.pa + bp), sb = __ldg(g.pb + bp), sc = __ldg(g.pa + kp), sd = __ldg(g.pb + kp);
  const int mol = __ldg(g.sh_mol + sa);
  if (__ldg(g.sh_mol + sc) != mol) return;
  extern __shared__ double smem_d[];
  double* rs = smem_d + threadIdx.x;
  Ctx<double> c = make_ctx<MD, double>(g, bp, kp, rs);
  c.chunk = MD::NCHUNK > 1 ? (int)blockIdx.z : -1;  // one ket chunk per grid z-slice
  QuartetInfo q{sa, sb, sc, sd, sa == sb, sc == sd, bp == kp, mol};
  TensorDigest<ncart(MD::LB), ncart(MD::LD)> dg(g, t, q);
  MD::run(c, dg);
}

// listed shell quartets of one class (mmdg_eri_quartets): one thread per (item, ket
// chunk), chunk-major
template <class MD, typename Real>
__global__ void __launch_bounds__(kThreads) k_quartets(Geometry g, QuartetArgs a, const QuartetItem* items, int n) {
  const long long idx = blockIdx.x * (long long)kThreads + threadIdx.x;
  if (idx >= (long long)n * MD::NCHUNK) return;
  const int chunk = (int)(idx / n);
  const QuartetItem it = items[idx - (long long)chunk * n];
  extern __shared__ double smem_d[];
  Real* rs = reinterpret_cast<Real*>(smem_d) + threadIdx.x;
  Ctx<Real> c = make_ctx<MD, Real>(g, it.bra, it.ket, rs);
  c.chunk = MD::NCHUNK > 1 ? chunk : -1;
  QuartetDigest<ncart(MD::LB), ncart(MD::LD)> dg(a, it.slot, it.flags);
  MD::run(c, dg);
}

// diagonal quartets (ab|ab) of one pair class: the Schwarz table
// (one thread per (pair, ket chunk), chunk-major)
template <class MD>
__global__ void __launch_bounds__(kThreads) k_schwarz(Geometry g, SchwarzArgs s, const int* list, int n) {
  const long long idx = blockIdx.x * (long long)kThreads + threadIdx.x;
  if (idx >= (long long)n * MD::NCHUNK) return;
  const int chunk = (int)(idx / n);
  const int bp = __ldg(list + (idx - (long long)chunk * n));
  const int sa = __ldg(g.pa + bp), sb = __ldg(g.pb + bp);
  extern __shared__ double smem_d[];
  double* rs = smem_d + threadIdx.x;
  Ctx<double> c = make_ctx<MD, double>(g, bp, bp, rs);
  c.chunk = MD::NCHUNK > 1 ? chunk : -1;
  QuartetInfo q{sa, sb, sa, sb, sa == sb, sa == sb, true, __ldg(g.sh_mol + sa)};
  SchwarzDigest<ncart(MD::LB), ncart(MD::LD)> dg(g, s, q, bp);
  MD::run(c, dg);
}

template <class MD, typename Real>
constexpr size_t smem_bytes() {
  return MD::RSMEM ? size_t(MD::HL) * kThreads * sizeof(Real) : 0;
}

}  // namespace mmdg

namespace mmdg {
// blocks of a persistent launch: every SM filled to the kernel's occupancy
// (grid > 0: an autotuned grid, capped at that occupancy)
template <typename K>
inline int persistent_blocks(K kernel, size_t smem, int grid = 0, int block = kThreads) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, block, smem);
  const int full = sms * (per > 0 ? per : 1);
  return grid > 0 && grid < full ? grid : full;
}
}  // namespace mmdg
