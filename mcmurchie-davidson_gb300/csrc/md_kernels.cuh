// md_kernels.cuh -- the shell-quartet kernels (one instantiation per angular class).
//
// One thread evaluates one contracted shell quartet (ab|cd) of a class list pair:
//   blockIdx.x        -> bra shell pair (slot in the bra class list)
//   blockIdx.y*128+tx -> ket shell pair (slot in the ket class list)
// Class lists are sorted by (primitive count, Schwarz bound descending), so a warp's
// 32 kets share their primitive loop trip counts and their screening outcome.
#pragma once
#include "md_device.cuh"
#include "md_gen.cuh"

namespace mmdg {

constexpr int kThreads = 128;

struct ClassLaunch {
  const int* bra;   // shell-pair indices of the bra class list
  const int* ket;   // shell-pair indices of the ket class list
  int nbra, nket;
  int same;         // bra class == ket class: only ket slot <= bra slot
  float qmin, qmax; // compute only quartets with qmin <= Q_bra*Q_ket < qmax (precision split)
};

__host__ __device__ constexpr int ncart(int l) { return (l + 1) * (l + 2) / 2; }

template <class MD, typename Real>
__device__ __forceinline__ Ctx<Real> make_ctx(const Geometry& g, int bp, int kp, Real* rs) {
  Ctx<Real> c;
  c.g = &g;
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

template <class MD, typename Real>
__global__ void __launch_bounds__(kThreads) k_fock(Geometry g, FockArgs f, ClassLaunch cl) {
  const int ib = blockIdx.x;
  const int jk = blockIdx.y * kThreads + threadIdx.x;
  if (ib >= cl.nbra || jk >= cl.nket) return;
  if (cl.same && jk > ib) return;
  const int bp = __ldg(cl.bra + ib), kp = __ldg(cl.ket + jk);
  const int sa = __ldg(g.pa + bp), sb = __ldg(g.pb + bp), sc = __ldg(g.pa + kp), sd = __ldg(g.pb + kp);
  const int mol = __ldg(g.sh_mol + sa);
  bool work = __ldg(g.sh_mol + sc) == mol;
  const float qq = __ldg(g.Q + bp) * __ldg(g.Q + kp);
  work = work && qq >= cl.qmin && qq < cl.qmax;
  if (work) {
    const float* D = f.Dsh + g.mol_sbase[mol];
    const int S = g.mol_ns[mol];
    const int a = __ldg(g.sh_local + sa), b = __ldg(g.sh_local + sb);
    const int c = __ldg(g.sh_local + sc), d = __ldg(g.sh_local + sd);
    const float dm = fmaxf(4.0f * fmaxf(__ldg(D + a * S + b), __ldg(D + c * S + d)),
                           fmaxf(fmaxf(__ldg(D + a * S + c), __ldg(D + a * S + d)),
                                 fmaxf(__ldg(D + b * S + c), __ldg(D + b * S + d))));
    work = qq * dm >= f.tolf_lo;
  }
  unsigned nfq = 0, nsq = 0, npq = 0;
  if (work) {
    extern __shared__ double smem_d[];
    Real* rs = reinterpret_cast<Real*>(smem_d) + threadIdx.x;
    Ctx<Real> c = make_ctx<MD, Real>(g, bp, kp, rs);
    QuartetInfo q{sa, sb, sc, sd, sa == sb, sc == sd, bp == kp, mol};
    FockDigest<ncart(MD::LB), ncart(MD::LD)> dg(g, f, q);
    MD::run(c, dg);
    nfq = dg.nfq;
    nsq = 1;
    npq = unsigned((c.bra_end - c.bra_begin) * (c.ket_end - c.ket_begin));
  }
  if (f.counters) {
    const unsigned mask = __activemask();
    const unsigned s0 = __reduce_add_sync(mask, nfq), s1 = __reduce_add_sync(mask, nsq),
                   s2 = __reduce_add_sync(mask, npq);
    if ((threadIdx.x & 31) == __ffs(mask) - 1 && s1) {
      atomicAdd(f.counters + 0, (unsigned long long)s0);
      atomicAdd(f.counters + 1, (unsigned long long)s1);
      atomicAdd(f.counters + 2, (unsigned long long)s2);
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
  QuartetInfo q{sa, sb, sc, sd, sa == sb, sc == sd, bp == kp, mol};
  TensorDigest<ncart(MD::LB), ncart(MD::LD)> dg(g, t, q);
  MD::run(c, dg);
}

// diagonal quartets (ab|ab) of one pair class: the Schwarz table
template <class MD>
__global__ void __launch_bounds__(kThreads) k_schwarz(Geometry g, SchwarzArgs s, const int* list, int n) {
  const int idx = blockIdx.x * kThreads + threadIdx.x;
  if (idx >= n) return;
  const int bp = __ldg(list + idx);
  const int sa = __ldg(g.pa + bp), sb = __ldg(g.pb + bp);
  extern __shared__ double smem_d[];
  double* rs = smem_d + threadIdx.x;
  Ctx<double> c = make_ctx<MD, double>(g, bp, bp, rs);
  QuartetInfo q{sa, sb, sa, sb, sa == sb, sa == sb, true, __ldg(g.sh_mol + sa)};
  SchwarzDigest<ncart(MD::LB), ncart(MD::LD)> dg(g, s, q, bp);
  MD::run(c, dg);
}

template <class MD, typename Real>
constexpr size_t smem_bytes() {
  return MD::RSMEM ? size_t(MD::HL) * kThreads * sizeof(Real) : 0;
}

}  // namespace mmdg
