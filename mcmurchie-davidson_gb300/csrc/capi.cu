// capi.cu -- C ABI (include/mmdg.h): context, basis set-up, primitive pairs,
// Schwarz table, Fock builds, ERI tensor, Boys evaluation.
//
// Host-side bookkeeping (shell pairs, class lists, offsets) is integer work done
// once per basis; every floating-point quantity of the hot path is computed on
// the GPU by the kernels below and in md_inst*.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/mmdg.h"
#include "md_dispatch.cuh"

using namespace mmdg;

// ------------------------------------------------------------------ errors
// fixed-size, so that recording an error never allocates
static thread_local char g_last_error[512];

static int fail_c(int code, const char* msg) {
  std::strncpy(g_last_error, msg, sizeof(g_last_error) - 1);
  g_last_error[sizeof(g_last_error) - 1] = 0;
  return code;
}
static int fail(int code, const std::string& msg) { return fail_c(code, msg.c_str()); }
#define CUDA_TRY(x)                                                                                  \
  do {                                                                                               \
    cudaError_t e_ = (x);                                                                            \
    if (e_ != cudaSuccess) return fail(MMDG_E_CUDA, std::string(#x ": ") + cudaGetErrorString(e_)); \
  } while (0)

extern "C" const char* mmdg_last_error(void) { return g_last_error; }

int mmdg_internal_fail(int code, const char* msg) { return fail_c(code, msg); }

// ------------------------------------------------------------------ device buffers
template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t alloc(size_t count) {
    release();
    n = count;
    if (count == 0) return cudaSuccess;
    return cudaMalloc(reinterpret_cast<void**>(&p), count * sizeof(T));
  }
  cudaError_t upload(const std::vector<T>& v) {
    cudaError_t e = alloc(v.size());
    if (e != cudaSuccess || v.empty()) return e;
    return cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
  }
};

// ------------------------------------------------------------------ Boys table
// F_m(T_k), T_k = k/16, by the Kummer-transformed series
//   F_m(T) = exp(-T) / (2m+1) * sum_i T^i / ((m+3/2)(m+5/2)...(m+1/2+i))
// at the highest order m = 14, then downward recursion
//   F_{m-1} = (2T F_m + exp(-T)) / (2m-1),
// all in double-double arithmetic (error-free transformations with fma), so the
// table is correctly rounded to double and identical on every host.
namespace {
struct dd {
  double hi, lo;
};
inline dd two_sum(double a, double b) {
  double s = a + b, bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
inline dd quick_two_sum(double a, double b) {
  double s = a + b;
  return {s, b - (s - a)};
}
inline dd dd_add(dd a, dd b) {
  dd s = two_sum(a.hi, b.hi);
  s.lo += a.lo + b.lo;
  return quick_two_sum(s.hi, s.lo);
}
inline dd dd_mul(dd a, dd b) {
  double p = a.hi * b.hi;
  double e = std::fma(a.hi, b.hi, -p);
  e += a.hi * b.lo + a.lo * b.hi;
  return quick_two_sum(p, e);
}
inline dd dd_mul_d(dd a, double b) {
  double p = a.hi * b;
  double e = std::fma(a.hi, b, -p);
  e += a.lo * b;
  return quick_two_sum(p, e);
}
inline dd dd_div_d(dd a, double b) {
  double q1 = a.hi / b;
  dd r = dd_add(a, dd_mul_d({q1, 0.0}, -b));
  double q2 = r.hi / b;
  r = dd_add(r, dd_mul_d({q2, 0.0}, -b));
  double q3 = r.hi / b;
  dd q = quick_two_sum(q1, q2);
  return dd_add(q, {q3, 0.0});
}
// exp(-x) for x = 1/16 by its Taylor series in double-double
dd dd_exp_m16() {
  dd term{1.0, 0.0}, sum{1.0, 0.0};
  for (int n = 1; n < 40; ++n) {
    term = dd_div_d(term, -16.0 * n);
    sum = dd_add(sum, term);
  }
  return sum;
}
}  // namespace

// Fills t64 (kBoysTabSize doubles) and, if non-null, t32; no heap allocation.
static void build_boys_table_raw(double* t64, float* t32) {
  for (int i = 0; i < kBoysTabSize; ++i) t64[i] = 0.0;
  const dd e16 = dd_exp_m16();
  dd eT{1.0, 0.0};
  const int mtop = kBoysLMax + 6;  // F_0 .. F_14
  double fact[8] = {1, 1, 2, 6, 24, 120, 720, 5040};
  for (int k = 0; k < kBoysNGrid; ++k) {
    if (k > 0) eT = dd_mul(eT, e16);
    const double T = k / 16.0;
    // series at m = mtop
    dd term{1.0, 0.0}, sum{1.0, 0.0};
    const double b = mtop + 1.5;
    for (int i = 0; i < 4000; ++i) {
      term = dd_div_d(dd_mul_d(term, T), b + i);
      sum = dd_add(sum, term);
      if (term.hi < sum.hi * 1e-34) break;
    }
    dd F[mtop + 1];
    F[mtop] = dd_div_d(dd_mul(eT, sum), 2.0 * mtop + 1.0);
    for (int m = mtop; m > 0; --m) F[m - 1] = dd_div_d(dd_add(dd_mul_d(F[m], 2.0 * T), eT), 2.0 * m - 1.0);
    for (int L = 0; L <= kBoysLMax; ++L) {
      for (int n = 0; n < 7; ++n) {
        const dd v = dd_div_d(F[L + n], fact[n]);
        t64[(L * kBoysNGrid + k) * kBoysRow + n] = v.hi + v.lo;
      }
      t64[(L * kBoysNGrid + k) * kBoysRow + 7] = T;  // the grid point, exact (k/16)
    }
    for (int n = 0; n < 8; ++n) {
      const dd v = dd_div_d(eT, fact[n]);
      t64[kBoysExpOff + k * kBoysRow + n] = v.hi + v.lo;
    }
  }
  if (t32)
    for (int i = 0; i < kBoysTabSize; ++i) t32[i] = float(t64[i]);
}

// computed once per process (every context uploads the same table)
static void build_boys_table(std::vector<double>& t64, std::vector<float>& t32) {
  static std::mutex mu;
  static std::vector<double> c64;
  static std::vector<float> c32;
  std::lock_guard<std::mutex> lock(mu);
  if (c64.empty()) {
    c64.assign(kBoysTabSize, 0.0);
    c32.assign(kBoysTabSize, 0.0f);
    build_boys_table_raw(c64.data(), c32.data());
  }
  t64 = c64;
  t32 = c32;
}

// ------------------------------------------------------------------ context
static int nnz_pair(int la, int lb) {
  int n = 0;
  for (int xa = la; xa >= 0; --xa)
    for (int ya = la - xa; ya >= 0; --ya) {
      int za = la - xa - ya;
      for (int xb = lb; xb >= 0; --xb)
        for (int yb = lb - xb; yb >= 0; --yb) {
          int zb = lb - xb - yb;
          n += (xa + xb + 1) * (ya + yb + 1) * (za + zb + 1);
        }
    }
  return n;
}
static int pair_class(int la, int lb) { return la * (la + 1) / 2 + lb; }
static const int kNumPairClasses = (MMDG_LMAX + 1) * (MMDG_LMAX + 2) / 2;
static const int kMaxStreams = 8;  // concurrent class streams of a Fock build

struct mmdg_context {
  int device = 0;
  bool have_basis = false;
  DevBuf<double> boys64;
  DevBuf<float> boys32;
  DevBuf<float> boysdf;  // the FP64 rows as (hi, lo) float pairs
  // basis
  int nmol = 0, nshell = 0;
  std::vector<int> mol_n, mol_ns;
  std::vector<long long> mol_base, mol_sbase, mol_tbase;
  long long ntot_nn = 0, ntot_ss = 0, ntot_tri = 0;
  DevBuf<double> d_center, d_exp, d_coef;
  DevBuf<int> d_L, d_nprim, d_poff, d_func, d_shmol, d_shlocal;
  DevBuf<long long> d_mol_base, d_mol_sbase, d_mol_tbase;
  DevBuf<int> d_mol_n, d_mol_ns;
  // primitive pairs whose Schwarz factor times the largest one is below prim_tol are
  // not stored (0: keep all); set before the basis (mmdg_set_prim_tol)
  double prim_tol = 1e-18;
  // pairs
  int npair = 0;
  long long nprimpair = 0, nE = 0;
  std::vector<int> pa, pb, pcls, pr_begin, pr_count;
  std::vector<long long> e_off;
  std::vector<int> pair_row;  // pair index of (s1, s1); (s1, s2 <= s1) is pair_row[s1] + s1 - s2
  std::vector<int> shell_L, shell_molv;
  DevBuf<int> d_pa, d_pb, d_prb, d_prc;
  DevBuf<long long> d_eoff;
  DevBuf<double4_32a> d_pP;
  DevBuf<float4> d_pPf;
  DevBuf<double> d_E64;
  DevBuf<float> d_E32;
  DevBuf<float> d_Q;
  // class lists (sorted by primitive count, then Q descending)
  std::vector<int> cls_count;
  DevBuf<int> d_cls[kNumPairClasses];
  DevBuf<int> d_cls_moff[kNumPairClasses];  // per class list: slot offset of every molecule [nmol+1]
  std::vector<std::vector<long long>> bucket_cap;  // per angular class: capacity of every bucket
  std::vector<long long> mol_shell0;        // first global shell of every molecule
  DevBuf<long long> d_mol_shell0;
  // tuning (autotuner): persistent grid per class (0 = occupancy), concurrent class streams
  int class_grid[MMDG_NCLASS] = {0};
  int class_block[MMDG_NCLASS] = {0};  // threads per block of the per-thread kernels (0: 128)
  int class_item[MMDG_NCLASS] = {0};   // quartets per work item of the warp kernels (0: adaptive up to 8)
  int nstreams = 1;
  cudaStream_t side[kMaxStreams] = {};
  cudaEvent_t fork_ev = nullptr, join_ev[kMaxStreams] = {};
  // CUDA graph of one Fock build (mmdg_fock_graph)
  cudaGraphExec_t graph = nullptr;
  const double* g_dP = nullptr;
  double* g_G = nullptr;
  double g_tol = -1.0, g_split = -1.0;
  cudaStream_t g_stream = nullptr;
  // sharded Fock build: owner of every shell pair and its canonical index
  DevBuf<int> d_pair_owner, d_pair_canon;
  int part = 0, nparts = 1;
  // screening / Fock scratch
  DevBuf<double> d_screen, d_sq;
  DevBuf<float> d_sqf, d_dPf, d_Dsh;
  DevBuf<unsigned long long> d_counters;
  // quartet lists of the Fock build (allocated on first use): per class a region of
  // capacity = number of candidate quartets, for FP64 and (on demand) FP32
  std::vector<long long> q_off, q_cap;
  long long q_total = 0;
  DevBuf<int2> d_q64, d_q32;
  // buckets: per pair-class list, slots grouped by primitive count; per class
  // (bra group, ket group) buckets with their offsets inside the class region
  std::vector<int> ngroup;
  DevBuf<int> d_gslot[kNumPairClasses];
  std::vector<int> kbase, nkeys;
  int total_keys = 0;
  DevBuf<long long> d_keyoff;
  DevBuf<unsigned> d_qn;  // [2*total_keys]: FP64 and FP32 bucket lengths
  DevBuf<unsigned long long> d_work;  // [2*MMDG_NCLASS]: work counters of the FP64 and FP32 class launches
  Geometry geom() const {
    Geometry g;
    g.pP = d_pP.p;
    g.pPf = d_pPf.p;
    g.E64 = d_E64.p;
    g.E32 = d_E32.p;
    g.pr_begin = d_prb.p;
    g.pr_count = d_prc.p;
    g.e_off = d_eoff.p;
    g.pa = d_pa.p;
    g.pb = d_pb.p;
    g.Q = d_Q.p;
    g.func = d_func.p;
    g.sh_mol = d_shmol.p;
    g.sh_local = d_shlocal.p;
    g.mol_base = d_mol_base.p;
    g.mol_n = d_mol_n.p;
    g.mol_sbase = d_mol_sbase.p;
    g.mol_ns = d_mol_ns.p;
    g.mol_tbase = d_mol_tbase.p;
    g.boys64 = boys64.p;
    g.boys32 = boys32.p;
    g.boysdf = boysdf.p;
    return g;
  }
};

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

extern "C" int mmdg_create(mmdg_context** out, int device) {
  if (!out) return fail(MMDG_E_ARG, "mmdg_create: null output pointer");
  int ndev = 0;
  CUDA_TRY(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev) return fail(MMDG_E_ARG, "mmdg_create: no such CUDA device");
  DeviceGuard dg(device);
  mmdg_context* h = new mmdg_context();
  h->device = device;
  std::vector<double> t64;
  std::vector<float> t32;
  build_boys_table(t64, t32);
  std::vector<float> tdf((size_t)kBoysTabSize / kBoysRow * kBoysDfRow);
  for (int r = 0; r < kBoysTabSize / kBoysRow; ++r)
    for (int j = 0; j < kBoysRow; ++j) {
      const double c = t64[(size_t)r * kBoysRow + j];
      const float hi = float(c);
      tdf[(size_t)r * kBoysDfRow + j] = hi;
      tdf[(size_t)r * kBoysDfRow + kBoysRow + j] = float(c - double(hi));
    }
  if (h->boys64.upload(t64) != cudaSuccess || h->boys32.upload(t32) != cudaSuccess ||
      h->boysdf.upload(tdf) != cudaSuccess) {
    delete h;
    return fail(MMDG_E_NOMEM, "mmdg_create: cannot allocate the Boys tables");
  }
  for (int g = 0; g < kNumGroups; ++g) {
    cudaError_t e = kGroupInit[g]();
    if (e != cudaSuccess) {
      delete h;
      return fail(MMDG_E_CUDA, std::string("mmdg_create: kernel set-up: ") + cudaGetErrorString(e));
    }
  }
  *out = h;
  return MMDG_OK;
}

extern "C" int mmdg_destroy(mmdg_context* h) {
  if (!h) return MMDG_OK;
  DeviceGuard dg(h->device);
  if (h->graph) cudaGraphExecDestroy(h->graph);
  for (int k = 0; k < kMaxStreams; ++k) {
    if (h->side[k]) cudaStreamDestroy(h->side[k]);
    if (h->join_ev[k]) cudaEventDestroy(h->join_ev[k]);
  }
  if (h->fork_ev) cudaEventDestroy(h->fork_ev);
  if (h->g_stream) cudaStreamDestroy(h->g_stream);
  delete h;
  return MMDG_OK;
}

// ------------------------------------------------------------------ pair kernel
// One thread per shell pair: primitive-pair data (p, P) and the E' tables
//   E'[fa fb][t u v] = c_a c_b exp(-mu |AB|^2) / p * n(fa) n(fb) * Ex_t Ey_u Ez_v
// with the 1D Hermite expansion coefficients of cython/util.pxi:13-28 built by
// the same recursion (base E_0^{00} = 1; the Gaussian factor is K_ab):
//   E^{i+1,j}_t = E^{ij}_{t-1}/(2p) + X_PA E^{ij}_t + (t+1) E^{ij}_{t+1}
//   E^{i,j+1}_t = E^{ij}_{t-1}/(2p) + X_PB E^{ij}_t + (t+1) E^{ij}_{t+1}
// n(lmn) = 1/sqrt((2l-1)!!(2m-1)!!(2n-1)!!) is the component part of the
// primitive normalisation of cython/basis.pxi:101-105.
__device__ __forceinline__ double comp_norm(int l) { return l >= 2 ? 0.57735026918962576 : 1.0; }

#include "pairs.cuh"

__global__ void k_build_pairs(PairBuildArgs a) {
  const int pr = blockIdx.x * blockDim.x + threadIdx.x;
  if (pr >= a.npair) return;
  const int sa = a.pa[pr], sb = a.pb[pr];
  const int la = a.L[sa], lb = a.L[sb];
  const int Ka = a.nprim[sa], Kb = a.nprim[sb];
  const double Ax = a.center[3 * sa], Ay = a.center[3 * sa + 1], Az = a.center[3 * sa + 2];
  const double Bx = a.center[3 * sb], By = a.center[3 * sb + 1], Bz = a.center[3 * sb + 2];
  const double ABx = Ax - Bx, ABy = Ay - By, ABz = Az - Bz;
  const double AB2 = ABx * ABx + ABy * ABy + ABz * ABz;
  int nnz = 0;
  for (int xa = la; xa >= 0; --xa)
    for (int ya = la - xa; ya >= 0; --ya)
      for (int xb = lb; xb >= 0; --xb)
        for (int yb = lb - xb; yb >= 0; --yb)
          nnz += (xa + xb + 1) * (ya + yb + 1) * ((la - xa - ya) + (lb - xb - yb) + 1);
  const double AB[3] = {ABx, ABy, ABz};
  const int nkeep = a.keep ? a.prc[pr] : Ka * Kb;
  for (int k = 0; k < nkeep; ++k) {
    const int kk = a.keep ? __ldg(a.keep + a.prb[pr] + k) : k;
    const int ka = kk / Kb, kb = kk - ka * Kb;
    const double ea = a.exps[a.poff[sa] + ka], eb = a.exps[a.poff[sb] + kb];
    const double p = ea + eb, ip = 1.0 / p, mu = ea * eb * ip;
    const double Px = (ea * Ax + eb * Bx) * ip, Py = (ea * Ay + eb * By) * ip, Pz = (ea * Az + eb * Bz) * ip;
    const double K = exp(-mu * AB2) * a.coefs[a.poff[sa] + ka] * a.coefs[a.poff[sb] + kb] * ip;
    const long long pp = a.prb[pr] + k;
    a.pP[pp] = make_double4_32a(p, Px, Py, Pz);
    if (a.pPf) {
      const float hx = float(Px), hy = float(Py), hz = float(Pz);
      a.pPf[2 * pp] = make_float4(float(p), hx, hy, hz);
      a.pPf[2 * pp + 1] = make_float4(0.f, float(Px - hx), float(Py - hy), float(Pz - hz));
    }
    // 1D tables E[d][i][j][t], i<=2, j<=2, t<=4
    double E[3][3][3][5];
    const double i2p = 0.5 * ip;
    for (int d = 0; d < 3; ++d) {
      const double XPA = -(eb * ip) * AB[d], XPB = (ea * ip) * AB[d];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          for (int t = 0; t < 5; ++t) E[d][i][j][t] = 0.0;
      E[d][0][0][0] = 1.0;
      for (int i = 0; i < la; ++i)
        for (int t = 0; t <= i + 1; ++t) {
          double v = XPA * E[d][i][0][t];
          if (t > 0) v += i2p * E[d][i][0][t - 1];
          if (t + 1 <= i) v += (t + 1) * E[d][i][0][t + 1];
          E[d][i + 1][0][t] = v;
        }
      for (int j = 0; j < lb; ++j)
        for (int i = 0; i <= la; ++i)
          for (int t = 0; t <= i + j + 1; ++t) {
            double v = XPB * E[d][i][j][t];
            if (t > 0) v += i2p * E[d][i][j][t - 1];
            if (t + 1 <= i + j) v += (t + 1) * E[d][i][j][t + 1];
            E[d][i][j + 1][t] = v;
          }
    }
    long long o = a.eoff[pr] + (long long)k * nnz;
    for (int xa = la; xa >= 0; --xa)
      for (int ya = la - xa; ya >= 0; --ya) {
        const int za = la - xa - ya;
        const double na = comp_norm(xa) * comp_norm(ya) * comp_norm(za);
        for (int xb = lb; xb >= 0; --xb)
          for (int yb = lb - xb; yb >= 0; --yb) {
            const int zb = lb - xb - yb;
            // sqrt(2 pi^{5/2}) per coefficient: a bra-ket product carries the
            // primitive ERI's 2 pi^{5/2} (cython/twoe.pyx:93)
            const double c = kSqrtTwoPi52 * K * na * comp_norm(xb) * comp_norm(yb) * comp_norm(zb);
            for (int t = 0; t <= xa + xb; ++t)
              for (int u = 0; u <= ya + yb; ++u)
                for (int v = 0; v <= za + zb; ++v) {
                  const double e = c * E[0][xa][xb][t] * E[1][ya][yb][u] * E[2][za][zb][v];
                  a.E64[o] = e;
                  if (a.E32) a.E32[o] = float(e);
                  ++o;
                }
          }
      }
  }
}

// sqrt of the screen table (FP64 and FP32 copies)
__global__ void k_sqrt_screen(const double* screen, double* sq, float* sqf, long long n) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double s = sqrt(fmax(screen[i], 0.0));
  sq[i] = s;
  sqf[i] = float(s);
}

// ------------------------------------------------------------------ set basis
// At most kMaxGroups primitive-count groups per pair-class list, so that a class has
// at most kMaxGroups^2 (bra group, ket group) buckets.
static const int kMaxGroups = 16;

// Partition of the sorted distinct primitive counts vals (with their frequencies)
// into at most gmax contiguous ranges minimising the idle lane iterations
// sum_t freq_t (max of its range - vals_t); returns the range index of every value.
static std::vector<int> group_counts(const std::vector<int>& vals, const std::vector<long long>& freq, int gmax) {
  const int m = (int)vals.size();
  std::vector<int> grp(m);
  if (m <= gmax) {
    for (int i = 0; i < m; ++i) grp[i] = i;
    return grp;
  }
  std::vector<double> F(m + 1, 0.0), S(m + 1, 0.0);
  for (int i = 0; i < m; ++i) {
    F[i + 1] = F[i] + double(freq[i]);
    S[i + 1] = S[i] + double(freq[i]) * vals[i];
  }
  auto cost = [&](int i, int j) { return double(vals[j]) * (F[j + 1] - F[i]) - (S[j + 1] - S[i]); };
  const double inf = 1e300;
  std::vector<std::vector<double>> dp(gmax + 1, std::vector<double>(m, inf));
  std::vector<std::vector<int>> cut(gmax + 1, std::vector<int>(m, 0));
  for (int j = 0; j < m; ++j) dp[1][j] = cost(0, j);
  for (int g = 2; g <= gmax; ++g)
    for (int j = g - 1; j < m; ++j)
      for (int i = g - 1; i <= j; ++i) {
        const double c = dp[g - 1][i - 1] + cost(i, j);
        if (c < dp[g][j]) {
          dp[g][j] = c;
          cut[g][j] = i;
        }
      }
  for (int g = gmax, j = m - 1; g >= 1; --g) {
    const int i = g > 1 ? cut[g][j] : 0;
    for (int t = i; t <= j; ++t) grp[t] = g - 1;
    j = i - 1;
  }
  return grp;
}

extern "C" int mmdg_set_basis(mmdg_context* h, int nmol, const int* mol_nfunc, int nshell, const int* shell_mol,
                              const int* shell_L, const int* shell_nprim, const double* shell_center,
                              const double* prim_exp, const double* prim_coef, const int* shell_func) {
  if (!h) return fail(MMDG_E_ARG, "mmdg_set_basis: null context");
  if (nmol < 1 || nshell < 1 || !mol_nfunc || !shell_mol || !shell_L || !shell_nprim || !shell_center ||
      !prim_exp || !prim_coef || !shell_func)
    return fail(MMDG_E_ARG, "mmdg_set_basis: empty basis or null array");
  DeviceGuard dgd(h->device);
  h->have_basis = false;
  // ---- molecules and shells
  h->nmol = nmol;
  h->nshell = nshell;
  h->mol_n.assign(mol_nfunc, mol_nfunc + nmol);
  h->mol_ns.assign(nmol, 0);
  std::vector<int> shlocal(nshell), poff(nshell);
  int total_prim = 0;
  for (int s = 0; s < nshell; ++s) {
    const int m = shell_mol[s];
    if (m < 0 || m >= nmol) return fail(MMDG_E_ARG, "mmdg_set_basis: shell_mol out of range");
    if (s > 0 && m < shell_mol[s - 1]) return fail(MMDG_E_ARG, "mmdg_set_basis: shells of a molecule must be contiguous");
    if (shell_L[s] < 0) return fail(MMDG_E_ARG, "mmdg_set_basis: negative angular momentum");
    if (shell_L[s] > MMDG_LMAX)
      return fail(MMDG_E_LMAX, "mmdg_set_basis: shell angular momentum " + std::to_string(shell_L[s]) +
                                   " above the supported maximum " + std::to_string(MMDG_LMAX));
    if (shell_nprim[s] < 1) return fail(MMDG_E_ARG, "mmdg_set_basis: shell without primitives");
    shlocal[s] = h->mol_ns[m]++;
    poff[s] = total_prim;
    total_prim += shell_nprim[s];
    const int nc = (shell_L[s] + 1) * (shell_L[s] + 2) / 2;
    for (int c = 0; c < MMDG_MAX_COMP; ++c) {
      const int f = shell_func[s * MMDG_MAX_COMP + c];
      if (c >= nc && f >= 0) return fail(MMDG_E_ARG, "mmdg_set_basis: function index on a missing component");
      if (f >= h->mol_n[m]) return fail(MMDG_E_ARG, "mmdg_set_basis: function index out of range");
    }
  }
  for (int p = 0; p < total_prim; ++p)
    if (!(prim_exp[p] > 0.0) || !std::isfinite(prim_exp[p]) || !std::isfinite(prim_coef[p]))
      return fail(MMDG_E_ARG, "mmdg_set_basis: exponents must be positive and finite");
  for (int s = 0; s < 3 * nshell; ++s)
    if (!std::isfinite(shell_center[s])) return fail(MMDG_E_ARG, "mmdg_set_basis: non-finite centre");
  h->mol_base.assign(nmol, 0);
  h->mol_sbase.assign(nmol, 0);
  h->mol_tbase.assign(nmol, 0);
  long long nn = 0, ss = 0, tt = 0;
  for (int m = 0; m < nmol; ++m) {
    h->mol_base[m] = nn;
    h->mol_sbase[m] = ss;
    h->mol_tbase[m] = tt;
    nn += (long long)h->mol_n[m] * h->mol_n[m];
    ss += (long long)h->mol_ns[m] * h->mol_ns[m];
    tt += (long long)h->mol_n[m] * (h->mol_n[m] + 1) / 2;
  }
  h->ntot_nn = nn;
  h->ntot_ss = ss;
  h->ntot_tri = tt;
  // ---- shell pairs within each molecule (a has the higher L)
  h->pa.clear();
  h->pb.clear();
  h->pcls.clear();
  h->pr_begin.clear();
  h->pr_count.clear();
  h->e_off.clear();
  long long npp = 0, ne = 0;
  h->pair_row.assign(nshell, 0);
  h->shell_L.assign(shell_L, shell_L + nshell);
  h->shell_molv.assign(shell_mol, shell_mol + nshell);
  for (int s1 = 0; s1 < nshell; ++s1) {
    h->pair_row[s1] = (int)h->pa.size();
    for (int s2 = s1; s2 >= 0 && shell_mol[s2] == shell_mol[s1]; --s2) {
      int a = s1, b = s2;
      if (shell_L[a] < shell_L[b]) std::swap(a, b);
      const int cls = pair_class(shell_L[a], shell_L[b]);
      const int np = shell_nprim[a] * shell_nprim[b];
      h->pa.push_back(a);
      h->pb.push_back(b);
      h->pcls.push_back(cls);
      h->pr_begin.push_back((int)npp);
      h->pr_count.push_back(np);
      h->e_off.push_back(ne);
      npp += np;
      ne += (long long)np * nnz_pair(shell_L[a], shell_L[b]);
    }
  }
  if (npp > 0x7fffffffLL) return fail(MMDG_E_ARG, "mmdg_set_basis: too many primitive pairs");
  h->npair = (int)h->pa.size();
  h->nprimpair = npp;
  h->nE = ne;
  // ---- upload
  std::vector<int> vL(shell_L, shell_L + nshell), vK(shell_nprim, shell_nprim + nshell);
  std::vector<int> vfunc(shell_func, shell_func + (size_t)nshell * MMDG_MAX_COMP), vmol(shell_mol, shell_mol + nshell);
  std::vector<double> vc(shell_center, shell_center + 3 * (size_t)nshell);
  std::vector<double> ve(prim_exp, prim_exp + total_prim), vco(prim_coef, prim_coef + total_prim);
  bool ok = h->d_L.upload(vL) == cudaSuccess && h->d_nprim.upload(vK) == cudaSuccess &&
            h->d_poff.upload(poff) == cudaSuccess && h->d_func.upload(vfunc) == cudaSuccess &&
            h->d_shmol.upload(vmol) == cudaSuccess && h->d_shlocal.upload(shlocal) == cudaSuccess &&
            h->d_center.upload(vc) == cudaSuccess && h->d_exp.upload(ve) == cudaSuccess &&
            h->d_coef.upload(vco) == cudaSuccess && h->d_mol_base.upload(h->mol_base) == cudaSuccess &&
            h->d_mol_sbase.upload(h->mol_sbase) == cudaSuccess && h->d_mol_tbase.upload(h->mol_tbase) == cudaSuccess &&
            h->d_mol_n.upload(h->mol_n) == cudaSuccess && h->d_mol_ns.upload(h->mol_ns) == cudaSuccess &&
            h->d_pa.upload(h->pa) == cudaSuccess && h->d_pb.upload(h->pb) == cudaSuccess &&
            h->d_prb.upload(h->pr_begin) == cudaSuccess && h->d_prc.upload(h->pr_count) == cudaSuccess &&
            h->d_eoff.upload(h->e_off) == cudaSuccess && h->d_pP.alloc(npp) == cudaSuccess &&
            h->d_pPf.alloc(2 * npp) == cudaSuccess && h->d_E64.alloc(ne) == cudaSuccess &&
            h->d_E32.alloc(ne) == cudaSuccess && h->d_Q.alloc(h->npair) == cudaSuccess &&
            h->d_screen.alloc(tt) == cudaSuccess && h->d_sq.alloc(tt) == cudaSuccess &&
            h->d_sqf.alloc(tt) == cudaSuccess && h->d_dPf.alloc(nn) == cudaSuccess &&
            h->d_Dsh.alloc(ss) == cudaSuccess && h->d_counters.alloc(kCounters * MMDG_NCLASS) == cudaSuccess;
  if (!ok) return fail(MMDG_E_NOMEM, "mmdg_set_basis: device allocation failed");
  // ---- primitive pairs
  {
    PairBuildArgs a;
    a.npair = h->npair;
    a.pa = h->d_pa.p;
    a.pb = h->d_pb.p;
    a.prb = h->d_prb.p;
    a.keep = nullptr;
    a.prc = nullptr;
    a.eoff = h->d_eoff.p;
    a.L = h->d_L.p;
    a.nprim = h->d_nprim.p;
    a.poff = h->d_poff.p;
    a.center = h->d_center.p;
    a.exps = h->d_exp.p;
    a.coefs = h->d_coef.p;
    a.pP = h->d_pP.p;
    a.pPf = h->d_pPf.p;
    a.E64 = h->d_E64.p;
    a.E32 = h->d_E32.p;
    k_build_pairs<<<(h->npair + 127) / 128, 128>>>(a);
    CUDA_TRY(cudaGetLastError());
  }
  // ---- Schwarz: diagonal quartets per pair class (unsorted lists)
  std::vector<std::vector<int>> lists(kNumPairClasses);
  for (int p = 0; p < h->npair; ++p) lists[h->pcls[p]].push_back(p);
  CUDA_TRY(cudaMemset(h->d_Q.p, 0, sizeof(float) * h->npair));
  CUDA_TRY(cudaMemset(h->d_screen.p, 0, sizeof(double) * (size_t)tt));
  Geometry g = h->geom();
  SchwarzArgs sa{h->d_screen.p, h->d_Q.p};
  {
    DevBuf<int> tmp[kNumPairClasses];
    for (int c = 0; c < kNumPairClasses; ++c) {
      if (lists[c].empty()) continue;
      if (tmp[c].upload(lists[c]) != cudaSuccess) return fail(MMDG_E_NOMEM, "mmdg_set_basis: allocation");
      const ClassEntry* ce = nullptr;
      for (const ClassEntry& e : kClasses)
        if (pair_class(e.la, e.lb) == c && pair_class(e.lc, e.ld) == c) ce = &e;
      CUDA_TRY(ce->schwarz(g, sa, tmp[c].p, (int)lists[c].size(), 0));
    }
    CUDA_TRY(cudaDeviceSynchronize());
  }
  {
    const long long n = tt;
    k_sqrt_screen<<<(unsigned)((n + 255) / 256), 256>>>(h->d_screen.p, h->d_sq.p, h->d_sqf.p, n);
    CUDA_TRY(cudaGetLastError());
  }
  // ---- primitive-pair pruning.  q_k = max over the diagonal components of
  // sqrt((a_i b_j|a_i b_j)) of one primitive pair k = (i, j), contraction weights
  // included (the Schwarz kernels run on "pairs" of one primitive each).  By
  // Cauchy-Schwarz a primitive quartet is bounded by q_k q_l <= q_k q_max, so dropping
  // the pairs with q_k q_max < prim_tol changes no contracted ERI by more than
  // (primitive quartets of the shell quartet) x prim_tol: 1.3e-15 at 1e-18 for
  // 36 x 36 primitive pairs, far below the 1e-12 screening of formPT.  The dropped
  // pairs are the tight-tight products on distant centres (Gaussian factor
  // exp(-mu |AB|^2) underflowing).  The largest pair of every shell pair is kept.
  if (h->prim_tol > 0.0 && npp > h->npair) {
    std::vector<int> xa(npp), xb(npp), xrb(npp), xrc(npp, 1);
    std::vector<long long> xeo(npp);
    std::vector<std::vector<int>> xl(kNumPairClasses);
    for (int p = 0; p < h->npair; ++p) {
      const int nz = nnz_pair(shell_L[h->pa[p]], shell_L[h->pb[p]]);
      for (int k = 0; k < h->pr_count[p]; ++k) {
        const int x = h->pr_begin[p] + k;
        xa[x] = h->pa[p];
        xb[x] = h->pb[p];
        xrb[x] = x;
        xeo[x] = h->e_off[p] + (long long)k * nz;
        xl[h->pcls[p]].push_back(x);
      }
    }
    std::vector<float> qp(npp);
    {
      DevBuf<int> dxa, dxb, dxrb, dxrc, dlist[kNumPairClasses];
      DevBuf<long long> dxeo;
      DevBuf<float> dqp;
      DevBuf<double> dscr;
      if (dxa.upload(xa) != cudaSuccess || dxb.upload(xb) != cudaSuccess || dxrb.upload(xrb) != cudaSuccess ||
          dxrc.upload(xrc) != cudaSuccess || dxeo.upload(xeo) != cudaSuccess || dqp.alloc(npp) != cudaSuccess ||
          dscr.alloc(1) != cudaSuccess)
        return fail(MMDG_E_NOMEM, "mmdg_set_basis: allocation (primitive screening)");
      CUDA_TRY(cudaMemset(dqp.p, 0, sizeof(float) * npp));
      Geometry gx = h->geom();
      gx.pa = dxa.p;
      gx.pb = dxb.p;
      gx.pr_begin = dxrb.p;
      gx.pr_count = dxrc.p;
      gx.e_off = dxeo.p;
      SchwarzArgs sx{dscr.p, dqp.p, 1};
      for (int c = 0; c < kNumPairClasses; ++c) {
        if (xl[c].empty()) continue;
        if (dlist[c].upload(xl[c]) != cudaSuccess) return fail(MMDG_E_NOMEM, "mmdg_set_basis: allocation");
        const ClassEntry* ce = nullptr;
        for (const ClassEntry& e : kClasses)
          if (pair_class(e.la, e.lb) == c && pair_class(e.lc, e.ld) == c) ce = &e;
        CUDA_TRY(ce->schwarz(gx, sx, dlist[c].p, (int)xl[c].size(), 0));
      }
      CUDA_TRY(cudaDeviceSynchronize());
      CUDA_TRY(cudaMemcpy(qp.data(), dqp.p, sizeof(float) * npp, cudaMemcpyDeviceToHost));
    }
    float qmax = 0.f;
    for (float v : qp) qmax = std::max(qmax, v);
    std::vector<int> keep;
    long long np2 = 0, ne2 = 0;
    for (int p = 0; p < h->npair; ++p) {
      const int nz = nnz_pair(shell_L[h->pa[p]], shell_L[h->pb[p]]);
      const int b0 = h->pr_begin[p], n0 = h->pr_count[p];
      int best = 0;
      for (int k = 1; k < n0; ++k)
        if (qp[b0 + k] > qp[b0 + best]) best = k;
      int kept = 0;
      for (int k = 0; k < n0; ++k)
        if (k == best || double(qp[b0 + k]) * double(qmax) >= h->prim_tol) {
          keep.push_back(k);
          ++kept;
        }
      h->pr_begin[p] = (int)np2;
      h->pr_count[p] = kept;
      h->e_off[p] = ne2;
      np2 += kept;
      ne2 += (long long)kept * nz;
    }
    if (np2 < npp) {
      h->d_pP.release();
      h->d_pPf.release();
      h->d_E64.release();
      h->d_E32.release();
      DevBuf<int> dkeep;
      if (dkeep.upload(keep) != cudaSuccess || h->d_prb.upload(h->pr_begin) != cudaSuccess ||
          h->d_prc.upload(h->pr_count) != cudaSuccess || h->d_eoff.upload(h->e_off) != cudaSuccess ||
          h->d_pP.alloc(np2) != cudaSuccess || h->d_pPf.alloc(2 * np2) != cudaSuccess ||
          h->d_E64.alloc(ne2) != cudaSuccess || h->d_E32.alloc(ne2) != cudaSuccess)
        return fail(MMDG_E_NOMEM, "mmdg_set_basis: device allocation failed (pruned pairs)");
      PairBuildArgs a;
      a.npair = h->npair;
      a.pa = h->d_pa.p;
      a.pb = h->d_pb.p;
      a.prb = h->d_prb.p;
      a.keep = dkeep.p;
      a.prc = h->d_prc.p;
      a.eoff = h->d_eoff.p;
      a.L = h->d_L.p;
      a.nprim = h->d_nprim.p;
      a.poff = h->d_poff.p;
      a.center = h->d_center.p;
      a.exps = h->d_exp.p;
      a.coefs = h->d_coef.p;
      a.pP = h->d_pP.p;
      a.pPf = h->d_pPf.p;
      a.E64 = h->d_E64.p;
      a.E32 = h->d_E32.p;
      k_build_pairs<<<(h->npair + 127) / 128, 128>>>(a);
      CUDA_TRY(cudaGetLastError());
      CUDA_TRY(cudaDeviceSynchronize());
      npp = np2;
      h->nprimpair = np2;
      h->nE = ne2;
    }
  }
  // ---- sorted class lists: molecule, primitive count ascending, Q descending
  std::vector<float> Q(h->npair);
  CUDA_TRY(cudaMemcpy(Q.data(), h->d_Q.p, sizeof(float) * h->npair, cudaMemcpyDeviceToHost));
  h->cls_count.assign(kNumPairClasses, 0);
  h->ngroup.assign(kNumPairClasses, 0);
  std::vector<std::vector<int>> slot_group(kNumPairClasses), slot_mol(kNumPairClasses);
  for (int c = 0; c < kNumPairClasses; ++c) {
    std::vector<int>& v = lists[c];
    std::stable_sort(v.begin(), v.end(), [&](int x, int y) {
      const int mx = shell_mol[h->pa[x]], my = shell_mol[h->pa[y]];
      if (mx != my) return mx < my;
      if (h->pr_count[x] != h->pr_count[y]) return h->pr_count[x] < h->pr_count[y];
      return Q[x] > Q[y];
    });
    h->cls_count[c] = (int)v.size();
    if (h->d_cls[c].upload(v) != cudaSuccess) return fail(MMDG_E_NOMEM, "mmdg_set_basis: allocation");
    // molecule offsets within the list
    std::vector<int> moff(nmol + 1, 0);
    for (int x : v) moff[shell_mol[h->pa[x]] + 1]++;
    for (int m = 0; m < nmol; ++m) moff[m + 1] += moff[m];
    if (h->d_cls_moff[c].upload(moff) != cudaSuccess) return fail(MMDG_E_NOMEM, "mmdg_set_basis: allocation");
    // primitive-count groups: contiguous ranges of the class's primitive counts (one
    // per distinct count when there are at most kMaxGroups of them)
    std::vector<int> all;
    for (int x : v) all.push_back(h->pr_count[x]);
    std::sort(all.begin(), all.end());
    std::vector<int> vals;
    std::vector<long long> freq;
    for (int x : all) {
      if (vals.empty() || vals.back() != x) {
        vals.push_back(x);
        freq.push_back(0);
      }
      ++freq.back();
    }
    const std::vector<int> grp = group_counts(vals, freq, kMaxGroups);
    std::vector<int> gs(v.size()), ms(v.size());
    for (size_t i = 0; i < v.size(); ++i) {
      gs[i] = grp[std::lower_bound(vals.begin(), vals.end(), h->pr_count[v[i]]) - vals.begin()];
      ms[i] = shell_mol[h->pa[v[i]]];
    }
    h->ngroup[c] = vals.empty() ? 0 : grp.back() + 1;
    if (h->d_gslot[c].upload(gs) != cudaSuccess) return fail(MMDG_E_NOMEM, "mmdg_set_basis: allocation");
    slot_group[c] = gs;
    slot_mol[c] = ms;
  }
  // bucket capacities per angular class: sum over molecules of the candidate counts
  {
    h->bucket_cap.assign(MMDG_NCLASS, {});
    int ci = 0;
    for (const ClassEntry& e : kClasses) {
      const int cb = pair_class(e.la, e.lb), ck = pair_class(e.lc, e.ld);
      const int Gb = h->ngroup[cb], Gk = h->ngroup[ck];
      std::vector<long long> cap((size_t)Gb * Gk, 0);
      // per molecule group sizes
      std::vector<long long> nb((size_t)nmol * (Gb ? Gb : 1), 0), nk((size_t)nmol * (Gk ? Gk : 1), 0);
      for (size_t i = 0; i < slot_group[cb].size(); ++i) nb[(size_t)slot_mol[cb][i] * Gb + slot_group[cb][i]]++;
      for (size_t i = 0; i < slot_group[ck].size(); ++i) nk[(size_t)slot_mol[ck][i] * Gk + slot_group[ck][i]]++;
      for (int m = 0; m < nmol; ++m)
        for (int gb = 0; gb < Gb; ++gb)
          for (int gk = 0; gk < Gk; ++gk) {
            const long long a = nb[(size_t)m * Gb + gb], b = nk[(size_t)m * Gk + gk];
            long long c2;
            if (cb != ck || gk < gb) c2 = a * b;
            else if (gk == gb) c2 = a * (a + 1) / 2;
            else c2 = 0;
            cap[(size_t)gb * Gk + gk] += c2;
          }
      h->bucket_cap[ci] = cap;
      ++ci;
    }
  }
  h->mol_shell0.assign(nmol, 0);
  for (int s = nshell - 1; s >= 0; --s) h->mol_shell0[shell_mol[s]] = s;
  if (h->d_mol_shell0.upload(h->mol_shell0) != cudaSuccess) return fail(MMDG_E_NOMEM, "mmdg_set_basis: allocation");
  if (h->graph) {
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  h->q_off.clear();
  h->d_q64.release();
  h->d_q32.release();
  CUDA_TRY(cudaDeviceSynchronize());
  h->have_basis = true;
  return MMDG_OK;
}

// device bytes held by a context (its buffers, the quartet lists included once a
// Fock build has allocated them)
extern "C" int mmdg_device_bytes(mmdg_context* h, long long* bytes) {
  if (!h || !bytes) return fail(MMDG_E_ARG, "mmdg_device_bytes: null argument");
  long long b = 0;
#define MMDG_ADD(buf) b += (long long)(h->buf).n * (long long)sizeof(*(h->buf).p)
  MMDG_ADD(boys64); MMDG_ADD(boys32); MMDG_ADD(boysdf);
  MMDG_ADD(d_center); MMDG_ADD(d_exp); MMDG_ADD(d_coef);
  MMDG_ADD(d_L); MMDG_ADD(d_nprim); MMDG_ADD(d_poff); MMDG_ADD(d_func); MMDG_ADD(d_shmol); MMDG_ADD(d_shlocal);
  MMDG_ADD(d_mol_base); MMDG_ADD(d_mol_sbase); MMDG_ADD(d_mol_tbase); MMDG_ADD(d_mol_n); MMDG_ADD(d_mol_ns);
  MMDG_ADD(d_pa); MMDG_ADD(d_pb); MMDG_ADD(d_prb); MMDG_ADD(d_prc); MMDG_ADD(d_eoff);
  MMDG_ADD(d_pP); MMDG_ADD(d_pPf); MMDG_ADD(d_E64); MMDG_ADD(d_E32); MMDG_ADD(d_Q);
  MMDG_ADD(d_mol_shell0); MMDG_ADD(d_screen); MMDG_ADD(d_sq); MMDG_ADD(d_sqf); MMDG_ADD(d_dPf); MMDG_ADD(d_Dsh);
  MMDG_ADD(d_counters); MMDG_ADD(d_q64); MMDG_ADD(d_q32); MMDG_ADD(d_keyoff); MMDG_ADD(d_qn); MMDG_ADD(d_work);
  MMDG_ADD(d_pair_owner); MMDG_ADD(d_pair_canon);
  for (int c = 0; c < kNumPairClasses; ++c) {
    MMDG_ADD(d_cls[c]); MMDG_ADD(d_cls_moff[c]); MMDG_ADD(d_gslot[c]);
  }
#undef MMDG_ADD
  *bytes = b;
  return MMDG_OK;
}

extern "C" int mmdg_get_screen(mmdg_context* h, double* screen, long long n) {
  if (!h || !screen) return fail(MMDG_E_ARG, "mmdg_get_screen: null argument");
  if (!h->have_basis) return fail(MMDG_E_STATE, "mmdg_get_screen: no basis set");
  if (n != h->ntot_tri) return fail(MMDG_E_ARG, "mmdg_get_screen: length must be sum N(N+1)/2");
  DeviceGuard dg(h->device);
  CUDA_TRY(cudaMemcpy(screen, h->d_screen.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
  return MMDG_OK;
}

// ------------------------------------------------------------------ ERI tensor
extern "C" int mmdg_eri_tensor(mmdg_context* h, double* out, void* stream) {
  if (!h || !out) return fail(MMDG_E_ARG, "mmdg_eri_tensor: null argument");
  if (!h->have_basis) return fail(MMDG_E_STATE, "mmdg_eri_tensor: no basis set");
  if (h->nmol != 1) return fail(MMDG_E_STATE, "mmdg_eri_tensor: defined for a single molecule");
  DeviceGuard dg(h->device);
  cudaStream_t st = (cudaStream_t)stream;
  const long long N = h->mol_n[0];
  CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(double) * N * N * N * N, st));
  Geometry g = h->geom();
  TensorArgs t{out};
  for (const ClassEntry& e : kClasses) {
    const int cb = pair_class(e.la, e.lb), ck = pair_class(e.lc, e.ld);
    if (!h->cls_count[cb] || !h->cls_count[ck]) continue;
    ClassLaunch cl{h->d_cls[cb].p, h->d_cls[ck].p, h->cls_count[cb], h->cls_count[ck], cb == ck, 0.f, 0.f};
    CUDA_TRY(e.tensor(g, t, cl, st));
  }
  return MMDG_OK;
}

// ------------------------------------------------------------------ listed shell quartets
// The caller's quartets (a b|c d) (global shell indices, the four of one molecule)
// are put in the class table's canonical form -- each pair with its higher-L shell
// first, the pair of higher class as the bra -- grouped by angular class and
// evaluated by one thread each; the digest writes every component back in the
// caller's order.
extern "C" int mmdg_eri_quartets(mmdg_context* h, long long n, const int* shells, double* out, int precision,
                                 void* stream) {
  if (!h || (n > 0 && (!shells || !out))) return fail(MMDG_E_ARG, "mmdg_eri_quartets: null argument");
  if (precision != 0 && precision != 1) return fail(MMDG_E_ARG, "mmdg_eri_quartets: precision must be 0 or 1");
  if (!h->have_basis) return fail(MMDG_E_STATE, "mmdg_eri_quartets: no basis set");
  if (n < 0 || n > 0x7fffffffLL / kQuartetBlock) return fail(MMDG_E_ARG, "mmdg_eri_quartets: bad quartet count");
  if (n == 0) return MMDG_OK;
  DeviceGuard dgd(h->device);
  cudaStream_t st = (cudaStream_t)stream;
  std::vector<std::vector<QuartetItem>> per(MMDG_NCLASS);
  int class_index[kNumPairClasses][kNumPairClasses];
  for (int x = 0; x < kNumPairClasses; ++x)
    for (int y = 0; y < kNumPairClasses; ++y) class_index[x][y] = -1;
  {
    int ci = 0;
    for (const ClassEntry& e : kClasses) class_index[pair_class(e.la, e.lb)][pair_class(e.lc, e.ld)] = ci++;
  }
  // canonical pair of shells (x, y): its index and whether y is the stored first shell
  auto pair_of = [&](int x, int y, int* flip) {
    const int s1 = std::max(x, y), s2 = std::min(x, y);
    const int p = h->pair_row[s1] + (s1 - s2);
    *flip = (h->pa[p] != x) ? 1 : 0;
    return p;
  };
  for (long long q = 0; q < n; ++q) {
    const int* sq = shells + 4 * q;
    for (int k = 0; k < 4; ++k)
      if (sq[k] < 0 || sq[k] >= h->nshell) return fail(MMDG_E_ARG, "mmdg_eri_quartets: shell index out of range");
    const int m = h->shell_molv[sq[0]];
    if (h->shell_molv[sq[1]] != m || h->shell_molv[sq[2]] != m || h->shell_molv[sq[3]] != m)
      return fail(MMDG_E_ARG, "mmdg_eri_quartets: the four shells of a quartet must belong to one molecule");
    int f1 = 0, f2 = 0;
    const int p1 = pair_of(sq[0], sq[1], &f1), p2 = pair_of(sq[2], sq[3], &f2);
    const int c1 = h->pcls[p1], c2 = h->pcls[p2];
    QuartetItem it;
    it.slot = (int)q;
    if (c1 >= c2) {
      it.bra = p1;
      it.ket = p2;
      it.flags = (f1 ? 2 : 0) | (f2 ? 4 : 0);
    } else {
      it.bra = p2;
      it.ket = p1;
      it.flags = 1 | (f1 ? 2 : 0) | (f2 ? 4 : 0);
    }
    per[class_index[h->pcls[it.bra]][h->pcls[it.ket]]].push_back(it);
  }
  std::vector<QuartetItem> all;
  std::vector<size_t> beg(MMDG_NCLASS + 1, 0);
  for (int c = 0; c < MMDG_NCLASS; ++c) {
    beg[c] = all.size();
    all.insert(all.end(), per[c].begin(), per[c].end());
  }
  beg[MMDG_NCLASS] = all.size();
  DevBuf<QuartetItem> d_items;
  if (d_items.alloc(all.size()) != cudaSuccess) return fail(MMDG_E_NOMEM, "mmdg_eri_quartets: allocation");
  CUDA_TRY(cudaMemcpyAsync(d_items.p, all.data(), sizeof(QuartetItem) * all.size(), cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(double) * (size_t)n * kQuartetBlock, st));
  Geometry g = h->geom();
  QuartetArgs qa{out};
  int ci = 0;
  for (const ClassEntry& e : kClasses) {
    const int cnt = (int)(beg[ci + 1] - beg[ci]);
    if (cnt) CUDA_TRY(e.quartets(precision, g, qa, d_items.p + beg[ci], cnt, st));
    ++ci;
  }
  CUDA_TRY(cudaStreamSynchronize(st));  // the item list is released on return
  return MMDG_OK;
}

// ------------------------------------------------------------------ Fock build
__global__ void k_prep_density(const double* dP, float* dPf, long long n) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  dPf[i] = float(fabs(dP[i]));
}

// per-molecule S x S block maxima of |dP|: one thread per (molecule, shell, shell)
__global__ void k_shell_dmax(const float* dPf, float* Dsh, const int* func, const int* L,
                             const long long* mol_base, const int* mol_n, const long long* mol_sbase,
                             const int* mol_ns, const long long* mol_shell0, int nmol, long long total) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= total) return;
  int lo = 0, hi = nmol - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    if (mol_sbase[mid] <= idx) lo = mid;
    else hi = mid - 1;
  }
  const int m = lo;
  const int S = mol_ns[m], N = mol_n[m];
  const long long loc = idx - mol_sbase[m];
  const int a = (int)(loc / S), b = (int)(loc % S);
  const int s1 = (int)(mol_shell0[m] + a), s2 = (int)(mol_shell0[m] + b);
  const float* D = dPf + mol_base[m];
  const int n1 = (L[s1] + 1) * (L[s1] + 2) / 2, n2 = (L[s2] + 1) * (L[s2] + 2) / 2;
  float mx = 0.f;
  for (int x = 0; x < n1; ++x) {
    const int i = func[s1 * kMaxComp + x];
    if (i < 0) continue;
    for (int y = 0; y < n2; ++y) {
      const int j = func[s2 * kMaxComp + y];
      if (j < 0) continue;
      mx = fmaxf(mx, D[(long long)i * N + j]);
    }
  }
  Dsh[idx] = mx;
}

static int fock_impl(mmdg_context* h, const double* dP, double* G, double tol, double fp32_below,
                     unsigned long long* counts, float* class_ms, void* stream);

extern "C" int mmdg_fock(mmdg_context* h, const double* dP, double* G, double tol, double fp32_below,
                         unsigned long long* counts, void* stream) {
  return fock_impl(h, dP, G, tol, fp32_below, counts, nullptr, stream);
}

extern "C" int mmdg_fock_timed(mmdg_context* h, const double* dP, double* G, double tol, double fp32_below,
                               unsigned long long* counts, float* class_ms, void* stream) {
  if (!class_ms) return fail(MMDG_E_ARG, "mmdg_fock_timed: null class_ms");
  return fock_impl(h, dP, G, tol, fp32_below, counts, class_ms, stream);
}

static int fock_impl(mmdg_context* h, const double* dP, double* G, double tol, double fp32_below,
                     unsigned long long* counts, float* class_ms, void* stream) {
  if (!h || !dP || !G) return fail(MMDG_E_ARG, "mmdg_fock: null argument");
  if (!h->have_basis) return fail(MMDG_E_STATE, "mmdg_fock: no basis set");
  if (!(tol >= 0.0) || !(fp32_below >= 0.0)) return fail(MMDG_E_ARG, "mmdg_fock: negative threshold");
  DeviceGuard dgd(h->device);
  cudaStream_t st = (cudaStream_t)stream;
  const long long nn = h->ntot_nn;
  CUDA_TRY(cudaMemsetAsync(G, 0, sizeof(double) * nn, st));
  CUDA_TRY(cudaMemsetAsync(h->d_counters.p, 0, sizeof(unsigned long long) * kCounters * MMDG_NCLASS, st));
  k_prep_density<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(dP, h->d_dPf.p, nn);
  CUDA_TRY(cudaGetLastError());
  {
    const long long n = h->ntot_ss;
    k_shell_dmax<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(h->d_dPf.p, h->d_Dsh.p, h->d_func.p, h->d_L.p,
                                                              h->d_mol_base.p, h->d_mol_n.p, h->d_mol_sbase.p,
                                                              h->d_mol_ns.p, h->d_mol_shell0.p, h->nmol, n);
    CUDA_TRY(cudaGetLastError());
  }
  Geometry g = h->geom();
  FockArgs f;
  f.dP = dP;
  f.dPf = h->d_dPf.p;
  f.G = G;
  f.sq = h->d_sq.p;
  f.sqf = h->d_sqf.p;
  f.Dsh = h->d_Dsh.p;
  f.tol = tol;
  f.tolf_lo = float(tol * (1.0 - 1e-4));
  f.tolf_hi = float(tol * (1.0 + 1e-4));
  f.counters = nullptr;
  f.work = nullptr;  // set per launch below
  f.pair_owner = h->nparts > 1 ? h->d_pair_owner.p : nullptr;
  f.pair_canon = h->d_pair_canon.p;
  f.part = h->part;
  const float split = float(fp32_below);
  // ---- quartet-list storage (first use): per class, buckets (bra group, ket group)
  if (h->q_off.empty()) {
    h->q_off.assign(MMDG_NCLASS, 0);
    h->q_cap.assign(MMDG_NCLASS, 0);
    h->kbase.assign(MMDG_NCLASS, 0);
    h->nkeys.assign(MMDG_NCLASS, 0);
    std::vector<long long> koff;
    long long tot = 0;
    int nk = 0;
    for (int ci = 0; ci < MMDG_NCLASS; ++ci) {
      const std::vector<long long>& cap = h->bucket_cap[ci];
      if ((int)cap.size() > kMaxKeys) return fail(MMDG_E_ARG, "mmdg_fock: too many primitive-count groups in one class");
      h->q_off[ci] = tot;
      h->kbase[ci] = nk;
      h->nkeys[ci] = (int)cap.size();
      long long rel = 0;
      for (long long c2 : cap) {
        koff.push_back(rel);
        rel += c2;
      }
      h->q_cap[ci] = rel;
      tot += rel;
      nk += (int)cap.size();
    }
    h->q_total = tot;
    h->total_keys = nk;
    if (h->d_q64.alloc(tot > 0 ? tot : 1) != cudaSuccess || h->d_qn.alloc(2 * (nk > 0 ? nk : 1)) != cudaSuccess ||
        h->d_work.alloc(2 * MMDG_NCLASS) != cudaSuccess ||
        h->d_keyoff.upload(koff.empty() ? std::vector<long long>{0} : koff) != cudaSuccess) {
      h->q_off.clear();
      return fail(MMDG_E_NOMEM, "mmdg_fock: cannot allocate the quartet lists");
    }
  }
  if (split > 0.f && !h->d_q32.p) {
    if (h->d_q32.alloc(h->q_total > 0 ? h->q_total : 1) != cudaSuccess)
      return fail(MMDG_E_NOMEM, "mmdg_fock: cannot allocate the FP32 quartet lists");
  }
  CUDA_TRY(cudaMemsetAsync(h->d_qn.p, 0, sizeof(unsigned) * 2 * (h->total_keys > 0 ? h->total_keys : 1), st));
  CUDA_TRY(cudaMemsetAsync(h->d_work.p, 0, sizeof(unsigned long long) * 2 * MMDG_NCLASS, st));
  cudaEvent_t ev[2 * MMDG_NCLASS];
  if (class_ms)
    for (int k = 0; k < 2 * MMDG_NCLASS; ++k) CUDA_TRY(cudaEventCreate(&ev[k]));
  // ---- screening and evaluation of every class; with several streams class c runs
  // both on stream c mod n (fork / join on events), so classes overlap
  const int ns = class_ms ? 1 : h->nstreams;
  if (ns > 1) {
    CUDA_TRY(cudaEventRecord(h->fork_ev, st));
    for (int k = 0; k < ns; ++k) CUDA_TRY(cudaStreamWaitEvent(h->side[k], h->fork_ev, 0));
  }
  int ci = 0;
  for (const ClassEntry& e : kClasses) {
    const int cb = pair_class(e.la, e.lb), ck = pair_class(e.lc, e.ld);
    if (h->cls_count[cb] && h->cls_count[ck]) {
      ClassLaunch cl{h->d_cls[cb].p, h->d_cls[ck].p, h->cls_count[cb], h->cls_count[ck], cb == ck, 0.f, split,
                     h->d_cls_moff[ck].p};
      QuartetLists ql{h->d_q64.p + h->q_off[ci],
                      split > 0.f ? h->d_q32.p + h->q_off[ci] : nullptr,
                      h->d_qn.p + h->kbase[ci],
                      h->d_qn.p + h->total_keys + h->kbase[ci],
                      h->d_keyoff.p + h->kbase[ci],
                      h->d_gslot[cb].p,
                      h->d_gslot[ck].p,
                      h->ngroup[ck],
                      h->nkeys[ci]};
      k_screen<<<cl.nbra, kThreads, 0, ns > 1 ? h->side[ci % ns] : st>>>(g, f, cl, ql);
      CUDA_TRY(cudaGetLastError());
    }
    ++ci;
  }
  ci = 0;
  for (const ClassEntry& e : kClasses) {
    const int cb = pair_class(e.la, e.lb), ck = pair_class(e.lc, e.ld);
    f.counters = h->d_counters.p + kCounters * ci;
    cudaStream_t cs = ns > 1 ? h->side[ci % ns] : st;
    if (class_ms) CUDA_TRY(cudaEventRecord(ev[2 * ci], st));
    if (h->cls_count[cb] && h->cls_count[ck]) {
      ClassLaunch cl{h->d_cls[cb].p, h->d_cls[ck].p, h->cls_count[cb], h->cls_count[ck], cb == ck, 0.f, split,
                     h->d_cls_moff[ck].p};
      const long long* ko = h->d_keyoff.p + h->kbase[ci];
      const int grid = h->class_grid[ci], blk = h->class_block[ci], item = h->class_item[ci];
      f.work = h->d_work.p + 2 * ci;
      CUDA_TRY(e.fock(0, g, f, cl, h->d_q64.p + h->q_off[ci], h->d_qn.p + h->kbase[ci], ko, h->nkeys[ci], grid, blk,
                      item, cs));
      if (split > 0.f) {
        f.work = h->d_work.p + 2 * ci + 1;
        CUDA_TRY(e.fock(1, g, f, cl, h->d_q32.p + h->q_off[ci], h->d_qn.p + h->total_keys + h->kbase[ci], ko,
                        h->nkeys[ci], grid, blk, item, cs));
      }
    }
    if (class_ms) CUDA_TRY(cudaEventRecord(ev[2 * ci + 1], st));
    ++ci;
  }
  if (ns > 1)
    for (int k = 0; k < ns; ++k) {
      CUDA_TRY(cudaEventRecord(h->join_ev[k], h->side[k]));
      CUDA_TRY(cudaStreamWaitEvent(st, h->join_ev[k], 0));
    }
  if (class_ms) {
    CUDA_TRY(cudaEventSynchronize(ev[2 * MMDG_NCLASS - 1]));
    for (int k = 0; k < MMDG_NCLASS; ++k) CUDA_TRY(cudaEventElapsedTime(&class_ms[k], ev[2 * k], ev[2 * k + 1]));
    for (int k = 0; k < 2 * MMDG_NCLASS; ++k) cudaEventDestroy(ev[k]);
  }
  if (counts) {
    CUDA_TRY(cudaMemcpyAsync(counts, h->d_counters.p, sizeof(unsigned long long) * kCounters * MMDG_NCLASS,
                             cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
  }
  return MMDG_OK;
}

// ------------------------------------------------------------------ F update, Boys
__global__ void k_fock_update(const double* G, const double* Fin, double* Fout, const long long* mol_base,
                              const int* mol_n, int nmol, long long nn) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= nn) return;
  // locate the molecule block (few molecules: linear; many: binary search)
  int lo = 0, hi = nmol - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) / 2;
    if (mol_base[mid] <= idx) lo = mid;
    else hi = mid - 1;
  }
  const long long b = mol_base[lo];
  const long long N = mol_n[lo];
  const long long loc = idx - b, i = loc / N, j = loc % N;
  Fout[idx] = Fin[idx] + 0.5 * (G[idx] + G[b + j * N + i]);
}

extern "C" int mmdg_fock_update(mmdg_context* h, const double* G, const double* F_in, double* F_out, void* stream) {
  if (!h || !G || !F_in || !F_out) return fail(MMDG_E_ARG, "mmdg_fock_update: null argument");
  if (!h->have_basis) return fail(MMDG_E_STATE, "mmdg_fock_update: no basis set");
  if (G == F_out) return fail(MMDG_E_ARG, "mmdg_fock_update: G must not alias F_out");
  DeviceGuard dg(h->device);
  const long long nn = h->ntot_nn;
  k_fock_update<<<(unsigned)((nn + 255) / 256), 256, 0, (cudaStream_t)stream>>>(G, F_in, F_out, h->d_mol_base.p,
                                                                               h->d_mol_n.p, h->nmol, nn);
  CUDA_TRY(cudaGetLastError());
  return MMDG_OK;
}

template <int L>
__global__ void k_boys(const double* tab, const double* T, double* out, long long n) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double F[L + 1];
  boys_eval<L>(tab, T[i], F);
  out[i] = F[L];
}

extern "C" int mmdg_boys(mmdg_context* h, int m, long long n, const double* T, double* out, void* stream) {
  if (!h || (!T && n) || (!out && n)) return fail(MMDG_E_ARG, "mmdg_boys: null argument");
  if (m < 0 || m > 8) return fail(MMDG_E_ARG, "mmdg_boys: order must be 0..8");
  if (n <= 0) return MMDG_OK;
  DeviceGuard dg(h->device);
  cudaStream_t st = (cudaStream_t)stream;
  const unsigned nb = (unsigned)((n + 255) / 256);
  switch (m) {
    case 0: k_boys<0><<<nb, 256, 0, st>>>(h->boys64.p, T, out, n); break;
    case 1: k_boys<1><<<nb, 256, 0, st>>>(h->boys64.p, T, out, n); break;
    case 2: k_boys<2><<<nb, 256, 0, st>>>(h->boys64.p, T, out, n); break;
    case 3: k_boys<3><<<nb, 256, 0, st>>>(h->boys64.p, T, out, n); break;
    case 4: k_boys<4><<<nb, 256, 0, st>>>(h->boys64.p, T, out, n); break;
    case 5: k_boys<5><<<nb, 256, 0, st>>>(h->boys64.p, T, out, n); break;
    case 6: k_boys<6><<<nb, 256, 0, st>>>(h->boys64.p, T, out, n); break;
    case 7: k_boys<7><<<nb, 256, 0, st>>>(h->boys64.p, T, out, n); break;
    default: k_boys<8><<<nb, 256, 0, st>>>(h->boys64.p, T, out, n); break;
  }
  CUDA_TRY(cudaGetLastError());
  return MMDG_OK;
}

// 1/sqrt(x) of the ERI kernels (rsqrt_dd: FP32 estimate + one third-order FP64 step)
// and CUDA's rsqrt side by side, for the accuracy test
__global__ void k_rsqrt(const double* x, double* ours, double* cuda, long long n) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  ours[i] = rsqrt_dd(x[i]);
  cuda[i] = rsqrt(x[i]);
}

extern "C" int mmdg_rsqrt(mmdg_context* h, long long n, const double* x, double* ours, double* cuda, void* stream) {
  if (!h || (n > 0 && (!x || !ours || !cuda))) return fail(MMDG_E_ARG, "mmdg_rsqrt: null argument");
  if (n <= 0) return MMDG_OK;
  DeviceGuard dg(h->device);
  k_rsqrt<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(x, ours, cuda, n);
  CUDA_TRY(cudaGetLastError());
  return MMDG_OK;
}

// ------------------------------------------------------------------ set screen, dense J/K
__global__ void k_pair_q_from_screen(const double* screen, float* Q, const int* pa, const int* pb, const int* L,
                                     const int* func, const int* sh_mol, const long long* mol_tbase, int npair) {
  const int pr = blockIdx.x * blockDim.x + threadIdx.x;
  if (pr >= npair) return;
  const int a = pa[pr], b = pb[pr];
  const long long tb = mol_tbase[sh_mol[a]];
  const int na = (L[a] + 1) * (L[a] + 2) / 2, nb = (L[b] + 1) * (L[b] + 2) / 2;
  float q = 0.f;
  for (int x = 0; x < na; ++x) {
    const int i = func[a * kMaxComp + x];
    if (i < 0) continue;
    for (int y = 0; y < nb; ++y) {
      int j = func[b * kMaxComp + y];
      if (j < 0) continue;
      int ii = i > j ? i : j, jj = i > j ? j : i;
      q = fmaxf(q, sqrtf(fmaxf(float(screen[tb + (long long)ii * (ii + 1) / 2 + jj]), 0.f)));
    }
  }
  // round up so that the shell bound stays an upper bound of the function bounds
  Q[pr] = q * (1.0f + 1e-6f);
}

extern "C" int mmdg_set_screen(mmdg_context* h, const double* screen, long long n) {
  if (!h || !screen) return fail(MMDG_E_ARG, "mmdg_set_screen: null argument");
  if (!h->have_basis) return fail(MMDG_E_STATE, "mmdg_set_screen: no basis set");
  if (n != h->ntot_tri) return fail(MMDG_E_ARG, "mmdg_set_screen: length must be sum N(N+1)/2");
  DeviceGuard dg(h->device);
  CUDA_TRY(cudaMemcpy(h->d_screen.p, screen, sizeof(double) * n, cudaMemcpyHostToDevice));
  k_sqrt_screen<<<(unsigned)((n + 255) / 256), 256>>>(h->d_screen.p, h->d_sq.p, h->d_sqf.p, n);
  CUDA_TRY(cudaGetLastError());
  k_pair_q_from_screen<<<(h->npair + 127) / 128, 128>>>(h->d_screen.p, h->d_Q.p, h->d_pa.p, h->d_pb.p, h->d_L.p,
                                                        h->d_func.p, h->d_shmol.p, h->d_mol_tbase.p, h->npair);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaDeviceSynchronize());
  return MMDG_OK;
}

// J_pq = sum_rs (pq|rs) P_sr,  K_pq = sum_rs (ps|qr) P_sr   (mmd/scf.py:97-98)
// one warp per (p,q); lanes stride over r,s
__global__ void k_jk_dense(const double* T, const double* P, double* J, double* K, long long N) {
  const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= N * N) return;
  const long long p = w / N, q = w % N;
  double j = 0.0, k = 0.0;
  for (long long x = lane; x < N * N; x += 32) {
    const long long r = x / N, s = x % N;
    const double psr = P[s * N + r];
    j = fma(T[((p * N + q) * N + r) * N + s], psr, j);
    k = fma(T[((p * N + s) * N + q) * N + r], psr, k);
  }
  for (int o = 16; o > 0; o >>= 1) {
    j += __shfl_xor_sync(0xffffffffu, j, o);
    k += __shfl_xor_sync(0xffffffffu, k, o);
  }
  if (lane == 0) {
    J[p * N + q] = j;
    K[p * N + q] = k;
  }
}

extern "C" int mmdg_jk_dense(mmdg_context* h, long long N, const double* T, const double* P, double* J, double* K,
                             void* stream) {
  if (!h || !T || !P || !J || !K || N <= 0) return fail(MMDG_E_ARG, "mmdg_jk_dense: bad argument");
  DeviceGuard dg(h->device);
  const long long warps = N * N;
  k_jk_dense<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, (cudaStream_t)stream>>>(T, P, J, K, N);
  CUDA_TRY(cudaGetLastError());
  return MMDG_OK;
}

// ------------------------------------------------------------------ one-electron integrals
// S, T, V and the dipole integrals (cython/onee.pyx:14-192): one thread per shell
// pair, generic loops (work O(pairs x primitives x atoms), negligible next to the
// two-electron part).  Same formulas as the reference: overlap E_0 products
// (onee.pyx:71-78), kinetic energy through E with l2+-2 (onee.pyx:103-133), dipole
// E_1 + X_PC E_0 (onee.pyx:81-101), nuclear attraction 2 pi / p sum E E E R
// (onee.pyx:175-192).
struct OneEArgs {
  int npair;
  const int *pa, *pb, *L, *nprim, *poff, *func, *sh_mol;
  const double *center, *exps, *coefs;
  const long long* mol_base;
  const int* mol_n;
  const int *atom_begin, *atom_end;   // per molecule
  const double* atom_xyz;             // [natom*3]
  const double* atom_Z;
  const double* origin;               // [nmol*3] dipole gauge origin (centre of nuclear charge)
  long long nn;                       // total packed size
  const double* boys;
  double *S, *T, *V, *M;              // M: 3 blocks of nn
};

// R^0_tuv (t+u+v <= L, L <= 4) of the nuclear attraction, R[(t*(L+1)+u)*(L+1)+v], from
// R^(n)_000 = (-2p)^n F_n(p |PC|^2), by the recursion of cython/util.pxi:33-50 level by
// level (compile-time bounds: the tables live in registers)
template <int L>
__device__ __forceinline__ void hermite_r_table(const double* boys, double p, double X, double Y, double Z,
                                                double* R) {
  constexpr int D = L + 1;
  double F[L + 1];
  boys_eval<L>(boys, p * (X * X + Y * Y + Z * Z), F);
  double R0[L + 1];
  double c = 1.0;
#pragma unroll
  for (int n = 0; n <= L; ++n) {
    R0[n] = c * F[n];
    c *= -2.0 * p;
  }
  double cur[D * D * D];
  cur[0] = R0[L];
#pragma unroll
  for (int n = L - 1; n >= 0; --n) {
    const int s = L - n;
    double nxt[D * D * D];
#pragma unroll
    for (int t = 0; t <= s; ++t)
#pragma unroll
      for (int u = 0; u <= s - t; ++u)
#pragma unroll
        for (int v = 0; v <= s - t - u; ++v) {
          double val;
          if (t + u + v == 0) val = R0[n];
          else if (t > 0) val = X * cur[((t - 1) * D + u) * D + v] + (t > 1 ? (t - 1) * cur[((t - 2) * D + u) * D + v] : 0.0);
          else if (u > 0) val = Y * cur[(u - 1) * D + v] + (u > 1 ? (u - 1) * cur[(u - 2) * D + v] : 0.0);
          else val = Z * cur[v - 1] + (v > 1 ? (v - 1) * cur[v - 2] : 0.0);
          nxt[(t * D + u) * D + v] = val;
        }
#pragma unroll
    for (int t = 0; t <= s; ++t)
#pragma unroll
      for (int u = 0; u <= s - t; ++u)
#pragma unroll
        for (int v = 0; v <= s - t - u; ++v) cur[(t * D + u) * D + v] = nxt[(t * D + u) * D + v];
  }
#pragma unroll
  for (int x = 0; x < D * D * D; ++x) R[x] = cur[x];
}

// One-electron integrals of the shell pairs of one pair class (la, lb) = (LA, LB),
// cython/onee.pyx:14-192 as assembled by mmd/molecule.py:235-276.  Grid: x = pair of
// the class list, y = nucleus of the pair's molecule (one thread per (pair, nucleus),
// so the nuclear-attraction sums run in parallel); the y = 0 thread also writes S, T
// and the dipole integrals; V is accumulated with atomics.  Angular momenta are
// template parameters, so every loop bound is a constant and the tables sit in
// registers (a runtime-L version kept them in local memory: 13 ms for (H2O)16
// 6-31G**).
template <int LA, int LB>
__global__ void __launch_bounds__(64) k_one_electron(OneEArgs a, const int* __restrict__ plist, int npair) {
  constexpr int NA = (LA + 1) * (LA + 2) / 2, NB = (LB + 1) * (LB + 2) / 2, L = LA + LB;
  constexpr int NJ = LB + 3, NT = LA + LB + 3, D = L + 1;
  const int x0 = blockIdx.x * blockDim.x + threadIdx.x;
  if (x0 >= npair) return;
  const int pr = plist[x0];
  const int sa = a.pa[pr], sb = a.pb[pr];
  const int m = a.sh_mol[sa];
  const int atom = a.atom_begin[m] + (int)blockIdx.y;
  if (atom >= a.atom_end[m]) return;
  const bool first = blockIdx.y == 0;
  const long long base = a.mol_base[m];
  const int N = a.mol_n[m];
  const double A[3] = {a.center[3 * sa], a.center[3 * sa + 1], a.center[3 * sa + 2]};
  const double B[3] = {a.center[3 * sb], a.center[3 * sb + 1], a.center[3 * sb + 2]};
  const double AB2 = (A[0] - B[0]) * (A[0] - B[0]) + (A[1] - B[1]) * (A[1] - B[1]) + (A[2] - B[2]) * (A[2] - B[2]);
  const double* O = a.origin + 3 * m;
  const double C[3] = {a.atom_xyz[3 * atom], a.atom_xyz[3 * atom + 1], a.atom_xyz[3 * atom + 2]};
  double accS[NA * NB], accT[NA * NB], accV[NA * NB], accM[3][NA * NB];
#pragma unroll
  for (int x = 0; x < NA * NB; ++x) {
    accS[x] = accT[x] = accV[x] = 0.0;
    accM[0][x] = accM[1][x] = accM[2][x] = 0.0;
  }
  const double PI = 3.141592653589793238462643383279;
  const int ka_n = a.nprim[sa], kb_n = a.nprim[sb], oa = a.poff[sa], ob = a.poff[sb];
  for (int ka = 0; ka < ka_n; ++ka)
    for (int kb = 0; kb < kb_n; ++kb) {
      const double ea = a.exps[oa + ka], eb = a.exps[ob + kb];
      const double p = ea + eb, ip = 1.0 / p, mu = ea * eb * ip;
      const double P[3] = {(ea * A[0] + eb * B[0]) * ip, (ea * A[1] + eb * B[1]) * ip, (ea * A[2] + eb * B[2]) * ip};
      const double cK = a.coefs[oa + ka] * a.coefs[ob + kb] * exp(-mu * AB2);
      // 1D E[d][i][j][t], i <= LA, j <= LB + 2 (kinetic), t <= i + j (cython/util.pxi:13-28)
      double E[3][LA + 1][NJ][NT];
      const double i2p = 0.5 * ip;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const double XPA = P[d] - A[d], XPB = P[d] - B[d];
#pragma unroll
        for (int i = 0; i <= LA; ++i)
#pragma unroll
          for (int j = 0; j < NJ; ++j)
#pragma unroll
            for (int t = 0; t < NT; ++t) E[d][i][j][t] = 0.0;
        E[d][0][0][0] = 1.0;
#pragma unroll
        for (int i = 0; i < LA; ++i)
#pragma unroll
          for (int t = 0; t <= i + 1; ++t) {
            double v = XPA * E[d][i][0][t];
            if (t > 0) v += i2p * E[d][i][0][t - 1];
            if (t + 1 <= i) v += (t + 1) * E[d][i][0][t + 1];
            E[d][i + 1][0][t] = v;
          }
#pragma unroll
        for (int j = 0; j < NJ - 1; ++j)
#pragma unroll
          for (int i = 0; i <= LA; ++i)
#pragma unroll
            for (int t = 0; t <= i + j + 1; ++t) {
              double v = XPB * E[d][i][j][t];
              if (t > 0) v += i2p * E[d][i][j][t - 1];
              if (t + 1 <= i + j) v += (t + 1) * E[d][i][j][t + 1];
              E[d][i][j + 1][t] = v;
            }
      }
      const double s3 = pow(PI * ip, 1.5) * cK;
      if (first) {  // overlap, kinetic, dipole
        int x = 0;
#pragma unroll
        for (int xa = LA; xa >= 0; --xa)
#pragma unroll
          for (int ya = LA - xa; ya >= 0; --ya) {
            const int za = LA - xa - ya;
#pragma unroll
            for (int xb = LB; xb >= 0; --xb)
#pragma unroll
              for (int yb = LB - xb; yb >= 0; --yb, ++x) {
                const int zb = LB - xb - yb;
                const double nab = comp_norm(xa) * comp_norm(ya) * comp_norm(za) * comp_norm(xb) * comp_norm(yb) *
                                   comp_norm(zb);
                const double Sx = E[0][xa][xb][0], Sy = E[1][ya][yb][0], Sz = E[2][za][zb][0];
                accS[x] += nab * s3 * Sx * Sy * Sz;
                const int lbv[3] = {xb, yb, zb};
                const int lav[3] = {xa, ya, za};
                double Td[3];
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                  const int l2 = lbv[d], l1 = lav[d];
                  double t = (2 * l2 + 1) * eb * E[d][l1][l2][0] - 2.0 * eb * eb * E[d][l1][l2 + 2][0];
                  if (l2 >= 2) t += -0.5 * l2 * (l2 - 1) * E[d][l1][l2 - 2][0];
                  Td[d] = t;
                }
                accT[x] += nab * s3 * (Td[0] * Sy * Sz + Td[1] * Sx * Sz + Td[2] * Sx * Sy);
                const double Dx = E[0][xa][xb][1] + (P[0] - O[0]) * Sx;
                const double Dy = E[1][ya][yb][1] + (P[1] - O[1]) * Sy;
                const double Dz = E[2][za][zb][1] + (P[2] - O[2]) * Sz;
                accM[0][x] += nab * s3 * Dx * Sy * Sz;
                accM[1][x] += nab * s3 * Sx * Dy * Sz;
                accM[2][x] += nab * s3 * Sx * Sy * Dz;
              }
          }
      }
      // nuclear attraction of this thread's nucleus
      double R[D * D * D];
      hermite_r_table<L>(a.boys, p, P[0] - C[0], P[1] - C[1], P[2] - C[2], R);
      const double pre = -a.atom_Z[atom] * 2.0 * PI * ip * cK;
      int y = 0;
#pragma unroll
      for (int xa = LA; xa >= 0; --xa)
#pragma unroll
        for (int ya = LA - xa; ya >= 0; --ya) {
          const int za = LA - xa - ya;
#pragma unroll
          for (int xb = LB; xb >= 0; --xb)
#pragma unroll
            for (int yb = LB - xb; yb >= 0; --yb, ++y) {
              const int zb = LB - xb - yb;
              const double nab = comp_norm(xa) * comp_norm(ya) * comp_norm(za) * comp_norm(xb) * comp_norm(yb) *
                                 comp_norm(zb);
              double v = 0.0;
#pragma unroll
              for (int t = 0; t <= xa + xb; ++t)
#pragma unroll
                for (int u = 0; u <= ya + yb; ++u)
#pragma unroll
                  for (int w = 0; w <= za + zb; ++w)
                    v += E[0][xa][xb][t] * E[1][ya][yb][u] * E[2][za][zb][w] * R[(t * D + u) * D + w];
              accV[y] += pre * nab * v;
            }
        }
    }
  // scatter (each function pair belongs to exactly one shell pair); V adds this
  // nucleus's share to the zeroed matrix
  int x = 0;
#pragma unroll
  for (int ca = 0; ca < NA; ++ca)
#pragma unroll
    for (int cb = 0; cb < NB; ++cb, ++x) {
      const int i = a.func[sa * kMaxComp + ca], j = a.func[sb * kMaxComp + cb];
      if (i < 0 || j < 0) continue;
      if (sa == sb && cb > ca) continue;  // (ca, cb) already wrote both V[i][j] and V[j][i]
      const long long ij = base + (long long)i * N + j, ji = base + (long long)j * N + i;
      atomicAdd(a.V + ij, accV[x]);
      if (ji != ij) atomicAdd(a.V + ji, accV[x]);
      if (!first) continue;
      a.S[ij] = accS[x];
      a.S[ji] = accS[x];
      a.T[ij] = accT[x];
      a.T[ji] = accT[x];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        a.M[d * a.nn + ij] = accM[d][x];
        a.M[d * a.nn + ji] = accM[d][x];
      }
    }
}

extern "C" int mmdg_one_electron(mmdg_context* h, int natom, const int* atom_mol, const double* atom_xyz,
                                 const double* atom_Z, const double* origin, double* S, double* T, double* V,
                                 double* M, void* stream) {
  if (!h || natom < 1 || !atom_mol || !atom_xyz || !atom_Z || !origin || !S || !T || !V || !M)
    return fail(MMDG_E_ARG, "mmdg_one_electron: bad argument");
  if (!h->have_basis) return fail(MMDG_E_STATE, "mmdg_one_electron: no basis set");
  DeviceGuard dg(h->device);
  std::vector<int> ab(h->nmol, 0), ae(h->nmol, 0);
  for (int i = 0; i < natom; ++i) {
    const int m = atom_mol[i];
    if (m < 0 || m >= h->nmol || (i > 0 && m < atom_mol[i - 1]))
      return fail(MMDG_E_ARG, "mmdg_one_electron: atoms must be sorted by molecule");
  }
  for (int m = 0, i = 0; m < h->nmol; ++m) {
    ab[m] = i;
    while (i < natom && atom_mol[i] == m) ++i;
    ae[m] = i;
  }
  DevBuf<int> d_ab, d_ae;
  DevBuf<double> d_xyz, d_Z, d_o;
  std::vector<double> vx(atom_xyz, atom_xyz + 3 * (size_t)natom), vZ(atom_Z, atom_Z + natom),
      vo(origin, origin + 3 * (size_t)h->nmol);
  if (d_ab.upload(ab) || d_ae.upload(ae) || d_xyz.upload(vx) || d_Z.upload(vZ) || d_o.upload(vo))
    return fail(MMDG_E_NOMEM, "mmdg_one_electron: allocation");
  cudaStream_t st = (cudaStream_t)stream;
  const long long nn = h->ntot_nn;
  CUDA_TRY(cudaMemsetAsync(S, 0, sizeof(double) * nn, st));
  CUDA_TRY(cudaMemsetAsync(T, 0, sizeof(double) * nn, st));
  CUDA_TRY(cudaMemsetAsync(V, 0, sizeof(double) * nn, st));
  CUDA_TRY(cudaMemsetAsync(M, 0, sizeof(double) * 3 * nn, st));
  OneEArgs a;
  a.npair = h->npair;
  a.pa = h->d_pa.p;
  a.pb = h->d_pb.p;
  a.L = h->d_L.p;
  a.nprim = h->d_nprim.p;
  a.poff = h->d_poff.p;
  a.func = h->d_func.p;
  a.sh_mol = h->d_shmol.p;
  a.center = h->d_center.p;
  a.exps = h->d_exp.p;
  a.coefs = h->d_coef.p;
  a.mol_base = h->d_mol_base.p;
  a.mol_n = h->d_mol_n.p;
  a.atom_begin = d_ab.p;
  a.atom_end = d_ae.p;
  a.atom_xyz = d_xyz.p;
  a.atom_Z = d_Z.p;
  a.origin = d_o.p;
  a.nn = nn;
  a.boys = h->boys64.p;
  a.S = S;
  a.T = T;
  a.V = V;
  a.M = M;
  int max_atoms = 1;
  for (int m = 0; m < h->nmol; ++m) max_atoms = std::max(max_atoms, ae[m] - ab[m]);
  // one launch per pair class (pairs are stored with la >= lb)
  static_assert(MMDG_LMAX == 2, "the one-electron dispatch covers l <= 2");
  for (int la = 0; la <= MMDG_LMAX; ++la)
    for (int lb = 0; lb <= la; ++lb) {
      const int c = pair_class(la, lb), n = h->cls_count[c];
      if (n == 0) continue;
      const dim3 grid((n + 63) / 64, max_atoms);
      const int* pl = h->d_cls[c].p;
      switch (c) {
        case 0: k_one_electron<0, 0><<<grid, 64, 0, st>>>(a, pl, n); break;
        case 1: k_one_electron<1, 0><<<grid, 64, 0, st>>>(a, pl, n); break;
        case 2: k_one_electron<1, 1><<<grid, 64, 0, st>>>(a, pl, n); break;
        case 3: k_one_electron<2, 0><<<grid, 64, 0, st>>>(a, pl, n); break;
        case 4: k_one_electron<2, 1><<<grid, 64, 0, st>>>(a, pl, n); break;
        default: k_one_electron<2, 2><<<grid, 64, 0, st>>>(a, pl, n); break;
      }
      CUDA_TRY(cudaGetLastError());
    }
  CUDA_TRY(cudaStreamSynchronize(st));  // the temporary atom buffers are freed on return
  return MMDG_OK;
}

// ------------------------------------------------------------------ peak probe
// Throughput of dependent-free FMA chains: the FP64 (DFMA) and FP32 (FFMA) roofline
// denominators of this GPU, measured at the clocks of the moment.
template <typename T>
__global__ void k_fma_probe(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
      x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

extern "C" int mmdg_measure_peaks(mmdg_context* h, double* fp64_tflops, double* fp32_tflops) {
  if (!h || !fp64_tflops || !fp32_tflops) return fail(MMDG_E_ARG, "mmdg_measure_peaks: null argument");
  DeviceGuard dg(h->device);
  int sms = 0;
  CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device));
  const int blocks = sms * 8, threads = 256;
  DevBuf<double> out;
  if (out.alloc((size_t)blocks * threads)) return fail(MMDG_E_NOMEM, "mmdg_measure_peaks: allocation");
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0));
  CUDA_TRY(cudaEventCreate(&e1));
  float ms = 0.f;
  const double n = double(blocks) * threads;
  k_fma_probe<double><<<blocks, threads>>>(out.p, 20, 0.999, 1e-3);
  CUDA_TRY(cudaEventRecord(e0));
  k_fma_probe<double><<<blocks, threads>>>(out.p, 400, 0.999, 1e-3);
  CUDA_TRY(cudaEventRecord(e1));
  CUDA_TRY(cudaEventSynchronize(e1));
  CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
  *fp64_tflops = 2.0 * 64 * 400 * n / (ms * 1e-3) / 1e12;
  float* fo = reinterpret_cast<float*>(out.p);
  k_fma_probe<float><<<blocks, threads>>>(fo, 200, 0.999f, 1e-3f);
  CUDA_TRY(cudaEventRecord(e0));
  k_fma_probe<float><<<blocks, threads>>>(fo, 20000, 0.999f, 1e-3f);
  CUDA_TRY(cudaEventRecord(e1));
  CUDA_TRY(cudaEventSynchronize(e1));
  CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
  *fp32_tflops = 2.0 * 64 * 20000 * n / (ms * 1e-3) / 1e12;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CUDA_TRY(cudaGetLastError());
  return MMDG_OK;
}

// FP64 pipes of this GPU: independent DFMA chains, independent FP64 tensor-core
// chains (mma.sync m8n8k4 f64: 512 FLOPs per warp instruction), and both in one
// kernel -- whether the two run side by side (time of both ~ the longer alone) or
// share one resource (time of both ~ the sum).  This is the measurement behind
// the choice of CUDA-core FP64 for the ERI transforms.
__device__ __forceinline__ void dmma_m8n8k4(double& d0, double& d1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};\n"
               : "+d"(d0), "+d"(d1)
               : "d"(a), "d"(b));
}

template <bool FMA, bool MMA>
__global__ void k_fp64_pipe_probe(double* out, int iters_fma, int iters_mma, double a, double b) {
  double x[8], c0[8], c1[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    x[k] = threadIdx.x + k;
    c0[k] = 1e-3 * k;
    c1[k] = 2e-3 * k;
  }
  const int iters = FMA && MMA ? (iters_fma > iters_mma ? iters_fma : iters_mma) : (FMA ? iters_fma : iters_mma);
  for (int i = 0; i < iters; ++i) {
    if (FMA && i < iters_fma) {
#pragma unroll
      for (int r = 0; r < 8; ++r)
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
    }
    if (MMA && i < iters_mma) {
#pragma unroll
      for (int k = 0; k < 8; ++k) dmma_m8n8k4(c0[k], c1[k], a, b);
    }
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k] + c0[k] + c1[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

extern "C" int mmdg_measure_fp64_pipes(mmdg_context* h, int warps_per_sm, double* res) {
  if (!h || !res) return fail(MMDG_E_ARG, "mmdg_measure_fp64_pipes: null argument");
  if (warps_per_sm < 1 || warps_per_sm > 64) return fail(MMDG_E_ARG, "mmdg_measure_fp64_pipes: 1..64 warps per SM");
  DeviceGuard dg(h->device);
  int sms = 0;
  CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device));
  const int threads = 256, blocks = sms * ((warps_per_sm * 32 + threads - 1) / threads);
  DevBuf<double> out;
  if (out.alloc((size_t)blocks * threads)) return fail(MMDG_E_NOMEM, "mmdg_measure_fp64_pipes: allocation");
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0));
  CUDA_TRY(cudaEventCreate(&e1));
  const int it_fma = 200, it_mma = 400;
  float ms[3] = {0.f, 0.f, 0.f};
  for (int rep = 0; rep < 2; ++rep) {  // first pass warms up
    CUDA_TRY(cudaEventRecord(e0));
    k_fp64_pipe_probe<true, false><<<blocks, threads>>>(out.p, it_fma, it_mma, 0.999, 1e-3);
    CUDA_TRY(cudaEventRecord(e1));
    CUDA_TRY(cudaEventSynchronize(e1));
    CUDA_TRY(cudaEventElapsedTime(&ms[0], e0, e1));
    CUDA_TRY(cudaEventRecord(e0));
    k_fp64_pipe_probe<false, true><<<blocks, threads>>>(out.p, it_fma, it_mma, 0.999, 1e-3);
    CUDA_TRY(cudaEventRecord(e1));
    CUDA_TRY(cudaEventSynchronize(e1));
    CUDA_TRY(cudaEventElapsedTime(&ms[1], e0, e1));
    CUDA_TRY(cudaEventRecord(e0));
    k_fp64_pipe_probe<true, true><<<blocks, threads>>>(out.p, it_fma, it_mma, 0.999, 1e-3);
    CUDA_TRY(cudaEventRecord(e1));
    CUDA_TRY(cudaEventSynchronize(e1));
    CUDA_TRY(cudaEventElapsedTime(&ms[2], e0, e1));
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CUDA_TRY(cudaGetLastError());
  const double nthr = double(blocks) * threads;
  res[0] = 2.0 * 64 * it_fma * nthr / (ms[0] * 1e-3) / 1e12;                 // DFMA TFLOP/s
  res[1] = 512.0 * 8 * it_mma * (nthr / 32) / (ms[1] * 1e-3) / 1e12;        // DMMA TFLOP/s
  res[2] = ms[0];
  res[3] = ms[1];
  res[4] = ms[2];
  return MMDG_OK;
}

void mmdg_fill_boys_table(double* t64) { build_boys_table_raw(t64, nullptr); }

// host copy of the Boys interpolation table (no GPU needed): for tests
extern "C" long long mmdg_boys_table(double* out, long long n) {
  if (!out) return kBoysTabSize;
  if (n < kBoysTabSize) return fail(MMDG_E_ARG, "mmdg_boys_table: buffer too small");
  std::vector<double> t64;
  std::vector<float> t32;
  build_boys_table(t64, t32);
  std::memcpy(out, t64.data(), sizeof(double) * kBoysTabSize);
  return kBoysTabSize;
}

// ------------------------------------------------------------------ tuning, CUDA graph
extern "C" int mmdg_set_tuning(mmdg_context* h, int cls, int grid_blocks) {
  if (!h) return fail(MMDG_E_ARG, "mmdg_set_tuning: null context");
  if (cls < 0 || cls >= MMDG_NCLASS || grid_blocks < 0) return fail(MMDG_E_ARG, "mmdg_set_tuning: bad class or grid");
  h->class_grid[cls] = grid_blocks;
  if (h->graph) {
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  return MMDG_OK;
}

// tile of a class's Fock kernel: threads per block of the per-thread kernels (64, 128
// or 256; classes with shared-memory R tables keep 128) and quartets per work item
// of the warp-cooperative kernels (1..8); 0 restores the default
extern "C" int mmdg_set_tile(mmdg_context* h, int cls, int block_threads, int item) {
  if (!h) return fail(MMDG_E_ARG, "mmdg_set_tile: null context");
  if (cls < 0 || cls >= MMDG_NCLASS) return fail(MMDG_E_ARG, "mmdg_set_tile: bad class");
  if (block_threads != 0 && block_threads != 64 && block_threads != 128 && block_threads != 256)
    return fail(MMDG_E_ARG, "mmdg_set_tile: threads per block must be 64, 128 or 256 (0: default)");
  if (item < 0 || item > 8) return fail(MMDG_E_ARG, "mmdg_set_tile: quartets per work item must be 0..8");
  h->class_block[cls] = block_threads;
  h->class_item[cls] = item;
  if (h->graph) {
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  return MMDG_OK;
}

// ------------------------------------------------------------------ nuclear gradient
#include "grad.cuh"

extern "C" int mmdg_rhf_gradient(mmdg_context* h, const double* P, const double* W, int natom,
                                 const double* atom_xyz, const double* atom_Z, const int* shell_atom, double qtol,
                                 double* grad, void* stream) {
  if (!h || !P || !W || !atom_xyz || !atom_Z || !shell_atom || !grad || natom < 1)
    return fail(MMDG_E_ARG, "mmdg_rhf_gradient: null argument");
  if (!h->have_basis) return fail(MMDG_E_STATE, "mmdg_rhf_gradient: no basis set");
  if (h->nmol != 1) return fail(MMDG_E_ARG, "mmdg_rhf_gradient: one molecule per context");
  for (int s = 0; s < h->nshell; ++s)
    if (shell_atom[s] < 0 || shell_atom[s] >= natom) return fail(MMDG_E_ARG, "mmdg_rhf_gradient: shell_atom out of range");
  DeviceGuard dgd(h->device);
  cudaStream_t st = (cudaStream_t)stream;
  DevBuf<double> dxyz, dZ, dg;
  DevBuf<int> dsa;
  if (dxyz.upload(std::vector<double>(atom_xyz, atom_xyz + 3 * natom)) != cudaSuccess ||
      dZ.upload(std::vector<double>(atom_Z, atom_Z + natom)) != cudaSuccess ||
      dsa.upload(std::vector<int>(shell_atom, shell_atom + h->nshell)) != cudaSuccess ||
      dg.alloc(3 * (size_t)natom) != cudaSuccess)
    return fail(MMDG_E_NOMEM, "mmdg_rhf_gradient: allocation");
  CUDA_TRY(cudaMemsetAsync(dg.p, 0, sizeof(double) * 3 * natom, st));
  GradArgs a;
  a.npair = h->npair;
  a.pa = h->d_pa.p;
  a.pb = h->d_pb.p;
  a.L = h->d_L.p;
  a.nprim = h->d_nprim.p;
  a.poff = h->d_poff.p;
  a.func = h->d_func.p;
  a.shell_atom = dsa.p;
  a.center = h->d_center.p;
  a.exps = h->d_exp.p;
  a.coefs = h->d_coef.p;
  if (!(qtol >= 0.0)) return fail(MMDG_E_ARG, "mmdg_rhf_gradient: qtol must be >= 0");
  a.Qpair = qtol > 0.0 ? h->d_Q.p : nullptr;
  a.qtol = qtol;
  a.natom = natom;
  a.xyz = dxyz.p;
  a.Z = dZ.p;
  a.P = P;
  a.W = W;
  a.N = h->mol_n[0];
  a.grad = dg.p;
  CUDA_TRY(mmdg_launch_rhf_gradient(a, st));
  std::vector<double> g(3 * (size_t)natom);
  CUDA_TRY(cudaMemcpyAsync(g.data(), dg.p, sizeof(double) * 3 * natom, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  // nuclear repulsion: d/dR_A sum_{B<C} Z_B Z_C / R_BC (mmd/forces.py:50-58)
  for (int A = 0; A < natom; ++A)
    for (int B = 0; B < natom; ++B) {
      if (A == B) continue;
      double d[3], r2 = 0.0;
      for (int x = 0; x < 3; ++x) {
        d[x] = atom_xyz[3 * A + x] - atom_xyz[3 * B + x];
        r2 += d[x] * d[x];
      }
      if (r2 == 0.0) continue;
      const double r3 = r2 * std::sqrt(r2);
      for (int x = 0; x < 3; ++x) g[3 * A + x] -= atom_Z[A] * atom_Z[B] * d[x] / r3;
    }
  for (int i = 0; i < 3 * natom; ++i) grad[i] = g[i];
  return MMDG_OK;
}

extern "C" int mmdg_set_prim_tol(mmdg_context* h, double tol) {
  if (!h) return fail(MMDG_E_ARG, "mmdg_set_prim_tol: null context");
  if (!(tol >= 0.0) || !std::isfinite(tol)) return fail(MMDG_E_ARG, "mmdg_set_prim_tol: tolerance must be >= 0");
  h->prim_tol = tol;
  return MMDG_OK;
}

extern "C" int mmdg_set_streams(mmdg_context* h, int nstreams) {
  if (!h) return fail(MMDG_E_ARG, "mmdg_set_streams: null context");
  if (nstreams < 1 || nstreams > kMaxStreams) return fail(MMDG_E_ARG, "mmdg_set_streams: 1 to 8 streams");
  DeviceGuard dg(h->device);
  if (!h->fork_ev) CUDA_TRY(cudaEventCreateWithFlags(&h->fork_ev, cudaEventDisableTiming));
  for (int k = 0; k < nstreams; ++k) {
    if (!h->side[k]) CUDA_TRY(cudaStreamCreateWithFlags(&h->side[k], cudaStreamNonBlocking));
    if (!h->join_ev[k]) CUDA_TRY(cudaEventCreateWithFlags(&h->join_ev[k], cudaEventDisableTiming));
  }
  h->nstreams = nstreams;
  if (h->graph) {
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  return MMDG_OK;
}

// Sharded Fock build: later builds of this context digest only the shell quartets of
// part `part` of `nparts`.  pair_owner[k] (host, 0..nparts-1) is the owner of the k-th
// shell pair in canonical order -- for each molecule, s1 ascending, then s2 = first
// shell of the molecule .. s1 (global shell indices), i.e. by s1(s1+1)/2 + s2 -- and a
// shell quartet belongs to the owner of its pair with the larger canonical index, so
// the parts' G add up to the full G.  nparts = 1 (pair_owner may be null) switches
// sharding off.
extern "C" int mmdg_set_partition(mmdg_context* h, int part, int nparts, const int* pair_owner, long long npairs) {
  if (!h) return fail(MMDG_E_ARG, "mmdg_set_partition: null context");
  if (!h->have_basis) return fail(MMDG_E_STATE, "mmdg_set_partition: no basis set");
  if (nparts < 1 || part < 0 || part >= nparts) return fail(MMDG_E_ARG, "mmdg_set_partition: bad part / nparts");
  DeviceGuard dgd(h->device);
  if (h->graph) {
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  if (nparts == 1) {
    h->part = 0;
    h->nparts = 1;
    return MMDG_OK;
  }
  if (!pair_owner || npairs != h->npair) return fail(MMDG_E_ARG, "mmdg_set_partition: one owner per shell pair");
  std::vector<int> own(h->npair), canon(h->npair);
  long long k = 0;
  for (int s1 = 0; s1 < h->nshell; ++s1) {
    int first = s1;
    while (first > 0 && h->shell_molv[first - 1] == h->shell_molv[s1]) --first;
    for (int s2 = first; s2 <= s1; ++s2, ++k) {
      const int o = pair_owner[k];
      if (o < 0 || o >= nparts) return fail(MMDG_E_ARG, "mmdg_set_partition: owner out of range");
      const int p = h->pair_row[s1] + (s1 - s2);
      own[p] = o;
      canon[p] = (s1 - first) * (s1 - first + 1) / 2 + (s2 - first);
    }
  }
  if (h->d_pair_owner.upload(own) != cudaSuccess || h->d_pair_canon.upload(canon) != cudaSuccess)
    return fail(MMDG_E_NOMEM, "mmdg_set_partition: allocation");
  h->part = part;
  h->nparts = nparts;
  return MMDG_OK;
}

extern "C" int mmdg_fock_graph(mmdg_context* h, const double* dP, double* G, double tol, double fp32_below,
                               void* stream) {
  if (!h || !dP || !G) return fail(MMDG_E_ARG, "mmdg_fock_graph: null argument");
  if (!h->have_basis) return fail(MMDG_E_STATE, "mmdg_fock_graph: no basis set");
  DeviceGuard dgd(h->device);
  cudaStream_t st = (cudaStream_t)stream;
  const bool same = h->graph && h->g_dP == dP && h->g_G == G && h->g_tol == tol && h->g_split == fp32_below;
  if (!same) {
    if (h->graph) {
      cudaGraphExecDestroy(h->graph);
      h->graph = nullptr;
    }
    // first build eagerly: allocates the quartet lists outside any capture
    int rc = fock_impl(h, dP, G, tol, fp32_below, nullptr, nullptr, st);
    if (rc) return rc;
    CUDA_TRY(cudaStreamSynchronize(st));
    if (!h->g_stream) CUDA_TRY(cudaStreamCreateWithFlags(&h->g_stream, cudaStreamNonBlocking));
    cudaGraph_t graph = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(h->g_stream, cudaStreamCaptureModeThreadLocal));
    rc = fock_impl(h, dP, G, tol, fp32_below, nullptr, nullptr, h->g_stream);
    cudaError_t e = cudaStreamEndCapture(h->g_stream, &graph);
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (e != cudaSuccess) return fail(MMDG_E_CUDA, std::string("mmdg_fock_graph: capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&h->graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(MMDG_E_CUDA, std::string("mmdg_fock_graph: instantiate: ") + cudaGetErrorString(e));
    h->g_dP = dP;
    h->g_G = G;
    h->g_tol = tol;
    h->g_split = fp32_below;
    return MMDG_OK;  // this call's build ran eagerly above
  }
  CUDA_TRY(cudaGraphLaunch(h->graph, st));
  return MMDG_OK;
}
