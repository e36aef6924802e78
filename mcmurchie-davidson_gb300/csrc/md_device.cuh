// md_device.cuh -- device building blocks of the McMurchie-Davidson ERI kernels.
//
// Numerics restate the reference (jjgoings/McMurchie-Davidson):
//   * Boys function F_m(T) (cython/util.pxi:54-55) by tabulated Taylor interpolation
//     plus downward recursion F_{m-1} = (2T F_m + e^{-T})/(2m-1); for T >= 48 the
//     asymptotic F_0 = sqrt(pi/T)/2 and upward recursion F_{m+1} = ((2m+1)F_m - e^{-T})/(2T).
//   * R^(n)_000 = (-2 alpha)^n F_n(alpha |PQ|^2) (cython/util.pxi:37-38) with the
//     prefactor 2 pi^{5/2} / (p q sqrt(p+q)) (cython/twoe.pyx:93) folded in.
//   * Fock digestion of one function quartet exactly as formPT (cython/fock.pyx:40-85):
//     canonical labels i>=j, k>=l, ij>=kl; Schwarz x density screening; degeneracy
//     s12*s34*s12_34; two Coulomb and four exchange updates of the unsymmetrised G.
//
// Every FP64 instruction goes through GB300's narrow FP64 pipe (measured 1.19
// TFLOP/s against 73 TFLOP/s FP32), so integer and FP32 work is used wherever the
// result does not need FP64: indices, screening (FP32 with a guard band; exact FP64
// only near the threshold), table lookups.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace mmdg {

constexpr int kMaxComp = 6;         // Cartesian components of a d shell
constexpr int kBoysNGrid = 768;     // T_k = k/16, k = 0..767 (T < 48)
constexpr int kBoysLMax = 8;        // highest order the ERI classes need ((dd|dd))
constexpr int kBoysRow = 8;         // doubles per (k, L) Taylor row (7 used)
constexpr int kBoysExpOff = kBoysNGrid * (kBoysLMax + 1) * kBoysRow;  // exp rows after the F rows
constexpr int kBoysTabSize = kBoysExpOff + kBoysNGrid * kBoysRow;
constexpr double kBoysTaylorMax = 48.0 - 1.0 / 32.0;
// the same rows as float pairs (hi, lo) for the double-float evaluation: a row is 16
// floats, hi[0..7] then lo[0..7], with hi + lo the FP64 coefficient to ~48 bits
constexpr int kBoysDfRow = 16;
constexpr double kTwoPi52 = 34.986836655249725;  // 2 pi^{5/2}
// sqrt(2 pi^{5/2}): folded into every E' coefficient by the pair kernel, so the
// product of a bra and a ket coefficient carries the 2 pi^{5/2} of the primitive ERI
// (cython/twoe.pyx:93) and the quartet code multiplies by 1/sqrt(p+q) only
constexpr double kSqrtTwoPi52 = 5.914967172795613;
constexpr double kHalfSqrtPi = 0.88622692545275801;

// A non-negative double as a float rounded toward zero, from its bit pattern on the
// integer pipe (exponent rebiased, top 23 mantissa bits kept: relative error below
// 2^-23); values below the normal float range (zero included) give 0.
__device__ __forceinline__ float f32_of_nonneg(double x) {
  const int hi = __double2hiint(x);
  const unsigned lo = (unsigned)__double2loint(x);
  const int fe = min((hi >> 20) - (1023 - 127), 254);
  return fe <= 0 ? 0.0f : __int_as_float((fe << 23) | ((hi & 0xfffff) << 3) | (int)(lo >> 29));
}

// a positive normal float as a double, exactly, on the integer pipe
__device__ __forceinline__ double f64_of_positive(float y) {
  const int b = __float_as_int(y);
  return __hiloint2double((((b >> 23) + (1023 - 127)) << 20) | ((b & 0x7fffff) >> 3), (b & 7) << 29);
}

// a finite float as a double, exactly, on the integer pipe (zero and subnormal: 0)
__device__ __forceinline__ double f64_of_float(float x) {
  const int b = __float_as_int(x);
  const int e = (b >> 23) & 0xff;
  if (e == 0) return 0.0;
  return __hiloint2double((b & 0x80000000) | ((e + (1023 - 127)) << 20) | ((b & 0x7fffff) >> 3), (b & 7) << 29);
}

// a double as a float rounded toward zero, sign kept, on the integer pipe (relative
// error below 2^-23; magnitudes below the normal float range give 0)
__device__ __forceinline__ float f32_of_double_tz(double x) {
  const int hi = __double2hiint(x);
  const unsigned lo = (unsigned)__double2loint(x);
  const int fe = min(((hi >> 20) & 0x7ff) - (1023 - 127), 254);
  return fe <= 0 ? 0.0f
                 : __int_as_float((hi & 0x80000000) | (fe << 23) | ((hi & 0xfffff) << 3) | (int)(lo >> 29));
}

// 1/sqrt(x) for a positive double whose magnitude is within the normal float range:
// the single-precision estimate y0 = rsqrtf(x) (special-function unit; x and y0
// moved between formats on the integer pipe) and one third-order step of the
// Newton/Householder iteration for the inverse square root,
//     e = 1 - x y0^2,   y = y0 (1 + e/2 + 3 e^2/8) = y0 + (y0/2) (e + (3e/4) e),
// whose error is 5/16 e^3 + O(e^4); |e| < 2^-20 leaves it far below double rounding.
// The factor 3e/4 only scales a term below 2^-40 of the result, so it is taken from
// the FP32 pipe (24 bits), and y0/2 is exact in FP32: four FP64 instructions (a
// product and three FMAs), the same rounding as the all-FP64 step.
__device__ __forceinline__ double rsqrt_dd(double x) {
  const float y0f = rsqrtf(f32_of_nonneg(x));
  const double y0 = f64_of_positive(y0f);
  const double e = fma(-x, y0 * y0, 1.0);  // y0 has 24 significant bits: y0^2 is exact
  const double b = fma(f64_of_float(0.75f * f32_of_double_tz(e)), e, e);  // e + 3e^2/4
  return fma(f64_of_positive(0.5f * y0f), b, y0);
}

// (-1)^s x by an integer XOR of the sign bit.  A select between x and -x compiles to
// an FP64 negation (an add) per term, which costs the FP64 pipe as much as the FMA it
// feeds; the XOR runs on the integer pipe.
__device__ __forceinline__ double flip_sign(double x, int s) {
  return __hiloint2double(__double2hiint(x) ^ (int)((unsigned)s << 31), __double2loint(x));
}
__device__ __forceinline__ float flip_sign(float x, int s) {
  return __int_as_float(__float_as_int(x) ^ (int)((unsigned)s << 31));
}

// ---------------------------------------------------------------------------------
// geometry shared by every kernel
struct Geometry {
  // primitive pairs
  const double4_32a* __restrict__ pP;   // (p, Px, Py, Pz) per primitive pair
  const float4* __restrict__ pPf;   // FP32: (p, Px, Py, Pz) rounded, then (0, Px, Py, Pz) remainders: 2 per pair
  const double* __restrict__ E64;   // E' tables, FP64
  const float* __restrict__ E32;    // E' tables, FP32
  // shell pairs
  const int* __restrict__ pr_begin;  // first primitive pair
  const int* __restrict__ pr_count;  // number of primitive pairs
  const long long* __restrict__ e_off;  // offset of the pair's E' table (prim k at e_off + k*nnz)
  const int* __restrict__ pa;        // shell a (la >= lb)
  const int* __restrict__ pb;        // shell b
  const float* __restrict__ Q;       // Schwarz bound max_{ij in ab} sqrt((ij|ij))
  // shells
  const int* __restrict__ func;      // [nshell*kMaxComp] molecule-local function index or -1
  const int* __restrict__ sh_mol;    // molecule of the shell
  const int* __restrict__ sh_local;  // molecule-local shell index
  // molecules (packed N_m x N_m blocks; one molecule for a single system)
  const long long* __restrict__ mol_base;    // offset of the molecule's N x N block
  const int* __restrict__ mol_n;             // N_m
  const long long* __restrict__ mol_sbase;   // offset of the molecule's S x S shell block
  const int* __restrict__ mol_ns;            // S_m
  const long long* __restrict__ mol_tbase;   // offset of the molecule's N(N+1)/2 pair table
  // Boys tables
  const double* __restrict__ boys64;  // [kBoysTabSize]
  const float* __restrict__ boys32;
  const float* __restrict__ boysdf;   // [kBoysTabSize / kBoysRow * kBoysDfRow]: (hi, lo) rows
};

// ---------------------------------------------------------------------------------
// Boys function: Fn[0..L] at T
// Table layout (L-major, so one class touches a contiguous 48 KB): row (L, k)
// holds c_n = F_{L+n}(T_k) / n!, n = 0..6, so that
//   F_L(T) = sum_n c_n y^n,  y = T_k - T,  |y| <= 1/32,
// and row (k, exp) holds e_n = exp(-T_k) / n!, n = 0..7, for exp(-T) = sum_n e_n y^n.
// Truncation: F_{L+7} |y|^7 / 7! < 6e-15 F_L and |y|^8/8! < 3e-17 relative.
// Horner evaluation of one Taylor row c_0..c_6 at y (six FMAs)
__device__ __forceinline__ double boys_row(const double2& c01, const double2& c23, const double2& c45, const double2& c67,
                                           double y) {
  double f = fma(c67.x, y, c45.y);
  f = fma(f, y, c45.x);
  f = fma(f, y, c23.y);
  f = fma(f, y, c23.x);
  f = fma(f, y, c01.y);
  return fma(f, y, c01.x);
}

// The table index k = round(16 T) and the branch test come from an FP32 copy of T
// (integer and FP32 pipes); slot 7 of every F row holds T_k itself, so y = T_k - T is
// one FP64 subtraction.  T_f <= T (truncated toward zero), so |y| stays within
// 1/32 + 2^-17.
template <int L>
__device__ __forceinline__ void boys_eval(const double* __restrict__ tab, double T, double* Fn) {
  const float Tf = f32_of_nonneg(T);
  if (Tf < float(kBoysTaylorMax)) {
    const int k = __float2int_rn(Tf * 16.0f);
    // a table row is 64 bytes (64-byte aligned): four 16-byte loads
    const double2* __restrict__ c = reinterpret_cast<const double2*>(tab + (L * kBoysNGrid + k) * kBoysRow);
    const double2 c01 = __ldg(c), c23 = __ldg(c + 1), c45 = __ldg(c + 2), c67 = __ldg(c + 3);
    const double y = c67.y - T;  // T_k - T
    Fn[L] = boys_row(c01, c23, c45, c67, y);
    if (L == 1) {
      // F_0 from its own row: 6 FMAs instead of exp(-T) (7) and one recursion step (3)
      const double2* __restrict__ c0 = reinterpret_cast<const double2*>(tab + k * kBoysRow);
      Fn[0] = boys_row(__ldg(c0), __ldg(c0 + 1), __ldg(c0 + 2), __ldg(c0 + 3), y);
    } else if (L > 1) {
      const double2* __restrict__ e = reinterpret_cast<const double2*>(tab + kBoysExpOff + k * kBoysRow);
      const double2 e01 = __ldg(e), e23 = __ldg(e + 1), e45 = __ldg(e + 2), e67 = __ldg(e + 3);
      double x = fma(e67.y, y, e67.x);
      x = fma(x, y, e45.y);
      x = fma(x, y, e45.x);
      x = fma(x, y, e23.y);
      x = fma(x, y, e23.x);
      x = fma(x, y, e01.y);
      const double eT = fma(x, y, e01.x);
      const double T2 = T + T;
#pragma unroll
      for (int m = L; m > 0; --m) Fn[m - 1] = fma(T2, Fn[m], eT) * (1.0 / double(2 * m - 1));
    }
  } else {
    // F_0 = sqrt(pi/T)/2 and F_{m+1} = ((2m+1) F_m - exp(-T)) / (2T); for T >= 48 and
    // m <= 4 the exp(-T) terms change F_m by less than 5e-15 relative and are dropped
    const double rs = rsqrt_dd(T);
    Fn[0] = kHalfSqrtPi * rs;
    if (L > 0) {
      const double iT = rs * rs;
      if (L > 4) {
        const double eTh = 0.5 * exp(-T);
#pragma unroll
        for (int m = 0; m < L; ++m) Fn[m + 1] = fma(double(m) + 0.5, Fn[m], -eTh) * iT;
      } else {
#pragma unroll
        for (int m = 0; m < L; ++m) Fn[m + 1] = (double(m) + 0.5) * iT * Fn[m];
      }
    }
  }
}

template <int L>
__device__ __forceinline__ void boys_eval(const float* __restrict__ tab, float T, float* Fn) {
  if (T < float(kBoysTaylorMax)) {
    int k = __float2int_rn(T * 16.0f);
    k = min(max(k, 0), kBoysNGrid - 1);
    const float y = fmaf(float(k), 0.0625f, -T);
    const float* __restrict__ c = tab + (L * kBoysNGrid + k) * kBoysRow;  // 32-byte rows
    const float4 c03 = __ldg(reinterpret_cast<const float4*>(c));
    float f = fmaf(__ldg(c + 4), y, c03.w);
    f = fmaf(f, y, c03.z);
    f = fmaf(f, y, c03.y);
    Fn[L] = fmaf(f, y, c03.x);
    if (L > 0) {
      const float* __restrict__ e = tab + kBoysExpOff + k * kBoysRow;
      const float4 e03 = __ldg(reinterpret_cast<const float4*>(e));
      float x = fmaf(__ldg(e + 4), y, e03.w);
      x = fmaf(x, y, e03.z);
      x = fmaf(x, y, e03.y);
      const float eT = fmaf(x, y, e03.x);
      const float T2 = T + T;
#pragma unroll
      for (int m = L; m > 0; --m) Fn[m - 1] = fmaf(T2, Fn[m], eT) * (1.0f / float(2 * m - 1));
    }
  } else {
    const float rs = rsqrtf(T);
    Fn[0] = float(kHalfSqrtPi) * rs;
    if (L > 0) {
      const float iT = rs * rs;
#pragma unroll
      for (int m = 0; m < L; ++m) Fn[m + 1] = (float(m) + 0.5f) * iT * Fn[m];
    }
  }
}

// ---------------------------------------------------------------------------------
// Double-float ("float pair") arithmetic on the FP32 pipe, after Dekker (1971) and
// Knuth's two-sum, with the FMA giving exact products: a value is hi + lo with
// |lo| <= ulp(hi)/2, about 48 significant bits.  Used where a result needs ~1e-14
// relative accuracy and the FP64 pipe (1/61 of the FP32 rate here) is the bottleneck.
struct DF {
  float hi, lo;
};
__device__ __forceinline__ DF df_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ DF df_fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = a + b;
  return {s, b - (s - a)};
}
// a * y + c: the Horner step
__device__ __forceinline__ DF df_fma(DF a, DF y, DF c) {
  const float p = a.hi * y.hi;
  float e = fmaf(a.hi, y.hi, -p);
  e = fmaf(a.hi, y.lo, e);
  e = fmaf(a.lo, y.hi, e);
  DF s = df_two_sum(p, c.hi);
  return df_fast_two_sum(s.hi, s.lo + (e + c.lo));
}

// a double as a float pair on the integer pipe: hi = the top 24 significant bits,
// lo = the next 29 rounded to 24 (|x| below 2^-74: lo = 0; below 2^-126: 0)
__device__ __forceinline__ DF df_of_double(double x) {
  const int hi = __double2hiint(x);
  const unsigned lo = (unsigned)__double2loint(x);
  const int e = (hi >> 20) & 0x7ff;
  const int sign = hi & 0x80000000;
  if (e < 1023 - 126) return {0.0f, 0.0f};
  const float h = __int_as_float(sign | ((e - (1023 - 127)) << 23) | ((hi & 0xfffff) << 3) | (int)(lo >> 29));
  float l = 0.0f;
  if (e >= 1023 - 74) {
    const float scale = __int_as_float((e - 1075 + 127) << 23);  // 2^(e - 1075)
    l = __int2float_rn((int)(lo & 0x1fffffffu)) * scale;
    l = sign ? -l : l;
  }
  return {h, l};
}

// sum_{n >= 1} c_n y^(n-1) over one table row (n up to 6, or 7 for an exp row), as a
// float pair: the terms n >= 5 (below 3e-10 of the row's sum for |y| <= 1/32) in FP32,
// n = 4..1 by double-float Horner steps
template <int DEG>
__device__ __forceinline__ DF df_row_tail(const float* __restrict__ row, DF y) {
  const float4 h0 = __ldg(reinterpret_cast<const float4*>(row)), h1 = __ldg(reinterpret_cast<const float4*>(row) + 1);
  const float4 l0 = __ldg(reinterpret_cast<const float4*>(row) + 2), l1 = __ldg(reinterpret_cast<const float4*>(row) + 3);
  float t = DEG == 7 ? fmaf(h1.w, y.hi, h1.z) : h1.z;  // c7 y + c6, or c6
  t = fmaf(t, y.hi, h1.y);                             // ... + c5
  DF p{t, 0.0f};
  p = df_fma(p, y, DF{h1.x, l1.x});
  p = df_fma(p, y, DF{h0.w, l0.w});
  p = df_fma(p, y, DF{h0.z, l0.z});
  p = df_fma(p, y, DF{h0.y, l0.y});
  return p;
}

// one Taylor row: c_0 + y * tail, the last step in FP64 (c_0 read from the FP64 row),
// so the float pair's ~2^-47 relative error reaches the result scaled by |y| <= 1/32
template <int DEG>
__device__ __forceinline__ double df_row(const float* __restrict__ row, const double* __restrict__ row64, double y,
                                         DF ydf) {
  const DF t = df_row_tail<DEG>(row, ydf);
  return fma(y, f64_of_float(t.hi) + f64_of_float(t.lo), __ldg(row64));
}

// Fn[0..L] for T < 48 - 1/32 from boys_eval's table with the Taylor rows evaluated
// mostly on the FP32 pipe: per row one FP64 add and one FP64 FMA (plus y = T_k - T
// once) instead of six FMAs; for L > 1 the exp row likewise, the downward recursion
// stays FP64.  Relative error of a row 2.2e-16 against its FP64 Horner evaluation
// (emulated over T < 48, L <= 4 and the exp rows).  T at or past the table takes
// boys_eval's asymptotic branch, and so does every T when the geometry carries no
// float-pair table (tdf null).
template <int L>
__device__ __forceinline__ void boys_eval_df(const float* __restrict__ tdf, const double* __restrict__ t64, double T,
                                             double* Fn) {
  const float Tf = f32_of_nonneg(T);
  if (tdf == nullptr || !(Tf < float(kBoysTaylorMax))) {
    boys_eval<L>(t64, T, Fn);
    return;
  }
  const int k = __float2int_rn(Tf * 16.0f);
  const double Tk = k == 0 ? 0.0 : f64_of_positive(float(k) * 0.0625f);  // k/16, exact
  const double y = Tk - T;
  const DF ydf = df_of_double(y);
  Fn[L] = df_row<6>(tdf + (L * kBoysNGrid + k) * kBoysDfRow, t64 + (L * kBoysNGrid + k) * kBoysRow, y, ydf);
  if (L == 1) {
    Fn[0] = df_row<6>(tdf + k * kBoysDfRow, t64 + k * kBoysRow, y, ydf);
  } else if (L > 1) {
    const double eT = df_row<7>(tdf + (kBoysExpOff / kBoysRow + k) * kBoysDfRow, t64 + kBoysExpOff + k * kBoysRow, y,
                                ydf);
    const double T2 = T + T;
#pragma unroll
    for (int m = L; m > 0; --m) Fn[m - 1] = fma(T2, Fn[m], eT) * (1.0 / double(2 * m - 1));
  }
}

// ---------------------------------------------------------------------------------
// per-quartet context handed to the generated class code
template <typename Real>
struct Ctx;

template <>
struct Ctx<double> {
  const Geometry* g;
  int chunk;  // ket chunk evaluated by this thread, -1 = all chunks
  mutable unsigned nasym;  // Boys evaluations on the asymptotic branch (counters)
  int bra_begin, bra_end, ket_begin, ket_end;
  long long ebra, eket;
  int nnz_ab, nnz_cd;
  double* rs;
  int rstr;

  template <typename R>
  __device__ __forceinline__ R* rsmem() const { return reinterpret_cast<R*>(rs); }
  __device__ __forceinline__ int rstride() const { return rstr; }
  __device__ __forceinline__ const double* ket_E(int j) const {
    return g->E64 + eket + (long long)(j - ket_begin) * nnz_cd;
  }
  __device__ __forceinline__ const double* bra_E(int i) const {
    return g->E64 + ebra + (long long)(i - bra_begin) * nnz_ab;
  }
  typedef double4_32a PP;
  __device__ __forceinline__ PP pp(int k) const { return g->pP[k]; }
  template <int L>
  __device__ __forceinline__ void hermite_r0(int i, int j, double* Rn, double& X, double& Y, double& Z) const {
    hermite_r0_pp<L>(g->pP[i], g->pP[j], Rn, X, Y, Z);
  }
  // R^(n)_000 = (p+q)^{-1/2} (-2 alpha)^n F_n(T), n = 0..L, T = alpha |PQ|^2, alpha =
  // pq/(p+q), and PQ = (X, Y, Z).  For L <= 4 the branch is taken before any FP64
  // work that only one side needs, on an FP32 estimate of T (FP32 and integer pipes):
  //   near (T < 48 - 1/32): 1/sqrt(p+q), alpha, T, the tabulated Boys function;
  //   far: the asymptotic F_n = (2n-1)!! sqrt(pi) / (2^{n+1} T^{n+1/2}) (the e^{-T}
  //   terms are below 5e-15 relative for n <= 4) turns R^(n) into the point-charge
  //   form R^(0) = sqrt(pi)/2 / (sqrt(pq) |PQ|), R^(n) = -(2n-1) R^(n-1) / |PQ|^2,
  //   which needs 1/sqrt(pq |PQ|^2) and no Boys function or alpha at all.
  // Both sides are one product chain, R^(n) = rr M^n B_n, with
  //   near: rr = 1/sqrt(p+q),      M = -2 pq rr^2 = -2 alpha, B_n = F_n(T);
  //   far:  rr = 1/sqrt(pq |PQ|^2), M = -pq rr^2 = -1/|PQ|^2,  B_n = (2n-1)!! sqrt(pi)/2,
  // so a warp whose lanes straddle T = 48 (most warps of the s and p classes: far
  // primitive quartets outnumber near ones about 4 to 1 in water clusters) issues the
  // reciprocal square root and the chain once, and only T and the Boys rows on the
  // near side; M's sign and factor 2 are set on the integer pipe.
  // A near lane whose FP64 T lands past the table still gets the asymptotic form
  // inside boys_eval (its own test), so the table is never read out of range.
  template <int L>
  __device__ __forceinline__ void hermite_r0_pp(const PP& a, const PP& b, double* Rn, double& X, double& Y,
                                                double& Z) const {
    X = a.y - b.y;
    Y = a.z - b.z;
    Z = a.w - b.w;
    const double r2 = fma(X, X, fma(Y, Y, Z * Z));
    if constexpr (L <= 4) {
      const double pq = a.x * b.x, s = a.x + b.x, pqr2 = pq * r2;
      const float Tf = __fdividef(f32_of_nonneg(pqr2), f32_of_nonneg(s));
      const bool far = Tf >= float(kBoysTaylorMax);
      const double rr = rsqrt_dd(far ? pqr2 : s);
      const double pqrr2 = pq * (rr * rr);  // near: alpha; far: 1/|PQ|^2
      double B[L + 1];
      if (far) {
        ++nasym;
        double f = kHalfSqrtPi;
#pragma unroll
        for (int n = 0; n <= L; ++n) {
          B[n] = f;
          f *= double(2 * n + 1);  // compile-time constants
        }
      } else {
        boys_eval_df<L>(g->boysdf, g->boys64, pqrr2 * r2, B);
      }
      double c = rr;  // 2 pi^{5/2} is folded into the E' coefficients
      Rn[0] = c * B[0];
      if (L > 0) {
        const unsigned hm = ((unsigned)__double2hiint(pqrr2) ^ 0x80000000u) + (far ? 0u : 0x00100000u);
        const double M = __hiloint2double((int)hm, __double2loint(pqrr2));
#pragma unroll
        for (int n = 1; n <= L; ++n) {
          c *= M;
          Rn[n] = c * B[n];
        }
      }
      return;
    }
    const double rsum = rsqrt_dd(a.x + b.x);
    const double alpha = a.x * b.x * (rsum * rsum);
    double F[L + 1];
    const double T = alpha * r2;
    nasym += f32_of_nonneg(T) >= float(kBoysTaylorMax) ? 1u : 0u;
    boys_eval<L>(g->boys64, T, F);
    double c = rsum;  // 2 pi^{5/2} is folded into the E' coefficients
    const double m2a = -2.0 * alpha;
#pragma unroll
    for (int n = 0; n <= L; ++n) {
      Rn[n] = c * F[n];
      c *= m2a;
    }
  }
};

template <>
struct Ctx<float> {
  const Geometry* g;
  int chunk;
  mutable unsigned nasym;
  int bra_begin, bra_end, ket_begin, ket_end;
  long long ebra, eket;
  int nnz_ab, nnz_cd;
  float* rs;
  int rstr;

  template <typename R>
  __device__ __forceinline__ R* rsmem() const { return reinterpret_cast<R*>(rs); }
  __device__ __forceinline__ int rstride() const { return rstr; }
  __device__ __forceinline__ const float* ket_E(int j) const {
    return g->E32 + eket + (long long)(j - ket_begin) * nnz_cd;
  }
  __device__ __forceinline__ const float* bra_E(int i) const {
    return g->E32 + ebra + (long long)(i - bra_begin) * nnz_ab;
  }
  struct PP {
    float4 hi;  // (p, P) rounded to FP32
    float4 lo;  // (0, P - hi): P as an unevaluated float pair
  };
  __device__ __forceinline__ PP pp(int k) const { return PP{g->pPf[2 * k], g->pPf[2 * k + 1]}; }
  template <int L>
  __device__ __forceinline__ void hermite_r0(int i, int j, float* Rn, float& X, float& Y, float& Z) const {
    hermite_r0_pp<L>(pp(i), pp(j), Rn, X, Y, Z);
  }
  template <int L>
  __device__ __forceinline__ void hermite_r0_pp(const PP& a, const PP& b, float* Rn, float& X, float& Y,
                                                float& Z) const {
    // P - Q from float pairs (hi + lo): the difference keeps FP32 relative precision
    // even for nearby centres ~10 bohr from the origin, without any FP64 instruction
    X = (a.hi.y - b.hi.y) + (a.lo.y - b.lo.y);
    Y = (a.hi.z - b.hi.z) + (a.lo.z - b.lo.z);
    Z = (a.hi.w - b.hi.w) + (a.lo.w - b.lo.w);
    const float r2 = fmaf(X, X, fmaf(Y, Y, Z * Z));
    const float pa = a.hi.x, pb = b.hi.x;
    const float rsum = rsqrtf(pa + pb);
    const float alpha = pa * pb * (rsum * rsum);
    float F[L + 1];
    const float T = alpha * r2;
    nasym += T >= float(kBoysTaylorMax) ? 1u : 0u;
    boys_eval<L>(g->boys32, T, F);
    float c = rsum;  // 2 pi^{5/2} is folded into the E' coefficients
    const float m2a = -2.0f * alpha;
#pragma unroll
    for (int n = 0; n <= L; ++n) {
      Rn[n] = c * F[n];
      c *= m2a;
    }
  }
};

// ---------------------------------------------------------------------------------
// shell-quartet description shared by the digests
struct QuartetInfo {
  int sa, sb, sc, sd;        // shells (bra pair a>=b in L, ket pair c>=d in L)
  bool same_ab, same_cd, same_pair;
  int mol;
};

__device__ __forceinline__ int tri(int i) { return i * (i + 1) / 2; }

// |x| of a double as a float rounded toward zero, from its bit pattern on the integer
// pipe (no FP64 instruction): exponent rebiased, top 23 mantissa bits kept; values
// below the normal float range give 0.  Relative error below 2^-23, far inside the
// screening test's guard band.
__device__ __forceinline__ float abs_f32_trunc(double x) {
  const int hi = __double2hiint(x) & 0x7fffffff;
  const unsigned lo = (unsigned)__double2loint(x);
  const int fe = min((hi >> 20) - (1023 - 127), 254);
  const int m = ((hi & 0xfffff) << 3) | (int)(lo >> 29);
  return fe <= 0 ? 0.0f : __int_as_float((fe << 23) | m);
}

// Fock (formPT) digest --------------------------------------------------------------
// per-class counters of a Fock build: [0] digested function quartets, [1] shell
// quartets, [2] primitive quartets, [3] bra-primitive passes (bra transforms),
// [4] primitive quartets whose Boys function took the asymptotic branch (T >= 48)
constexpr int kCounters = 5;

struct FockArgs {
  const double* dP;      // packed per-molecule N x N (density difference)
  const float* dPf;      // FP32 copy of |dP| for screening
  double* G;             // packed per-molecule N x N, accumulated (unsymmetrised)
  const double* sq;      // sqrt(screen) per molecule-local function pair, packed N(N+1)/2
  const float* sqf;      // FP32 copy
  const float* Dsh;      // per-molecule S x S shell-block max |dP|
  double tol;
  float tolf_lo, tolf_hi;  // FP32 guard band around tol
  unsigned long long* counters;  // per class, kCounters entries (see kCounters)
  // sharded build (mmdg_set_partition): a shell quartet is kept only if the owner of
  // its pair with the larger canonical index is `part` (pair_owner null: no sharding)
  const int* pair_owner;  // per shell pair
  const int* pair_canon;  // canonical index s1(s1+1)/2 + s2 of every shell pair (per molecule)
  int part;
  // per launch: the next unclaimed work item of the launch's list (zeroed before every
  // build); warps claim items from it, so the SMs that draw cheap quartets draw more
  unsigned long long* work;
};

template <int NB, int ND>
struct FockDigest {
  const Geometry& g;
  const FockArgs& f;
  QuartetInfo q;
  long long base;
  long long tbase;
  int N;
  unsigned int nfq;

  __device__ __forceinline__ FockDigest(const Geometry& g_, const FockArgs& f_, const QuartetInfo& q_)
      : g(g_), f(f_), q(q_), nfq(0) {
    base = g.mol_base[q.mol];
    tbase = g.mol_tbase[q.mol];
    N = g.mol_n[q.mol];
  }

  template <typename Real>
  __device__ __forceinline__ void put(int ca, int cb, int cc, int cd, Real vr) {
    if (q.same_ab && ca < cb) return;
    if (q.same_cd && cc < cd) return;
    if (q.same_pair && (ca * NB + cb) < (cc * ND + cd)) return;
    int i = __ldg(g.func + q.sa * kMaxComp + ca);
    int j = __ldg(g.func + q.sb * kMaxComp + cb);
    int k = __ldg(g.func + q.sc * kMaxComp + cc);
    int l = __ldg(g.func + q.sd * kMaxComp + cd);
    if ((i | j | k | l) < 0) return;
    if (i < j) { int t = i; i = j; j = t; }
    if (k < l) { int t = k; k = l; l = t; }
    int ij = tri(i) + j, kl = tri(k) + l;
    if (ij < kl) {
      int t = i; i = k; k = t;
      t = j; j = l; l = t;
      t = ij; ij = kl; kl = t;
    }
    const long long rI = base + (long long)i * N, rJ = base + (long long)j * N;
    const long long rK = base + (long long)k * N;
    // the six density elements, loaded once for the screening test and the scatter
    const double* dP = f.dP;
    const double d_ij = __ldg(dP + rI + j), d_kl = __ldg(dP + rK + l), d_ik = __ldg(dP + rI + k);
    const double d_il = __ldg(dP + rI + l), d_jk = __ldg(dP + rJ + k), d_jl = __ldg(dP + rJ + l);
    // screening: sqrt(screen[ij]) sqrt(screen[kl]) max(4|dP_ij|,4|dP_kl|,|dP_ik|,|dP_il|,|dP_jk|,|dP_jl|) < tol
    {
      float dm = fmaxf(4.0f * fmaxf(abs_f32_trunc(d_ij), abs_f32_trunc(d_kl)),
                       fmaxf(fmaxf(abs_f32_trunc(d_ik), abs_f32_trunc(d_il)),
                             fmaxf(abs_f32_trunc(d_jk), abs_f32_trunc(d_jl))));
      const float bf = __ldg(f.sqf + tbase + ij) * __ldg(f.sqf + tbase + kl) * dm;
      if (bf < f.tolf_lo) return;
      if (bf < f.tolf_hi) {  // near the threshold: the reference's test in FP64
        double d = fmax(4.0 * fmax(fabs(d_ij), fabs(d_kl)),
                        fmax(fmax(fabs(d_ik), fabs(d_il)), fmax(fabs(d_jk), fabs(d_jl))));
        if (f.sq[tbase + ij] * f.sq[tbase + kl] * d < f.tol) return;
      }
    }
    // degeneracy s12 * s34 * s12_34 in {1,2,4,8} (fock.pyx:60-70) and the exchange
    // weight -1/4 are powers of two: applied exactly on the exponent field (integer
    // pipe) instead of FP64 multiplies.  Values whose exponent field is below 64
    // (|v| < 1e-289, zeros included) contribute nothing at double precision.
    const long long bits = __double_as_longlong(double(vr));
    if (((bits >> 52) & 0x7ff) < 64) { ++nfq; return; }
    const long long deg = (long long)((i != j) + (k != l) + !(i == k && j == l));
    const double v = __longlong_as_double(bits + (deg << 52));
    const double vq = __longlong_as_double((bits + ((deg - 2) << 52)) ^ (long long)0x8000000000000000ULL);
    double* G = f.G;
    atomicAdd(G + rI + j, d_kl * v);
    atomicAdd(G + rK + l, d_ij * v);
    atomicAdd(G + rI + k, d_jl * vq);
    atomicAdd(G + rJ + l, d_ik * vq);
    atomicAdd(G + rI + l, d_jk * vq);
    atomicAdd(G + rK + j, d_il * vq);
    ++nfq;
  }
};

// ERI tensor digest (doERIs, twoe.pyx:12-31): the eight symmetric copies -----------
struct TensorArgs {
  double* out;  // N^4 of molecule 0
};

template <int NB, int ND>
struct TensorDigest {
  const Geometry& g;
  const TensorArgs& t;
  QuartetInfo q;
  long long N;
  __device__ __forceinline__ TensorDigest(const Geometry& g_, const TensorArgs& t_, const QuartetInfo& q_)
      : g(g_), t(t_), q(q_) {
    N = g.mol_n[q.mol];
  }
  template <typename Real>
  __device__ __forceinline__ void put(int ca, int cb, int cc, int cd, Real vr) {
    if (q.same_ab && ca < cb) return;
    if (q.same_cd && cc < cd) return;
    if (q.same_pair && (ca * NB + cb) < (cc * ND + cd)) return;
    const long long i = __ldg(g.func + q.sa * kMaxComp + ca);
    const long long j = __ldg(g.func + q.sb * kMaxComp + cb);
    const long long k = __ldg(g.func + q.sc * kMaxComp + cc);
    const long long l = __ldg(g.func + q.sd * kMaxComp + cd);
    if ((i | j | k | l) < 0) return;
    const double v = double(vr);
    double* o = t.out;
    o[((i * N + j) * N + k) * N + l] = v;
    o[((k * N + l) * N + i) * N + j] = v;
    o[((j * N + i) * N + l) * N + k] = v;
    o[((l * N + k) * N + j) * N + i] = v;
    o[((j * N + i) * N + k) * N + l] = v;
    o[((l * N + k) * N + i) * N + j] = v;
    o[((i * N + j) * N + l) * N + k] = v;
    o[((k * N + l) * N + j) * N + i] = v;
  }
};

// Listed shell quartets (mmdg_eri_quartets; the reference's ERI(a, b, c, d),
// twoe.pyx:36-50, on whole shells): every component of the caller's (ab|cd) in the
// caller's shell order, at out[q*1296 + ((ca*6+cb)*6+cc)*6+cd] -----------------------
constexpr int kQuartetBlock = kMaxComp * kMaxComp * kMaxComp * kMaxComp;

struct QuartetArgs {
  double* out;  // n * kQuartetBlock
};

// one listed quartet: canonical bra / ket shell pair, output slot, orientation flags
//   bit 0: the caller's first pair is the canonical ket
//   bit 1: the caller's first pair lists the canonical second shell first
//   bit 2: the same for the caller's second pair
struct QuartetItem {
  int bra, ket, slot, flags;
};

template <int NB, int ND>
struct QuartetDigest {
  const QuartetArgs& a;
  long long base;
  int flags;
  __device__ __forceinline__ QuartetDigest(const QuartetArgs& a_, int slot, int flags_)
      : a(a_), base((long long)slot * kQuartetBlock), flags(flags_) {}
  template <typename Real>
  __device__ __forceinline__ void put(int ca, int cb, int cc, int cd, Real vr) {
    int b0 = ca, b1 = cb, k0 = cc, k1 = cd;
    int u0, u1, u2, u3;
    if (flags & 1) {
      u0 = (flags & 2) ? k1 : k0;
      u1 = (flags & 2) ? k0 : k1;
      u2 = (flags & 4) ? b1 : b0;
      u3 = (flags & 4) ? b0 : b1;
    } else {
      u0 = (flags & 2) ? b1 : b0;
      u1 = (flags & 2) ? b0 : b1;
      u2 = (flags & 4) ? k1 : k0;
      u3 = (flags & 4) ? k0 : k1;
    }
    a.out[base + ((u0 * kMaxComp + u1) * kMaxComp + u2) * kMaxComp + u3] = double(vr);
  }
};

// Schwarz digest (Molecule.build screen dict, molecule.py:95-99) ---------------------
struct SchwarzArgs {
  double* screen;  // packed per-molecule N(N+1)/2: (ij|ij)
  float* Qpair;    // per shell pair: max sqrt((ij|ij)), written via atomicMax on the bits
  int prim;        // primitive mode: every "pair" is one primitive pair; only Qpair is
                   // written, over all diagonal component pairs, from an FP64 square root
};

template <int NB, int ND>
struct SchwarzDigest {
  const Geometry& g;
  const SchwarzArgs& s;
  QuartetInfo q;
  int pair;
  long long tbase;
  __device__ __forceinline__ SchwarzDigest(const Geometry& g_, const SchwarzArgs& s_, const QuartetInfo& q_, int pair_)
      : g(g_), s(s_), q(q_), pair(pair_) {
    tbase = g.mol_tbase[q.mol];
  }
  template <typename Real>
  __device__ __forceinline__ void put(int ca, int cb, int cc, int cd, Real vr) {
    if (ca != cc || cb != cd) return;
    if (!s.prim && q.same_ab && ca < cb) return;
    int i = __ldg(g.func + q.sa * kMaxComp + ca);
    int j = __ldg(g.func + q.sb * kMaxComp + cb);
    if ((i | j) < 0) return;
    if (i < j) { int t = i; i = j; j = t; }
    const double v = double(vr);
    if (s.prim) {
      const float r = float(sqrt(fmax(v, 0.0)));
      atomicMax(reinterpret_cast<int*>(s.Qpair + pair), __float_as_int(r));
      return;
    }
    s.screen[tbase + tri(i) + j] = v;
    const float r = sqrtf(fmaxf(float(v), 0.0f));
    atomicMax(reinterpret_cast<int*>(s.Qpair + pair), __float_as_int(r));
  }
};

}  // namespace mmdg
