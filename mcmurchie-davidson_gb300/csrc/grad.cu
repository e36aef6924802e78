// grad.cu -- analytic RHF nuclear gradient on the GPU.
//
// dE/dR_A = 2 sum_ij P_ij dH_ij/dR_A - 2 sum_ij W_ij dS_ij/dR_A
//         + sum_ijkl (2 P_ij P_kl - P_ik P_jl) d(ij|kl)/dR_A + dV_nn/dR_A
// with W = P F P, the reference's expression (mmd/forces.py:61-97, P = C_occ C_occ^T),
// evaluated without ever forming a derivative-integral tensor: a thread computes the
// derivative integrals of one shell pair and nucleus (one-electron terms), a warp those
// of one unique shell quartet (two-electron terms), and both contract them at once
// with the densities.
//
// Derivatives of a Cartesian Gaussian with respect to its centre (cython/grad.pyx:
// 101-108): d/dA_x G_i = 2a G_{i+1} - i G_{i-1}, so the Hermite coefficients of a
// differentiated product are 2a E^{i+1,j}_t - i E^{i-1,j}_t (centre A) or
// 2b E^{i,j+1}_t - j E^{i,j-1}_t (centre B).  Translational invariance gives the
// remaining centre: d/dD = -(d/dA + d/dB + d/dC) for a quartet, d/dB = -d/dA for the
// overlap and kinetic integrals, and d/dC = -(d/dA + d/dB) for the attraction of
// nucleus C (its Hellmann-Feynman term).
//
// These kernels are generic (runtime loops over angular momenta, s..d shells, total
// angular momentum up to 9), one launch each per gradient; the Boys function comes from its
// defining series (downward recursion) below T = 35 and from upward recursion off
// F_0 = sqrt(pi/T)/2 erf(sqrt T) above.
#include <cuda_runtime.h>
#include <math.h>

#include "grad.cuh"

namespace {

constexpr int kLmaxShell = 2;                 // d shells
constexpr int kEi = kLmaxShell + 2;           // i (or j) up to l + 1 (ERI) / l + 2 (kinetic)
constexpr int kEj = kLmaxShell + 3;
constexpr int kEt = 2 * kLmaxShell + 4;       // t up to i + j
constexpr int kLtot = 4 * kLmaxShell + 1;     // total angular momentum of a differentiated quartet
constexpr int kRsize = (kLtot + 1) * (kLtot + 2) * (kLtot + 3) / 6;
constexpr double kPi = 3.14159265358979323846;

__device__ __forceinline__ double comp_norm(int l) { return l >= 2 ? 0.57735026918962576 : 1.0; }

// Cartesian exponents of component c of a shell of angular momentum L (the order of
// mmd/molecule.py:104-115: x^L first, then decreasing x, then decreasing y)
__device__ __forceinline__ void lmn_of(int L, int c, int& l, int& m, int& n) {
  int k = 0;
  for (int x = L; x >= 0; --x)
    for (int y = L - x; y >= 0; --y) {
      if (k == c) {
        l = x;
        m = y;
        n = L - x - y;
        return;
      }
      ++k;
    }
  l = m = n = 0;
}

// 1D Hermite expansion coefficients E[i][j][t] of G_i(x; a, A) G_j(x; b, B) for
// i <= imax, j <= jmax (cython/util.pxi:13-28 recursion; the Gaussian factor is
// applied by the caller)
struct E1 {
  double v[kEi][kEj][kEt];
};

__device__ void hermite_1d(E1& E, int imax, int jmax, double p, double XPA, double XPB) {
  const double i2p = 0.5 / p;
  for (int i = 0; i <= imax; ++i)
    for (int j = 0; j <= jmax; ++j)
      for (int t = 0; t < kEt; ++t) E.v[i][j][t] = 0.0;
  E.v[0][0][0] = 1.0;
  for (int i = 0; i < imax; ++i)
    for (int t = 0; t <= i + 1; ++t) {
      double v = XPA * E.v[i][0][t];
      if (t > 0) v += i2p * E.v[i][0][t - 1];
      if (t + 1 <= i) v += (t + 1) * E.v[i][0][t + 1];
      E.v[i + 1][0][t] = v;
    }
  for (int j = 0; j < jmax; ++j)
    for (int i = 0; i <= imax; ++i)
      for (int t = 0; t <= i + j + 1 && t < kEt; ++t) {
        double v = XPB * E.v[i][j][t];
        if (t > 0) v += i2p * E.v[i][j][t - 1];
        if (t + 1 <= i + j) v += (t + 1) * E.v[i][j][t + 1];
        E.v[i][j + 1][t] = v;
      }
}

// F_m(T), m = 0..M (M <= kLtot + 1)
__device__ void boys_series(int M, double T, double* F) {
  const double e = exp(-T);
  if (T < 35.0) {
    double term = 1.0 / (2 * M + 1), sum = term;
    for (int i = 0; i < 400; ++i) {
      term *= 2.0 * T / (2 * M + 2 * i + 3);
      sum += term;
      if (term < 1e-17 * sum) break;
    }
    F[M] = e * sum;
    for (int m = M; m > 0; --m) F[m - 1] = (2.0 * T * F[m] + e) / (2 * m - 1);
  } else {
    const double st = sqrt(T);
    F[0] = 0.5 * sqrt(kPi) / st * erf(st);
    for (int m = 0; m < M; ++m) F[m + 1] = ((2 * m + 1) * F[m] - e) / (2.0 * T);
  }
}

// packed Hermite index of (t, u, v): order k = t+u+v, then s = u+v, then v
__device__ __forceinline__ int ridx(int t, int u, int v) {
  const int k = t + u + v, s = u + v;
  return k * (k + 1) * (k + 2) / 6 + s * (s + 1) / 2 + v;
}

// R_{tuv}(alpha, X, Y, Z) for t+u+v <= M in place (cython/util.pxi:33-50 recursion,
// run downward in the auxiliary index n over a single buffer)
__device__ void hermite_r(int M, double alpha, double X, double Y, double Z, const double* F, double* R) {
  double f = 1.0;
  for (int n = M; n >= 0; --n) {
    // orders M-n .. 1 of level n from level n+1 (descending order keeps inputs intact)
    for (int k = M - n; k >= 1; --k)
      for (int t = k; t >= 0; --t)
        for (int u = k - t; u >= 0; --u) {
          const int v = k - t - u;
          double r;
          if (t > 0) {
            r = X * R[ridx(t - 1, u, v)];
            if (t > 1) r += (t - 1) * R[ridx(t - 2, u, v)];
          } else if (u > 0) {
            r = Y * R[ridx(t, u - 1, v)];
            if (u > 1) r += (u - 1) * R[ridx(t, u - 2, v)];
          } else {
            r = Z * R[ridx(t, u, v - 1)];
            if (v > 1) r += (v - 1) * R[ridx(t, u, v - 2)];
          }
          R[ridx(t, u, v)] = r;
        }
    f = 1.0;
    for (int i = 0; i < n; ++i) f *= -2.0 * alpha;
    R[0] = f * F[n];
  }
}

// ------------------------------------------------------------------ one-electron terms
// One thread per (shell pair, nucleus): the nucleus' attraction terms, and for
// nucleus 0 also the overlap and kinetic terms of the pair.
__global__ void k_grad_one(GradArgs a) {
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (tid >= (long long)a.npair * a.natom) return;
  const int pr = (int)(tid / a.natom), cnuc = (int)(tid - (long long)pr * a.natom);
  const int sa = a.pa[pr], sb = a.pb[pr];
  const int la = a.L[sa], lb = a.L[sb];
  const int Ka = a.nprim[sa], Kb = a.nprim[sb];
  const int atA = a.shell_atom[sa], atB = a.shell_atom[sb];
  const double A[3] = {a.center[3 * sa], a.center[3 * sa + 1], a.center[3 * sa + 2]};
  const double B[3] = {a.center[3 * sb], a.center[3 * sb + 1], a.center[3 * sb + 2]};
  const double fac = sa == sb ? 1.0 : 2.0;  // (i, j) and (j, i) of two different shells
  const int nca = (la + 1) * (la + 2) / 2, ncb = (lb + 1) * (lb + 2) / 2;
  double gA[3] = {0, 0, 0};
  E1 E[3];
  double R[kRsize], F[kLtot + 2];
  // ---- overlap and kinetic: d/dB = -d/dA
  for (int ka = 0; ka < (cnuc == 0 ? Ka : 0); ++ka)
    for (int kb = 0; kb < Kb; ++kb) {
      const double ea = a.exps[a.poff[sa] + ka], eb = a.exps[a.poff[sb] + kb];
      const double p = ea + eb, mu = ea * eb / p;
      double AB2 = 0.0;
      for (int d = 0; d < 3; ++d) AB2 += (A[d] - B[d]) * (A[d] - B[d]);
      const double K = exp(-mu * AB2) * a.coefs[a.poff[sa] + ka] * a.coefs[a.poff[sb] + kb];
      const double sq = sqrt(kPi / p);
      for (int d = 0; d < 3; ++d)
        hermite_1d(E[d], la + 1, lb + 2, p, -(eb / p) * (A[d] - B[d]), (ea / p) * (A[d] - B[d]));
      for (int ca = 0; ca < nca; ++ca) {
        const int fi = a.func[sa * kGradMaxComp + ca];
        if (fi < 0) continue;
        int ia[3];
        lmn_of(la, ca, ia[0], ia[1], ia[2]);
        for (int cb = 0; cb < ncb; ++cb) {
          const int fj = a.func[sb * kGradMaxComp + cb];
          if (fj < 0) continue;
          int jb[3];
          lmn_of(lb, cb, jb[0], jb[1], jb[2]);
          const double nrm = comp_norm(ia[0]) * comp_norm(ia[1]) * comp_norm(ia[2]) * comp_norm(jb[0]) *
                             comp_norm(jb[1]) * comp_norm(jb[2]);
          const double Pij = a.P[(long long)fi * a.N + fj], Wij = a.W[(long long)fi * a.N + fj];
          // 1D overlap S(i, j) and kinetic T(i, j) (cython/onee.pyx:103-133 decomposition)
          auto S1 = [&](int d, int i, int j) { return (i < 0 || j < 0) ? 0.0 : E[d].v[i][j][0] * sq; };
          auto T1 = [&](int d, int i, int j) {
            if (i < 0) return 0.0;
            double t = eb * (2 * j + 1) * S1(d, i, j) - 2.0 * eb * eb * S1(d, i, j + 2);
            if (j >= 2) t -= 0.5 * j * (j - 1) * S1(d, i, j - 2);
            return t;
          };
          for (int d = 0; d < 3; ++d) {
            // derivative in direction d of the bra: 2a f(i+1) - i f(i-1)
            double dS = 1.0, dT = 0.0;
            double Sd[3], Td[3];
            for (int e = 0; e < 3; ++e) {
              if (e == d) {
                Sd[e] = 2.0 * ea * S1(e, ia[e] + 1, jb[e]) - ia[e] * S1(e, ia[e] - 1, jb[e]);
                Td[e] = 2.0 * ea * T1(e, ia[e] + 1, jb[e]) - ia[e] * T1(e, ia[e] - 1, jb[e]);
              } else {
                Sd[e] = S1(e, ia[e], jb[e]);
                Td[e] = T1(e, ia[e], jb[e]);
              }
            }
            dS = Sd[0] * Sd[1] * Sd[2];
            dT = Td[0] * Sd[1] * Sd[2] + Sd[0] * Td[1] * Sd[2] + Sd[0] * Sd[1] * Td[2];
            gA[d] += fac * K * nrm * (2.0 * Pij * dT - 2.0 * Wij * dS);
          }
        }
      }
    }
  if (cnuc == 0)
    for (int d = 0; d < 3; ++d) {
      atomicAdd(a.grad + 3 * atA + d, gA[d]);
      atomicAdd(a.grad + 3 * atB + d, -gA[d]);
    }
  // ---- nuclear attraction of this thread's nucleus: basis terms on A and B, and the
  // Hellmann-Feynman term on the nucleus, -(A + B)
  {
    const int c = cnuc;
    const double C[3] = {a.xyz[3 * c], a.xyz[3 * c + 1], a.xyz[3 * c + 2]};
    const double Zc = a.Z[c];
    double vA[3] = {0, 0, 0}, vB[3] = {0, 0, 0};
    for (int ka = 0; ka < Ka; ++ka)
      for (int kb = 0; kb < Kb; ++kb) {
        const double ea = a.exps[a.poff[sa] + ka], eb = a.exps[a.poff[sb] + kb];
        const double p = ea + eb, mu = ea * eb / p;
        double AB2 = 0.0, P[3];
        for (int d = 0; d < 3; ++d) {
          AB2 += (A[d] - B[d]) * (A[d] - B[d]);
          P[d] = (ea * A[d] + eb * B[d]) / p;
        }
        const double K = exp(-mu * AB2) * a.coefs[a.poff[sa] + ka] * a.coefs[a.poff[sb] + kb];
        for (int d = 0; d < 3; ++d)
          hermite_1d(E[d], la + 1, lb + 1, p, -(eb / p) * (A[d] - B[d]), (ea / p) * (A[d] - B[d]));
        const int M = la + lb + 1;
        const double X = P[0] - C[0], Y = P[1] - C[1], Z = P[2] - C[2];
        boys_series(M, p * (X * X + Y * Y + Z * Z), F);
        hermite_r(M, p, X, Y, Z, F, R);
        const double pref = -Zc * 2.0 * kPi / p * K;
        for (int ca = 0; ca < nca; ++ca) {
          const int fi = a.func[sa * kGradMaxComp + ca];
          if (fi < 0) continue;
          int ia[3];
          lmn_of(la, ca, ia[0], ia[1], ia[2]);
          for (int cb = 0; cb < ncb; ++cb) {
            const int fj = a.func[sb * kGradMaxComp + cb];
            if (fj < 0) continue;
            int jb[3];
            lmn_of(lb, cb, jb[0], jb[1], jb[2]);
            const double nrm = comp_norm(ia[0]) * comp_norm(ia[1]) * comp_norm(ia[2]) * comp_norm(jb[0]) *
                               comp_norm(jb[1]) * comp_norm(jb[2]);
            const double w = fac * 2.0 * a.P[(long long)fi * a.N + fj] * pref * nrm;
            // V(i, j) with one index of one dimension shifted by s = +-1 on centre A or B
            auto V = [&](int d, int ia_d, int jb_d) {
              if (ia_d < 0 || jb_d < 0) return 0.0;
              int ii[3] = {ia[0], ia[1], ia[2]}, jj[3] = {jb[0], jb[1], jb[2]};
              ii[d] = ia_d;
              jj[d] = jb_d;
              double s = 0.0;
              for (int t = 0; t <= ii[0] + jj[0]; ++t)
                for (int u = 0; u <= ii[1] + jj[1]; ++u)
                  for (int v = 0; v <= ii[2] + jj[2]; ++v)
                    s += E[0].v[ii[0]][jj[0]][t] * E[1].v[ii[1]][jj[1]][u] * E[2].v[ii[2]][jj[2]][v] *
                         R[ridx(t, u, v)];
              return s;
            };
            for (int d = 0; d < 3; ++d) {
              vA[d] += w * (2.0 * ea * V(d, ia[d] + 1, jb[d]) - ia[d] * V(d, ia[d] - 1, jb[d]));
              vB[d] += w * (2.0 * eb * V(d, ia[d], jb[d] + 1) - jb[d] * V(d, ia[d], jb[d] - 1));
            }
          }
        }
      }
    for (int d = 0; d < 3; ++d) {
      atomicAdd(a.grad + 3 * atA + d, vA[d]);
      atomicAdd(a.grad + 3 * atB + d, vB[d]);
      atomicAdd(a.grad + 3 * c + d, -(vA[d] + vB[d]));
    }
  }
}

// ------------------------------------------------------------------ two-electron terms
// A warp per unique shell quartet (bra pair ip >= ket pair iq).  Every unique function
// quartet counts once, with the degeneracy of cython/fock.pyx:60-70 and the density
// factor 2 P_ij P_kl - (P_ik P_jl + P_il P_jk) / 2 (the exchange term averaged over the
// quartet's permutations); the warp keeps those weights in shared memory.  Per
// primitive quartet the lanes share two transforms of the Hermite integrals R:
//   W[cd][tuv]   = sum_{tau nu phi} E^cd (-1)^(tau+nu+phi) R[t+tau, u+nu, v+phi],
//                  t+u+v up to the bra's L + 1 (one per ket component pair), and
//   V[ab][tau..] = sum_{tuv} E^ab R[t+tau, u+nu, v+phi],
//                  tau+nu+phi up to the ket's L + 1 (one per bra component pair);
// the derivatives on the bra centres are then short sums of differentiated bra
// coefficients against W, those on centre c of differentiated ket coefficients
// against V, and centre d follows from translational invariance.
constexpr int kGradWarps = 2;                          // warps per block
constexpr int kHmax = (2 * kLmaxShell + 2) * (2 * kLmaxShell + 3) * (2 * kLmaxShell + 4) / 6;  // H(2l+1)
constexpr int kNab = 36;                               // component pairs of a d-d pair
constexpr int kGradSmemPerWarp = 2 * kNab * kHmax + kNab * kNab;  // W, V, weights (doubles)

__device__ __forceinline__ int hcount(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }

__global__ void __launch_bounds__(32 * kGradWarps) k_grad_two(GradArgs a) {
  extern __shared__ double gsm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* Ws = gsm + warp * kGradSmemPerWarp;
  double* Vs = Ws + kNab * kHmax;
  double* Gam = Vs + kNab * kHmax;
  const long long q = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nq = (long long)a.npair * (a.npair + 1) / 2;
  if (q >= nq) return;  // whole warps leave together (blockDim is a multiple of 32)
  // (ip, iq) from the triangular index q = ip (ip + 1) / 2 + iq
  int ip = (int)((sqrt(8.0 * (double)q + 1.0) - 1.0) * 0.5);
  while ((long long)ip * (ip + 1) / 2 > q) --ip;
  while ((long long)(ip + 1) * (ip + 2) / 2 <= q) ++ip;
  const int iq = (int)(q - (long long)ip * (ip + 1) / 2);
  if (a.Qpair && (double)a.Qpair[ip] * (double)a.Qpair[iq] < a.qtol) return;
  const int s[4] = {a.pa[ip], a.pb[ip], a.pa[iq], a.pb[iq]};
  int Ls[4], nc[4];
  for (int k = 0; k < 4; ++k) {
    Ls[k] = a.L[s[k]];
    nc[k] = (Ls[k] + 1) * (Ls[k] + 2) / 2;
  }
  const int nab = nc[0] * nc[1], ncd = nc[2] * nc[3];
  const int Lp = Ls[0] + Ls[1], Lq = Ls[2] + Ls[3], M = Lp + Lq + 1;
  const int HW = hcount(Lp + 1), HV = hcount(Lq + 1);
  const bool same_ab = s[0] == s[1], same_cd = s[2] == s[3], same_pair = ip == iq;
  const int N = a.N;
  // ---- density weights of the unique function quartets (0: not counted here)
  for (int fq = lane; fq < nab * ncd; fq += 32) {
    const int cab = fq / ncd, ccd = fq - cab * ncd;
    const int ca = cab / nc[1], cb = cab - ca * nc[1], cc = ccd / nc[3], cd = ccd - cc * nc[3];
    double w = 0.0;
    int i = a.func[s[0] * kGradMaxComp + ca], j = a.func[s[1] * kGradMaxComp + cb];
    int k = a.func[s[2] * kGradMaxComp + cc], l = a.func[s[3] * kGradMaxComp + cd];
    const bool skip = (same_ab && ca < cb) || (same_cd && cc < cd) || (same_pair && cab < ccd) || i < 0 || j < 0 ||
                      k < 0 || l < 0;
    if (!skip) {
      if (i < j) { int t = i; i = j; j = t; }
      if (k < l) { int t = k; k = l; l = t; }
      const int ij = i * (i + 1) / 2 + j, kl = k * (k + 1) / 2 + l;
      if (ij < kl) {
        int t = i; i = k; k = t;
        t = j; j = l; l = t;
      }
      const double deg = (i != j ? 2.0 : 1.0) * (k != l ? 2.0 : 1.0) * (ij != kl ? 2.0 : 1.0);
      const double* Pm = a.P;
      const double gam = 2.0 * Pm[(long long)i * N + j] * Pm[(long long)k * N + l] -
                         0.5 * (Pm[(long long)i * N + k] * Pm[(long long)j * N + l] +
                                Pm[(long long)i * N + l] * Pm[(long long)j * N + k]);
      int l3[4][3];
      lmn_of(Ls[0], ca, l3[0][0], l3[0][1], l3[0][2]);
      lmn_of(Ls[1], cb, l3[1][0], l3[1][1], l3[1][2]);
      lmn_of(Ls[2], cc, l3[2][0], l3[2][1], l3[2][2]);
      lmn_of(Ls[3], cd, l3[3][0], l3[3][1], l3[3][2]);
      double nrm = 1.0;
      for (int x = 0; x < 4; ++x)
        for (int d = 0; d < 3; ++d) nrm *= comp_norm(l3[x][d]);
      w = deg * gam * nrm;
    }
    Gam[fq] = w;
  }
  __syncwarp();
  double Cn[4][3];
  for (int k = 0; k < 4; ++k)
    for (int d = 0; d < 3; ++d) Cn[k][d] = a.center[3 * s[k] + d];
  double g[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};  // centres a, b, c
  E1 Eb[3], Ek[3];
  double R[kRsize], F[kLtot + 2];
  for (int k0 = 0; k0 < a.nprim[s[0]]; ++k0)
    for (int k1 = 0; k1 < a.nprim[s[1]]; ++k1) {
      const double ea = a.exps[a.poff[s[0]] + k0], eb = a.exps[a.poff[s[1]] + k1];
      const double p = ea + eb;
      double AB2 = 0.0, P[3];
      for (int d = 0; d < 3; ++d) {
        AB2 += (Cn[0][d] - Cn[1][d]) * (Cn[0][d] - Cn[1][d]);
        P[d] = (ea * Cn[0][d] + eb * Cn[1][d]) / p;
      }
      const double Kab = exp(-ea * eb / p * AB2) * a.coefs[a.poff[s[0]] + k0] * a.coefs[a.poff[s[1]] + k1];
      for (int d = 0; d < 3; ++d)
        hermite_1d(Eb[d], Ls[0] + 1, Ls[1] + 1, p, -(eb / p) * (Cn[0][d] - Cn[1][d]), (ea / p) * (Cn[0][d] - Cn[1][d]));
      for (int k2 = 0; k2 < a.nprim[s[2]]; ++k2)
        for (int k3 = 0; k3 < a.nprim[s[3]]; ++k3) {
          const double ec = a.exps[a.poff[s[2]] + k2], ed = a.exps[a.poff[s[3]] + k3];
          const double qq = ec + ed;
          double CD2 = 0.0, Q[3];
          for (int d = 0; d < 3; ++d) {
            CD2 += (Cn[2][d] - Cn[3][d]) * (Cn[2][d] - Cn[3][d]);
            Q[d] = (ec * Cn[2][d] + ed * Cn[3][d]) / qq;
          }
          const double Kcd = exp(-ec * ed / qq * CD2) * a.coefs[a.poff[s[2]] + k2] * a.coefs[a.poff[s[3]] + k3];
          for (int d = 0; d < 3; ++d)
            hermite_1d(Ek[d], Ls[2] + 1, Ls[3] + 1, qq, -(ed / qq) * (Cn[2][d] - Cn[3][d]),
                       (ec / qq) * (Cn[2][d] - Cn[3][d]));
          const double alpha = p * qq / (p + qq);
          const double X = P[0] - Q[0], Y = P[1] - Q[1], Z = P[2] - Q[2];
          boys_series(M, alpha * (X * X + Y * Y + Z * Z), F);
          hermite_r(M, alpha, X, Y, Z, F, R);
          const double pref = 2.0 * pow(kPi, 2.5) / (p * qq * sqrt(p + qq)) * Kab * Kcd;
          // ---- W: one ket component pair per lane
          for (int ccd = lane; ccd < ncd; ccd += 32) {
            const int cc = ccd / nc[3], cd = ccd - cc * nc[3];
            int lc3[3], ld3[3];
            lmn_of(Ls[2], cc, lc3[0], lc3[1], lc3[2]);
            lmn_of(Ls[3], cd, ld3[0], ld3[1], ld3[2]);
            double* W = Ws + ccd * HW;
            for (int h = 0; h < HW; ++h) W[h] = 0.0;
            for (int ta = 0; ta <= lc3[0] + ld3[0]; ++ta)
              for (int nu = 0; nu <= lc3[1] + ld3[1]; ++nu)
                for (int ph = 0; ph <= lc3[2] + ld3[2]; ++ph) {
                  double e = Ek[0].v[lc3[0]][ld3[0]][ta] * Ek[1].v[lc3[1]][ld3[1]][nu] * Ek[2].v[lc3[2]][ld3[2]][ph];
                  if (e == 0.0) continue;
                  if ((ta + nu + ph) & 1) e = -e;
                  for (int t = 0; t <= Lp + 1; ++t)
                    for (int u = 0; u <= Lp + 1 - t; ++u)
                      for (int v = 0; v <= Lp + 1 - t - u; ++v)
                        W[ridx(t, u, v)] += e * R[ridx(t + ta, u + nu, v + ph)];
                }
          }
          // ---- V: one bra component pair per lane
          for (int cab = lane; cab < nab; cab += 32) {
            const int ca = cab / nc[1], cb = cab - ca * nc[1];
            int la3[3], lb3[3];
            lmn_of(Ls[0], ca, la3[0], la3[1], la3[2]);
            lmn_of(Ls[1], cb, lb3[0], lb3[1], lb3[2]);
            double* V = Vs + cab * HV;
            for (int h = 0; h < HV; ++h) V[h] = 0.0;
            for (int t = 0; t <= la3[0] + lb3[0]; ++t)
              for (int u = 0; u <= la3[1] + lb3[1]; ++u)
                for (int v = 0; v <= la3[2] + lb3[2]; ++v) {
                  const double e = Eb[0].v[la3[0]][lb3[0]][t] * Eb[1].v[la3[1]][lb3[1]][u] * Eb[2].v[la3[2]][lb3[2]][v];
                  if (e == 0.0) continue;
                  for (int ta = 0; ta <= Lq + 1; ++ta)
                    for (int nu = 0; nu <= Lq + 1 - ta; ++nu)
                      for (int ph = 0; ph <= Lq + 1 - ta - nu; ++ph)
                        V[ridx(ta, nu, ph)] += e * R[ridx(t + ta, u + nu, v + ph)];
                }
          }
          __syncwarp();
          // ---- derivatives of every function quartet
          for (int fq = lane; fq < nab * ncd; fq += 32) {
            const double wgt = Gam[fq];
            if (wgt == 0.0) continue;
            const int cab = fq / ncd, ccd = fq - cab * ncd;
            const int ca = cab / nc[1], cb = cab - ca * nc[1], cc = ccd / nc[3], cd = ccd - cc * nc[3];
            int la3[3], lb3[3], lc3[3], ld3[3];
            lmn_of(Ls[0], ca, la3[0], la3[1], la3[2]);
            lmn_of(Ls[1], cb, lb3[0], lb3[1], lb3[2]);
            lmn_of(Ls[2], cc, lc3[0], lc3[1], lc3[2]);
            lmn_of(Ls[3], cd, ld3[0], ld3[1], ld3[2]);
            const double* W = Ws + ccd * HW;
            const double* V = Vs + cab * HV;
            const double w = wgt * pref;
            for (int d = 0; d < 3; ++d) {
              // centres a and b against W (bra extent one higher along d)
              double sa_ = 0.0, sb_ = 0.0;
              const int ext[3] = {la3[0] + lb3[0] + (d == 0), la3[1] + lb3[1] + (d == 1), la3[2] + lb3[2] + (d == 2)};
              for (int t = 0; t <= ext[0]; ++t)
                for (int u = 0; u <= ext[1]; ++u)
                  for (int v = 0; v <= ext[2]; ++v) {
                    const int tt[3] = {t, u, v};
                    double ea_ = 1.0, eb_ = 1.0;
                    for (int e = 0; e < 3; ++e) {
                      if (e == d) {
                        double da = 2.0 * ea * Eb[e].v[la3[e] + 1][lb3[e]][tt[e]];
                        if (la3[e] > 0) da -= la3[e] * Eb[e].v[la3[e] - 1][lb3[e]][tt[e]];
                        double db = 2.0 * eb * Eb[e].v[la3[e]][lb3[e] + 1][tt[e]];
                        if (lb3[e] > 0) db -= lb3[e] * Eb[e].v[la3[e]][lb3[e] - 1][tt[e]];
                        ea_ *= da;
                        eb_ *= db;
                      } else {
                        const double base = Eb[e].v[la3[e]][lb3[e]][tt[e]];
                        ea_ *= base;
                        eb_ *= base;
                      }
                    }
                    const double wv = W[ridx(t, u, v)];
                    sa_ += ea_ * wv;
                    sb_ += eb_ * wv;
                  }
              // centre c against V (ket extent one higher along d)
              double sc_ = 0.0;
              const int kex[3] = {lc3[0] + ld3[0] + (d == 0), lc3[1] + ld3[1] + (d == 1), lc3[2] + ld3[2] + (d == 2)};
              for (int ta = 0; ta <= kex[0]; ++ta)
                for (int nu = 0; nu <= kex[1]; ++nu)
                  for (int ph = 0; ph <= kex[2]; ++ph) {
                    const int tk[3] = {ta, nu, ph};
                    double e = 1.0;
                    for (int x = 0; x < 3; ++x) {
                      if (x == d) {
                        double dc = 2.0 * ec * Ek[x].v[lc3[x] + 1][ld3[x]][tk[x]];
                        if (lc3[x] > 0) dc -= lc3[x] * Ek[x].v[lc3[x] - 1][ld3[x]][tk[x]];
                        e *= dc;
                      } else {
                        e *= Ek[x].v[lc3[x]][ld3[x]][tk[x]];
                      }
                    }
                    sc_ += ((ta + nu + ph) & 1 ? -e : e) * V[ridx(ta, nu, ph)];
                  }
              g[0][d] += w * sa_;
              g[1][d] += w * sb_;
              g[2][d] += w * sc_;
            }
          }
          __syncwarp();
        }
    }
  for (int x = 0; x < 3; ++x)
    for (int d = 0; d < 3; ++d)
      for (int o = 16; o > 0; o >>= 1) g[x][d] += __shfl_xor_sync(0xffffffffu, g[x][d], o);
  if (lane != 0) return;
  const int at[4] = {a.shell_atom[s[0]], a.shell_atom[s[1]], a.shell_atom[s[2]], a.shell_atom[s[3]]};
  for (int d = 0; d < 3; ++d) {
    atomicAdd(a.grad + 3 * at[0] + d, g[0][d]);
    atomicAdd(a.grad + 3 * at[1] + d, g[1][d]);
    atomicAdd(a.grad + 3 * at[2] + d, g[2][d]);
    atomicAdd(a.grad + 3 * at[3] + d, -(g[0][d] + g[1][d] + g[2][d]));
  }
}

}  // namespace

cudaError_t mmdg_launch_rhf_gradient(const GradArgs& a, cudaStream_t st) {
  if (a.npair <= 0) return cudaSuccess;
  const long long n1 = (long long)a.npair * a.natom;
  k_grad_one<<<(unsigned)((n1 + 63) / 64), 64, 0, st>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const long long nq = (long long)a.npair * (a.npair + 1) / 2;
  const size_t smem = sizeof(double) * kGradSmemPerWarp * kGradWarps;
  e = cudaFuncSetAttribute(k_grad_two, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const long long nthreads = nq * 32;
  k_grad_two<<<(unsigned)((nthreads + 32 * kGradWarps - 1) / (32 * kGradWarps)), 32 * kGradWarps, smem, st>>>(a);
  return cudaGetLastError();
}
