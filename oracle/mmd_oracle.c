/*
 * mmd_oracle.c -- CPU restatement of the reference's two-electron hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle: the parity tests, smoke() and
 * the CPU-baseline leg of bench.py call it to check results.  The product library
 * (libmmdg.so) never links, loads or calls it.
 *
 * Every function restates one routine of jjgoings/McMurchie-Davidson, cited by
 * file:line within that project.  Numerics follow the reference step for step
 * (same recursions, same loop order, same screening and degeneracy rules) so
 * that results agree to rounding.  The only piece that is not a restatement of
 * reference code is the Boys function: the reference calls SciPy's
 * ``scipy.special.cython_special.hyp1f1`` (third-party; SciPy 1.18.1 where the
 * fixtures were made, unpinned by the reference's requirements.txt:2 "scipy>=0.19.0"),
 * evaluating F_m(T) = 1F1(m+1/2; m+3/2; -T) / (2m+1)   (cython/util.pxi:54-55).
 * Here 1F1 is evaluated through Kummer's transformation
 *     1F1(a; b; -T) = exp(-T) 1F1(b-a; b; T),  b-a = 1,
 * i.e.  F_m(T) = exp(-T)/(2m+1) * sum_k T^k / ((m+3/2)(m+5/2)...(m+1/2+k)),
 * a series of positive terms (no cancellation), summed in double-double; for
 * T > 200 (and m < T/4) the asymptotic value Gamma(m+1/2) / (2 T^(m+1/2)) is
 * used, whose relative error exp(-T) T^(m+1/2)/Gamma(m+1/2) is below 1e-60 there.
 * The pins are tests/test012.py:12-69 of the reference (50 literature values)
 * and the compiled reference itself (tests/golden).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_PI 3.141592653589793238462643383279 /* cython/util.pxi:7 */

/* ---------------------------------------------------------------- Boys */
/* Double-double arithmetic (error-free transformations with fma): the series below
 * is summed to ~1e-30 relative on every host -- x86 and Arm alike (on aarch64 a
 * `long double` is software quad precision, far too slow for the bench-size checks). */
typedef struct {
  double hi, lo;
} odd;
static odd odd_two_sum(double a, double b) {
  double s = a + b, bb = s - a;
  odd r = {s, (a - (s - bb)) + (b - bb)};
  return r;
}
static odd odd_quick(double a, double b) {
  double s = a + b;
  odd r = {s, b - (s - a)};
  return r;
}
static odd odd_add(odd a, odd b) {
  odd s = odd_two_sum(a.hi, b.hi);
  s.lo += a.lo + b.lo;
  return odd_quick(s.hi, s.lo);
}
static odd odd_mul_d(odd a, double b) {
  double p = a.hi * b;
  double e = fma(a.hi, b, -p) + a.lo * b;
  return odd_quick(p, e);
}
static odd odd_div_d(odd a, double b) {
  double q1 = a.hi / b;
  odd r = odd_add(a, odd_mul_d((odd){q1, 0.0}, -b));
  double q2 = r.hi / b;
  return odd_quick(q1, q2);
}

double oracle_boys(double m, double T) {
  const double mi = floor(m);
  if (T > 200.0 && m < T / 4.0) {
    /* Gamma(m+1/2) / (2 T^(m+1/2)); for integer m, Gamma(m+1/2) = sqrt(pi) prod_{k=1..m} (k-1/2) */
    if (mi == m && m >= 0.0 && m < 200.0) {
      odd g = {1.772453850905516, -7.666586499825799e-17}; /* sqrt(pi), double-double */
      odd tp = {1.0, 0.0};
      for (int k = 1; k <= (int)m; ++k) {
        g = odd_mul_d(g, k - 0.5);
        tp = odd_mul_d(tp, T);
      }
      const double st = sqrt(T);
      return (g.hi + g.lo) / (2.0 * (tp.hi + tp.lo) * st);
    }
    return tgamma(m + 0.5) / (2.0 * pow(T, m + 0.5));
  }
  /* Kummer: F_m(T) = exp(-T)/(2m+1) * sum_k T^k / ((m+3/2)(m+5/2)...(m+1/2+k)) */
  odd term = {1.0, 0.0}, sum = {1.0, 0.0};
  const double b = m + 1.5;
  for (int k = 0; k < 100000; ++k) {
    term = odd_div_d(odd_mul_d(term, T), b + (double)k);
    sum = odd_add(sum, term);
    if (term.hi < sum.hi * 1e-20) break;  /* far below the double result's rounding */
  }
  /* exp(-T) correctly rounded to within an ulp by libm; the product and the division
   * add two roundings: ~3e-16 relative overall */
  return exp(-T) * (sum.hi + sum.lo) / (2.0 * m + 1.0);
}

/* ------------------------------------------- Hermite E (cython/util.pxi:13-28) */
double oracle_E(int i, int j, int t, double Qx, double a, double b) {
  double p = a + b;
  double u = a * b / p;
  if (t < 0 || t > i + j) return 0.0;
  if (i == 0 && j == 0 && t == 0) return exp(-u * Qx * Qx);
  if (j == 0)
    return (1.0 / (2.0 * p)) * oracle_E(i - 1, j, t - 1, Qx, a, b) - (u * Qx / a) * oracle_E(i - 1, j, t, Qx, a, b) +
           (t + 1) * oracle_E(i - 1, j, t + 1, Qx, a, b);
  return (1.0 / (2.0 * p)) * oracle_E(i, j - 1, t - 1, Qx, a, b) + (u * Qx / b) * oracle_E(i, j - 1, t, Qx, a, b) +
         (t + 1) * oracle_E(i, j - 1, t + 1, Qx, a, b);
}

/* ------------------------------------ Hermite Coulomb R (cython/util.pxi:33-50) */
double oracle_R(int t, int u, int v, int n, double p, double PCx, double PCy, double PCz, double RPC) {
  double T = p * RPC * RPC;
  double val = 0.0;
  if (t == 0 && u == 0 && v == 0) {
    val += pow(-2.0 * p, n) * oracle_boys((double)n, T);
  } else if (t == 0 && u == 0) {
    if (v > 1) val += (v - 1) * oracle_R(t, u, v - 2, n + 1, p, PCx, PCy, PCz, RPC);
    val += PCz * oracle_R(t, u, v - 1, n + 1, p, PCx, PCy, PCz, RPC);
  } else if (t == 0) {
    if (u > 1) val += (u - 1) * oracle_R(t, u - 2, v, n + 1, p, PCx, PCy, PCz, RPC);
    val += PCy * oracle_R(t, u - 1, v, n + 1, p, PCx, PCy, PCz, RPC);
  } else {
    if (t > 1) val += (t - 1) * oracle_R(t - 2, u, v, n + 1, p, PCx, PCy, PCz, RPC);
    val += PCx * oracle_R(t - 1, u, v, n + 1, p, PCx, PCy, PCz, RPC);
  }
  return val;
}

/* --------------------------- primitive ERI (cython/twoe.pyx:56-94) */
double oracle_primitive_eri(double a, const long* lmn1, const double* A, double b, const long* lmn2, const double* B,
                            double c, const long* lmn3, const double* C, double d, const long* lmn4, const double* D) {
  long l1 = lmn1[0], m1 = lmn1[1], n1 = lmn1[2];
  long l2 = lmn2[0], m2 = lmn2[1], n2 = lmn2[2];
  long l3 = lmn3[0], m3 = lmn3[1], n3 = lmn3[2];
  long l4 = lmn4[0], m4 = lmn4[1], n4 = lmn4[2];
  double p = a + b, q = c + d;
  double alpha = p * q / (p + q);
  double Px = (a * A[0] + b * B[0]) / p, Py = (a * A[1] + b * B[1]) / p, Pz = (a * A[2] + b * B[2]) / p;
  double Qx = (c * C[0] + d * D[0]) / q, Qy = (c * C[1] + d * D[1]) / q, Qz = (c * C[2] + d * D[2]) / q;
  double RPQ = sqrt(pow(Px - Qx, 2) + pow(Py - Qy, 2) + pow(Pz - Qz, 2));
  double val = 0.0;
  for (long t = 0; t < l1 + l2 + 1; ++t)
    for (long u = 0; u < m1 + m2 + 1; ++u)
      for (long v = 0; v < n1 + n2 + 1; ++v)
        for (long tau = 0; tau < l3 + l4 + 1; ++tau)
          for (long nu = 0; nu < m3 + m4 + 1; ++nu)
            for (long phi = 0; phi < n3 + n4 + 1; ++phi)
              val += oracle_E(l1, l2, t, A[0] - B[0], a, b) * oracle_E(m1, m2, u, A[1] - B[1], a, b) *
                     oracle_E(n1, n2, v, A[2] - B[2], a, b) * oracle_E(l3, l4, tau, C[0] - D[0], c, d) *
                     oracle_E(m3, m4, nu, C[1] - D[1], c, d) * oracle_E(n3, n4, phi, C[2] - D[2], c, d) *
                     pow(-1.0, (double)(tau + nu + phi)) *
                     oracle_R(t + tau, u + nu, v + phi, 0, alpha, Px - Qx, Py - Qy, Pz - Qz, RPQ);
  val *= 2.0 * pow(ORACLE_PI, 2.5) / (p * q * sqrt(p + q));
  return val;
}

/* ------------------------------------------- contracted basis (cython/basis.pxi) */
typedef struct {
  double origin[3];
  long shell[3];
  long num_exps;
  const double* exps;
  const double* coefs; /* contraction-normalised coefficients (basis.pxi:109-120) */
  const double* norm;  /* primitive norms (basis.pxi:101-105) */
} oracle_basis;

/* (2n-1)!! with the gamma-formula convention (-1)!! = 1 that the reference's
 * normalisation was written against (basis.pxi:104-110). */
static double fact2_odd(long k) { /* k = 2l-1 */
  double r = 1.0;
  for (long x = k; x > 1; x -= 2) r *= (double)x;
  return r;
}

/* Basis.normalize (cython/basis.pxi:87-120): fills norm[] and rescales coefs[] in place. */
void oracle_normalize(const long* shell, long num_exps, const double* exps, double* coefs, double* norm) {
  long l = shell[0], m = shell[1], n = shell[2];
  long L = l + m + n;
  for (long ia = 0; ia < num_exps; ++ia)
    norm[ia] = sqrt(pow(2.0, 2.0 * L + 1.5) * pow(exps[ia], L + 1.5) / fact2_odd(2 * l - 1) / fact2_odd(2 * m - 1) /
                    fact2_odd(2 * n - 1) / pow(ORACLE_PI, 1.5));
  double prefactor = pow(ORACLE_PI, 1.5) * fact2_odd(2 * l - 1) * fact2_odd(2 * m - 1) * fact2_odd(2 * n - 1) / pow(2.0, (double)L);
  double N = 0.0;
  for (long ia = 0; ia < num_exps; ++ia)
    for (long ib = 0; ib < num_exps; ++ib)
      N += norm[ia] * norm[ib] * coefs[ia] * coefs[ib] / pow(exps[ia] + exps[ib], L + 1.5);
  N *= prefactor;
  N = pow(N, -0.5);
  for (long ia = 0; ia < num_exps; ++ia) coefs[ia] *= N;
}

/* ERI over contracted functions (cython/twoe.pyx:36-50) */
double oracle_eri(const oracle_basis* a, const oracle_basis* b, const oracle_basis* c, const oracle_basis* d) {
  double eri = 0.0;
  for (long ja = 0; ja < a->num_exps; ++ja)
    for (long jb = 0; jb < b->num_exps; ++jb)
      for (long jc = 0; jc < c->num_exps; ++jc)
        for (long jd = 0; jd < d->num_exps; ++jd)
          eri += a->norm[ja] * b->norm[jb] * c->norm[jc] * d->norm[jd] * a->coefs[ja] * b->coefs[jb] *
                 c->coefs[jc] * d->coefs[jd] *
                 oracle_primitive_eri(a->exps[ja], a->shell, a->origin, b->exps[jb], b->shell, b->origin,
                                      c->exps[jc], c->shell, c->origin, d->exps[jd], d->shell, d->origin);
  return eri;
}

/* Flat-array form used by the ctypes wrapper: function f has origin[3f..],
 * shell[3f..], nprim[f] primitives starting at off[f] in exps/coefs/norm. */
typedef struct {
  const double* origin;
  const long* shell;
  const long* nprim;
  const long* off;
  const double* exps;
  const double* coefs;
  const double* norm;
} oracle_bfs;

static void bfs_get(const oracle_bfs* B, long f, oracle_basis* out) {
  for (int k = 0; k < 3; ++k) {
    out->origin[k] = B->origin[3 * f + k];
    out->shell[k] = B->shell[3 * f + k];
  }
  out->num_exps = B->nprim[f];
  out->exps = B->exps + B->off[f];
  out->coefs = B->coefs + B->off[f];
  out->norm = B->norm + B->off[f];
}

double oracle_eri_flat(const oracle_bfs* B, long i, long j, long k, long l) {
  oracle_basis a, b, c, d;
  bfs_get(B, i, &a);
  bfs_get(B, j, &b);
  bfs_get(B, k, &c);
  bfs_get(B, l, &d);
  return oracle_eri(&a, &b, &c, &d);
}

/* doERIs (cython/twoe.pyx:12-31): unique quartets ij >= kl, eight symmetric copies. */
void oracle_doERIs(long N, double* TwoE, const oracle_bfs* B) {
#define T4(i, j, k, l) TwoE[(((i) * N + (j)) * N + (k)) * N + (l)]
  for (long i = 0; i < N; ++i)
    for (long j = 0; j < i + 1; ++j) {
      long ij = i * (i + 1) / 2 + j;
      for (long k = 0; k < N; ++k)
        for (long l = 0; l < k + 1; ++l) {
          long kl = k * (k + 1) / 2 + l;
          if (ij >= kl) {
            double val = oracle_eri_flat(B, i, j, k, l);
            T4(i, j, k, l) = val;
            T4(k, l, i, j) = val;
            T4(j, i, l, k) = val;
            T4(l, k, j, i) = val;
            T4(j, i, k, l) = val;
            T4(l, k, i, j) = val;
            T4(i, j, l, k) = val;
            T4(k, l, j, i) = val;
          }
        }
    }
#undef T4
}

/* Schwarz table of Molecule.build (mmd/molecule.py:95-99): screen[p(p+1)/2+q] = (pq|pq). */
void oracle_screen(long N, const oracle_bfs* B, double* screen) {
  for (long p = 0; p < N; ++p)
    for (long q = 0; q < p + 1; ++q) screen[p * (p + 1) / 2 + q] = oracle_eri_flat(B, p, q, p, q);
}

/* formPT (cython/fock.pyx:13-87) for a real density difference dP = P - P_old,
 * restricted to the canonical bra pairs ij in [ij_lo, ij_hi) and, when `owner` is
 * given, to the function quartets whose shell quartet belongs to `part`.  The
 * restriction is test support (parallel checks and the sharded Fock build): the
 * loop body is the reference's.  Ownership: function f lies in shell func_shell[f]
 * (0..S-1, one molecule); a shell pair (s1 >= s2) has the canonical index
 * s1(s1+1)/2 + s2; a shell quartet belongs to owner[] of its pair with the larger
 * canonical index (owner[] is indexed by canonical pair index).
 * G (N*N, zeroed here) receives the unsymmetrised two-electron Fock update. */
static long formPT_impl(long N, const oracle_bfs* B, const double* eri_table, const double* P, const double* P_old,
                        const double* screen, double tol, double* G, long ij_lo, long ij_hi, const long* func_shell,
                        const int* owner, int part);

long oracle_formPT_part(long N, const oracle_bfs* B, const double* P, const double* P_old, const double* screen,
                        double tol, double* G, long ij_lo, long ij_hi, const long* func_shell, const int* owner,
                        int part) {
  return formPT_impl(N, B, NULL, P, P_old, screen, tol, G, ij_lo, ij_hi, func_shell, owner, part);
}

/* formPT with the ERIs read from a table of the unique quartets in doERIs loop order
 * (eri_table[ij(ij+1)/2 + kl], as oracle_eri_unique writes them) instead of being
 * recomputed: the same values, so the same G; test support for large checks. */
long oracle_formPT_table(long N, const double* eri_table, const double* P, const double* P_old, const double* screen,
                         double tol, double* G) {
  return formPT_impl(N, NULL, eri_table, P, P_old, screen, tol, G, 0, N * (N + 1) / 2, NULL, NULL, 0);
}

static long formPT_impl(long N, const oracle_bfs* B, const double* eri_table, const double* P, const double* P_old,
                        const double* screen, double tol, double* G, long ij_lo, long ij_hi, const long* func_shell,
                        const int* owner, int part) {
  double* dP = (double*)malloc(sizeof(double) * N * N);
  for (long x = 0; x < N * N; ++x) {
    dP[x] = P[x] - P_old[x];
    G[x] = 0.0;
  }
  long computed = 0;
#define D(a, b) dP[(a) * N + (b)]
#define GG(a, b) G[(a) * N + (b)]
#define SPAIR(x, y) ((x) >= (y) ? (x) * ((x) + 1) / 2 + (y) : (y) * ((y) + 1) / 2 + (x))
  for (long i = 0; i < N; ++i)
    for (long j = 0; j < i + 1; ++j) {
      long ij = i * (i + 1) / 2 + j;
      if (ij < ij_lo || ij >= ij_hi) continue;
      for (long k = 0; k < N; ++k)
        for (long l = 0; l < k + 1; ++l) {
          long kl = k * (k + 1) / 2 + l;
          if (ij < kl) continue;
          if (owner) {
            long c1 = SPAIR(func_shell[i], func_shell[j]), c2 = SPAIR(func_shell[k], func_shell[l]);
            if (owner[c1 >= c2 ? c1 : c2] != part) continue;
          }
          double bound = sqrt(screen[ij]) * sqrt(screen[kl]);
          double v[6] = {fabs(4 * D(i, j)), fabs(4 * D(k, l)), fabs(D(i, k)), fabs(D(i, l)), fabs(D(j, k)), fabs(D(j, l))};
          double dmax = v[0];
          for (int q = 1; q < 6; ++q)
            if (v[q] > dmax) dmax = v[q];
          bound *= dmax;
          if (bound < tol) continue;
          double s12 = (i == j) ? 1.0 : 2.0;
          double s34 = (k == l) ? 1.0 : 2.0;
          double s12_34 = (i == k) ? ((j == l) ? 1.0 : 2.0) : 2.0;
          double eri = s12 * s34 * s12_34 *
                       (eri_table ? eri_table[ij * (ij + 1) / 2 + kl] : oracle_eri_flat(B, i, j, k, l));
          ++computed;
          GG(i, j) += D(k, l) * eri;
          GG(k, l) += D(i, j) * eri;
          GG(i, k) += -0.25 * D(j, l) * eri;
          GG(j, l) += -0.25 * D(i, k) * eri;
          GG(i, l) += -0.25 * D(j, k) * eri;
          GG(k, j) += -0.25 * D(i, l) * eri;
        }
    }
#undef SPAIR
#undef D
#undef GG
  free(dP);
  return computed;
}

/* formPT (cython/fock.pyx:13-87) over every function quartet. */
long oracle_formPT(long N, const oracle_bfs* B, const double* P, const double* P_old, const double* screen, double tol,
                   double* G) {
  return oracle_formPT_part(N, B, P, P_old, screen, tol, G, 0, N * (N + 1) / 2, NULL, NULL, 0);
}

/* The unique ERIs of doERIs (cython/twoe.pyx:12-31) with canonical bra pair ij in
 * [ij_lo, ij_hi), in loop order (ij ascending, then kl = 0..ij): out receives
 * sum_{ij} (ij+1) values.  Test support: splits doERIs over processes. */
void oracle_eri_unique(long N, const oracle_bfs* B, long ij_lo, long ij_hi, double* out) {
  long o = 0;
  for (long i = 0; i < N; ++i)
    for (long j = 0; j < i + 1; ++j) {
      long ij = i * (i + 1) / 2 + j;
      if (ij < ij_lo || ij >= ij_hi) continue;
      for (long k = 0; k < N; ++k)
        for (long l = 0; l < k + 1; ++l) {
          long kl = k * (k + 1) / 2 + l;
          if (kl > ij) continue;
          out[o++] = oracle_eri_flat(B, i, j, k, l);
        }
    }
}

/* ------------------------------------------------ memoised shell-quartet ERIs
 * All component ERIs of four shells at once, with the Hermite E (util.pxi:13-28)
 * and R (util.pxi:33-50) recursions memoised per primitive pair / primitive
 * quartet.  Each memo entry is computed by the same expression from the same
 * child values as the plain recursion, and every sum runs in the order of
 * oracle_eri / oracle_primitive_eri, so the results equal oracle_eri_flat bit for
 * bit (pinned in the CPU tests); only repeated evaluations are skipped.  Shells
 * are lists of functions that share origin and exponents (one Cartesian shell). */
#define ORACLE_EMAX 3 /* i, j <= 2 */
#define ORACLE_TMAX 6
typedef struct {
  double Qx, a, b;
  double val[ORACLE_EMAX][ORACLE_EMAX][ORACLE_TMAX];
  char have[ORACLE_EMAX][ORACLE_EMAX][ORACLE_TMAX];
} emo;

static double emo_E(emo* m, int i, int j, int t) {
  double p = m->a + m->b;
  double u = m->a * m->b / p;
  if (t < 0 || t > i + j) return 0.0;
  if (m->have[i][j][t]) return m->val[i][j][t];
  double r;
  if (i == 0 && j == 0 && t == 0)
    r = exp(-u * m->Qx * m->Qx);
  else if (j == 0)
    r = (1.0 / (2.0 * p)) * emo_E(m, i - 1, j, t - 1) - (u * m->Qx / m->a) * emo_E(m, i - 1, j, t) +
        (t + 1) * emo_E(m, i - 1, j, t + 1);
  else
    r = (1.0 / (2.0 * p)) * emo_E(m, i, j - 1, t - 1) + (u * m->Qx / m->b) * emo_E(m, i, j - 1, t) +
        (t + 1) * emo_E(m, i, j - 1, t + 1);
  m->val[i][j][t] = r;
  m->have[i][j][t] = 1;
  return r;
}

#define ORACLE_RMAX 9 /* t, u, v, n <= 8 */
typedef struct {
  double p, PCx, PCy, PCz, RPC;
  double val[ORACLE_RMAX][ORACLE_RMAX][ORACLE_RMAX][ORACLE_RMAX];
  char have[ORACLE_RMAX][ORACLE_RMAX][ORACLE_RMAX][ORACLE_RMAX];
} rmo;

static double rmo_R(rmo* m, int t, int u, int v, int n) {
  if (m->have[t][u][v][n]) return m->val[t][u][v][n];
  double T = m->p * m->RPC * m->RPC;
  double val = 0.0;
  if (t == 0 && u == 0 && v == 0) {
    val += pow(-2.0 * m->p, n) * oracle_boys((double)n, T);
  } else if (t == 0 && u == 0) {
    if (v > 1) val += (v - 1) * rmo_R(m, t, u, v - 2, n + 1);
    val += m->PCz * rmo_R(m, t, u, v - 1, n + 1);
  } else if (t == 0) {
    if (u > 1) val += (u - 1) * rmo_R(m, t, u - 2, v, n + 1);
    val += m->PCy * rmo_R(m, t, u - 1, v, n + 1);
  } else {
    if (t > 1) val += (t - 1) * rmo_R(m, t - 2, u, v, n + 1);
    val += m->PCx * rmo_R(m, t - 1, u, v, n + 1);
  }
  m->val[t][u][v][n] = val;
  m->have[t][u][v][n] = 1;
  return val;
}

/* out[((x*nb + y)*nc + z)*nd + w] = ERI(fa[x], fb[y], fc[z], fd[w]) */
void oracle_eri_shell(const oracle_bfs* B, const long* fa, long na, const long* fb, long nb, const long* fc, long nc,
                      const long* fd, long nd, double* out) {
  oracle_basis A, Bb, C, Dd;
  bfs_get(B, fa[0], &A);
  bfs_get(B, fb[0], &Bb);
  bfs_get(B, fc[0], &C);
  bfs_get(B, fd[0], &Dd);
  const long ntot = na * nb * nc * nd;
  for (long x = 0; x < ntot; ++x) out[x] = 0.0;
  emo* e1 = (emo*)malloc(sizeof(emo) * 3);
  emo* e2 = (emo*)malloc(sizeof(emo) * 3);
  rmo* r = (rmo*)malloc(sizeof(rmo));
  for (long ja = 0; ja < A.num_exps; ++ja)
    for (long jb = 0; jb < Bb.num_exps; ++jb) {
      const double a = A.exps[ja], b = Bb.exps[jb];
      for (int dim = 0; dim < 3; ++dim) {
        memset(e1[dim].have, 0, sizeof(e1[dim].have));
        e1[dim].Qx = A.origin[dim] - Bb.origin[dim];
        e1[dim].a = a;
        e1[dim].b = b;
      }
      for (long jc = 0; jc < C.num_exps; ++jc)
        for (long jd = 0; jd < Dd.num_exps; ++jd) {
          const double c = C.exps[jc], d = Dd.exps[jd];
          for (int dim = 0; dim < 3; ++dim) {
            memset(e2[dim].have, 0, sizeof(e2[dim].have));
            e2[dim].Qx = C.origin[dim] - Dd.origin[dim];
            e2[dim].a = c;
            e2[dim].b = d;
          }
          /* geometry of oracle_primitive_eri, the same expressions */
          double p = a + b, q = c + d;
          double alpha = p * q / (p + q);
          double Px = (a * A.origin[0] + b * Bb.origin[0]) / p, Py = (a * A.origin[1] + b * Bb.origin[1]) / p,
                 Pz = (a * A.origin[2] + b * Bb.origin[2]) / p;
          double Qx = (c * C.origin[0] + d * Dd.origin[0]) / q, Qy = (c * C.origin[1] + d * Dd.origin[1]) / q,
                 Qz = (c * C.origin[2] + d * Dd.origin[2]) / q;
          double RPQ = sqrt(pow(Px - Qx, 2) + pow(Py - Qy, 2) + pow(Pz - Qz, 2));
          memset(r->have, 0, sizeof(r->have));
          r->p = alpha;
          r->PCx = Px - Qx;
          r->PCy = Py - Qy;
          r->PCz = Pz - Qz;
          r->RPC = RPQ;
          const double pref = 2.0 * pow(ORACLE_PI, 2.5) / (p * q * sqrt(p + q));
          for (long x = 0; x < na; ++x)
            for (long y = 0; y < nb; ++y)
              for (long z = 0; z < nc; ++z)
                for (long w = 0; w < nd; ++w) {
                  oracle_basis fa_, fb_, fc_, fd_;
                  bfs_get(B, fa[x], &fa_);
                  bfs_get(B, fb[y], &fb_);
                  bfs_get(B, fc[z], &fc_);
                  bfs_get(B, fd[w], &fd_);
                  const long l1 = fa_.shell[0], m1 = fa_.shell[1], n1 = fa_.shell[2];
                  const long l2 = fb_.shell[0], m2 = fb_.shell[1], n2 = fb_.shell[2];
                  const long l3 = fc_.shell[0], m3 = fc_.shell[1], n3 = fc_.shell[2];
                  const long l4 = fd_.shell[0], m4 = fd_.shell[1], n4 = fd_.shell[2];
                  double val = 0.0;
                  for (long t = 0; t < l1 + l2 + 1; ++t)
                    for (long u = 0; u < m1 + m2 + 1; ++u)
                      for (long v = 0; v < n1 + n2 + 1; ++v)
                        for (long tau = 0; tau < l3 + l4 + 1; ++tau)
                          for (long nu = 0; nu < m3 + m4 + 1; ++nu)
                            for (long phi = 0; phi < n3 + n4 + 1; ++phi)
                              val += emo_E(&e1[0], (int)l1, (int)l2, (int)t) * emo_E(&e1[1], (int)m1, (int)m2, (int)u) *
                                     emo_E(&e1[2], (int)n1, (int)n2, (int)v) *
                                     emo_E(&e2[0], (int)l3, (int)l4, (int)tau) *
                                     emo_E(&e2[1], (int)m3, (int)m4, (int)nu) *
                                     emo_E(&e2[2], (int)n3, (int)n4, (int)phi) * pow(-1.0, (double)(tau + nu + phi)) *
                                     rmo_R(r, (int)(t + tau), (int)(u + nu), (int)(v + phi), 0);
                  val *= pref;
                  out[((x * nb + y) * nc + z) * nd + w] +=
                      fa_.norm[ja] * fb_.norm[jb] * fc_.norm[jc] * fd_.norm[jd] * fa_.coefs[ja] * fb_.coefs[jb] *
                      fc_.coefs[jc] * fd_.coefs[jd] * val;
                }
        }
    }
  free(e1);
  free(e2);
  free(r);
}
