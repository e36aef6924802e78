// ao2mo.cu -- the AO -> MO four-index transform of the ERI tensor (mmd/postscf.py:26-27:
// four einsums with the MO coefficients, one index at a time).
//
// One quarter transform contracts the last index with C and writes the new index
// first:
//     out[S, p, q, r] = sum_s in[p, q, r, s] C[s, S]
// so four calls of the same kernel turn (pq|rs) into (PQ|RS) in the original index
// order: pqrs -> Spqr -> RSpq -> QRSp -> PQRS.  Each call is a GEMM
// out (N x N^3) = C^T (N x N) . in^T (N x N^3) in FP64: 64 x 64 output tiles per
// 256-thread block, 4 x 4 outputs per thread, the K dimension staged through shared
// memory 16 at a time.  An FP64 warp instruction holds the FP64 pipe of its
// sub-partition for ~64 cycles on this GPU, so the eight shared-memory loads around
// a thread's 16 independent FMAs per k step cost nothing; the 16 accumulators keep
// the pipe fed.
#include <cuda_runtime.h>

#include "../../include/mmdg.h"

int mmdg_internal_fail(int code, const char* msg);

namespace {

constexpr int TS = 64;  // output rows (new index S) per block
constexpr int TMv = 64; // output columns (old flattened pqr) per block
constexpr int TK = 16;  // contracted index s per stage

__global__ void __launch_bounds__(256) k_quarter(const double* __restrict__ in, const double* __restrict__ C,
                                                 double* __restrict__ out, int N, long long M) {
  __shared__ double Cs[TK][TS + 1];    // C[s0 + k, S0 + j]
  __shared__ double Is[TK][TMv + 1];   // in[m0 + j, s0 + k] (transposed)
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int S0 = blockIdx.y * TS;
  const long long m0 = (long long)blockIdx.x * TMv;
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
  for (int s0 = 0; s0 < N; s0 += TK) {
    for (int e = threadIdx.x; e < TK * TS; e += 256) {
      const int k = e / TS, j = e - k * TS;
      const int s = s0 + k, S = S0 + j;
      Cs[k][j] = (s < N && S < N) ? C[(long long)s * N + S] : 0.0;
    }
    for (int e = threadIdx.x; e < TK * TMv; e += 256) {
      const int j = e / TK, k = e - j * TK;  // k fastest: coalesced along s
      const int s = s0 + k;
      const long long m = m0 + j;
      Is[k][j] = (s < N && m < M) ? in[m * N + s] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < TK; ++k) {
      double cv[4], iv[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) cv[a] = Cs[k][ty * 4 + a];
#pragma unroll
      for (int b = 0; b < 4; ++b) iv[b] = Is[k][tx + 16 * b];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = fma(cv[a], iv[b], acc[a][b]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int S = S0 + ty * 4 + a;
    if (S >= N) continue;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const long long m = m0 + tx + 16 * b;
      if (m < M) out[(long long)S * M + m] = acc[a][b];
    }
  }
}

}  // namespace

extern "C" int mmdg_ao2mo(long long N, const double* C, const double* eri_in, double* eri_out, double* work,
                          void* stream) {
  if (N <= 0 || !C || !eri_in || !eri_out || !work)
    return mmdg_internal_fail(MMDG_E_ARG, "mmdg_ao2mo: bad argument");
  if (N > 1290) return mmdg_internal_fail(MMDG_E_ARG, "mmdg_ao2mo: N^3 exceeds the grid (N <= 1290)");
  if (eri_out == eri_in || work == eri_in || work == eri_out)
    return mmdg_internal_fail(MMDG_E_ARG, "mmdg_ao2mo: eri_in, eri_out and work must be distinct");
  cudaStream_t st = (cudaStream_t)stream;
  const long long M = N * N * N;
  const dim3 grid((unsigned)((M + TMv - 1) / TMv), (unsigned)((N + TS - 1) / TS));
  const double* src[4] = {eri_in, work, eri_out, work};
  double* dst[4] = {work, eri_out, work, eri_out};
  for (int q = 0; q < 4; ++q) {
    k_quarter<<<grid, 256, 0, st>>>(src[q], C, dst[q], (int)N, M);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return mmdg_internal_fail(MMDG_E_CUDA, cudaGetErrorString(e));
  }
  return MMDG_OK;
}
