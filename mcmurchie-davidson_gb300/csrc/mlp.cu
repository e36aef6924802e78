// mlp.cu -- kernels of the learned initial-guess network: a 3-layer MLP with BF16
// weights and FP32 accumulation, trained and served on the GPU.
//
// The network maps atom-pair features to density-matrix blocks (the SCF's initial
// guess; the reference starts from P = 0, mmd/scf.py:15,23-24).  Sizes are tiny
// (~100 k parameters, ~1 M training pairs), so the GEMMs are shared-memory tiled
// FP32 FMA kernels reading BF16 weights; they are a few ms per epoch and not a hot
// path of the ERI work.
//
//   gemm:   C[M,N] (+)= op(A)[M,K] op(B)[K,N], A/B in FP32 or BF16, C in FP32
//   act:    Y = silu(Z + b) (stores Z + b for the backward), or identity
//   loss:   dY = 2 (Y - T) * mask / count, and the loss value
//   adam:   FP32 master weights, BF16 copies refreshed in the same pass
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/mmdg.h"
#include "pairs.cuh"

namespace {

constexpr int TM = 64, TN = 64, TK = 16;

template <typename T>
__device__ __forceinline__ float ld(const T* p, long long i);
template <>
__device__ __forceinline__ float ld<float>(const float* p, long long i) { return p[i]; }
template <>
__device__ __forceinline__ float ld<__nv_bfloat16>(const __nv_bfloat16* p, long long i) {
  return __bfloat162float(p[i]);
}

// C = alpha * op(A) op(B) + beta * C;  op(A): ta ? A^T (A stored K x M) : A (M x K)
template <typename TA, typename TB>
__global__ void __launch_bounds__(256) k_gemm(int M, int N, int K, const TA* A, int lda, int ta, const TB* B, int ldb,
                                              int tb, float* C, int ldc, float beta) {
  __shared__ float As[TK][TM + 1];
  __shared__ float Bs[TK][TN + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
  // split K over blockIdx.z (the weight gradients: M x N small, K = batch rows)
  const int kspan = (K + gridDim.z - 1) / gridDim.z;
  const int kbeg = blockIdx.z * kspan, kend = min(K, kbeg + kspan);
  float acc[4][4] = {};
  for (int k0 = kbeg; k0 < kend; k0 += TK) {
    for (int e = threadIdx.x; e < TK * TM; e += 256) {
      const int kk = e / TM, mm = e % TM;
      const int m = m0 + mm, k = k0 + kk;
      float v = 0.f;
      if (m < M && k < kend) v = ta ? ld(A, (long long)k * lda + m) : ld(A, (long long)m * lda + k);
      As[kk][mm] = v;
    }
    for (int e = threadIdx.x; e < TK * TN; e += 256) {
      const int kk = e / TN, nn = e % TN;
      const int n = n0 + nn, k = k0 + kk;
      float v = 0.f;
      if (n < N && k < kend) v = tb ? ld(B, (long long)n * ldb + k) : ld(B, (long long)k * ldb + n);
      Bs[kk][nn] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int m = m0 + ty * 4 + i, n = n0 + tx * 4 + j;
      if (m < M && n < N) {
        float* c = C + (long long)m * ldc + n;
        if (gridDim.z > 1)
          atomicAdd(c, acc[i][j]);  // C zeroed by the launcher
        else
          *c = beta != 0.f ? fmaf(beta, *c, acc[i][j]) : acc[i][j];
      }
    }
}

// Z = X + b (row broadcast), Y = silu(Z) (or Y = Z); Z kept for the backward
__global__ void k_bias_act(float* Z, float* Y, const float* b, long long rows, int cols, int silu) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= rows * cols) return;
  const float z = Z[i] + b[i % cols];
  Z[i] = z;
  Y[i] = silu ? z / (1.f + expf(-z)) : z;
}

// dZ = dY * silu'(Z)
__global__ void k_act_grad(const float* Z, const float* dY, float* dZ, long long n, int silu) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (!silu) {
    dZ[i] = dY[i];
    return;
  }
  const float z = Z[i], s = 1.f / (1.f + expf(-z));
  dZ[i] = dY[i] * s * (1.f + z * (1.f - s));
}

// column sums: db[c] = sum_r dZ[r, c] (row chunks of 1024, FP32 atomics; db zeroed first)
__global__ void k_colsum(const float* dZ, float* db, long long rows, int cols) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  const long long r0 = (long long)blockIdx.y * 1024, r1 = min(rows, r0 + 1024);
  float s = 0.f;
  for (long long r = r0; r < r1; ++r) s += dZ[r * cols + c];
  atomicAdd(db + c, s);
}

__global__ void k_mse(const float* Y, const float* T, const float* mask, float* dY, double* loss, long long n,
                      float inv_count) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  float l = 0.f;
  if (i < n) {
    const float d = (Y[i] - T[i]) * mask[i];
    dY[i] = 2.f * d * inv_count;
    l = d * d * inv_count;
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, (double)l);
}

__global__ void k_adam(float* w, __nv_bfloat16* wb, const float* g, float* m, float* v, long long n, float lr,
                       float b1, float b2, float eps, float c1, float c2) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  w[i] = wi;
  if (wb) wb[i] = __float2bfloat16(wi);
}

__global__ void k_to_bf16(const float* w, __nv_bfloat16* wb, long long n) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) wb[i] = __float2bfloat16(w[i]);
}

unsigned nb(long long n, int t = 256) { return (unsigned)((n + t - 1) / t); }

int launch_fail(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) return MMDG_OK;
  return mmdg_internal_fail(MMDG_E_CUDA, what);
}

}  // namespace

// C = op(A) op(B) (+ beta C): a_bf16 / b_bf16 select BF16 operands (weights)
extern "C" int mmdg_mlp_gemm(int M, int N, int K, const void* A, int lda, int ta, int a_bf16, const void* B, int ldb,
                             int tb, int b_bf16, float* C, int ldc, float beta, void* stream) {
  if (M < 0 || N < 0 || K < 0 || !A || !B || !C) return mmdg_internal_fail(MMDG_E_ARG, "mmdg_mlp_gemm: bad argument");
  if (!M || !N) return MMDG_OK;
  dim3 grid((N + TN - 1) / TN, (M + TM - 1) / TM);
  cudaStream_t st = (cudaStream_t)stream;
  // few output tiles and a long K (weight gradients over a batch): split K over
  // enough blocks to fill the GPU, partial tiles added with atomics into a zeroed C
  const long long tiles = (long long)grid.x * grid.y;
  if (beta == 0.f && tiles < 304 && K >= 1024) {
    const int split = (int)std::min<long long>((K + 511) / 512, (608 + tiles - 1) / tiles);
    if (split > 1) {
      grid.z = split;
      if (cudaMemsetAsync(C, 0, sizeof(float) * (size_t)M * ldc, st) != cudaSuccess)
        return mmdg_internal_fail(MMDG_E_CUDA, "mmdg_mlp_gemm: memset");
    }
  }
  if (a_bf16 && !b_bf16)
    k_gemm<__nv_bfloat16, float><<<grid, 256, 0, st>>>(M, N, K, (const __nv_bfloat16*)A, lda, ta, (const float*)B, ldb,
                                                        tb, C, ldc, beta);
  else if (!a_bf16 && b_bf16)
    k_gemm<float, __nv_bfloat16><<<grid, 256, 0, st>>>(M, N, K, (const float*)A, lda, ta, (const __nv_bfloat16*)B, ldb,
                                                        tb, C, ldc, beta);
  else if (!a_bf16 && !b_bf16)
    k_gemm<float, float><<<grid, 256, 0, st>>>(M, N, K, (const float*)A, lda, ta, (const float*)B, ldb, tb, C, ldc, beta);
  else
    return mmdg_internal_fail(MMDG_E_ARG, "mmdg_mlp_gemm: at most one BF16 operand");
  return launch_fail("mmdg_mlp_gemm: launch");
}

extern "C" int mmdg_mlp_bias_act(float* Z, float* Y, const float* b, long long rows, int cols, int silu, void* stream) {
  if (!Z || !Y || !b || rows < 0 || cols <= 0) return mmdg_internal_fail(MMDG_E_ARG, "mmdg_mlp_bias_act: bad argument");
  if (!rows) return MMDG_OK;
  k_bias_act<<<nb(rows * cols), 256, 0, (cudaStream_t)stream>>>(Z, Y, b, rows, cols, silu);
  return launch_fail("mmdg_mlp_bias_act: launch");
}

extern "C" int mmdg_mlp_act_grad(const float* Z, const float* dY, float* dZ, long long n, int silu, void* stream) {
  if (!Z || !dY || !dZ || n < 0) return mmdg_internal_fail(MMDG_E_ARG, "mmdg_mlp_act_grad: bad argument");
  if (!n) return MMDG_OK;
  k_act_grad<<<nb(n), 256, 0, (cudaStream_t)stream>>>(Z, dY, dZ, n, silu);
  return launch_fail("mmdg_mlp_act_grad: launch");
}

extern "C" int mmdg_mlp_colsum(const float* dZ, float* db, long long rows, int cols, void* stream) {
  if (!dZ || !db || rows < 0 || cols <= 0) return mmdg_internal_fail(MMDG_E_ARG, "mmdg_mlp_colsum: bad argument");
  cudaStream_t st = (cudaStream_t)stream;
  if (cudaMemsetAsync(db, 0, sizeof(float) * cols, st) != cudaSuccess)
    return mmdg_internal_fail(MMDG_E_CUDA, "mmdg_mlp_colsum: memset");
  if (!rows) return MMDG_OK;
  dim3 grid(nb(cols, 128), (unsigned)((rows + 1023) / 1024));
  k_colsum<<<grid, 128, 0, st>>>(dZ, db, rows, cols);
  return launch_fail("mmdg_mlp_colsum: launch");
}

extern "C" int mmdg_mlp_mse(const float* Y, const float* T, const float* mask, float* dY, double* loss, long long n,
                            float inv_count, void* stream) {
  if (!Y || !T || !mask || !dY || !loss || n < 0) return mmdg_internal_fail(MMDG_E_ARG, "mmdg_mlp_mse: bad argument");
  if (!n) return MMDG_OK;
  k_mse<<<nb(n), 256, 0, (cudaStream_t)stream>>>(Y, T, mask, dY, loss, n, inv_count);
  return launch_fail("mmdg_mlp_mse: launch");
}

extern "C" int mmdg_mlp_adam(float* w, void* w_bf16, const float* g, float* m, float* v, long long n, float lr,
                             float b1, float b2, float eps, int step, void* stream) {
  if (!w || !g || !m || !v || n < 0 || step < 1) return mmdg_internal_fail(MMDG_E_ARG, "mmdg_mlp_adam: bad argument");
  const float c1 = 1.f / (1.f - powf(b1, (float)step)), c2 = 1.f / (1.f - powf(b2, (float)step));
  k_adam<<<nb(n), 256, 0, (cudaStream_t)stream>>>(w, (__nv_bfloat16*)w_bf16, g, m, v, n, lr, b1, b2, eps, c1, c2);
  return launch_fail("mmdg_mlp_adam: launch");
}

extern "C" int mmdg_mlp_to_bf16(const float* w, void* w_bf16, long long n, void* stream) {
  if (!w || !w_bf16 || n < 0) return mmdg_internal_fail(MMDG_E_ARG, "mmdg_mlp_to_bf16: bad argument");
  if (!n) return MMDG_OK;
  k_to_bf16<<<nb(n), 256, 0, (cudaStream_t)stream>>>(w, (__nv_bfloat16*)w_bf16, n);
  return launch_fail("mmdg_mlp_to_bf16: launch");
}
