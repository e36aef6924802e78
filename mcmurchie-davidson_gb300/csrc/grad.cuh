// grad.cuh -- analytic RHF nuclear gradient kernels (defined in grad.cu).
#pragma once
#include <cuda_runtime.h>

constexpr int kGradMaxComp = 6;  // Cartesian components per shell slot (d)

struct GradArgs {
  // shells and the shell pairs (every unordered pair of shells of the molecule once)
  int npair;
  const int *pa, *pb;
  const int *L, *nprim, *poff, *func, *shell_atom;
  const double *center, *exps, *coefs;
  const float* Qpair;  // Schwarz bound per shell pair (null: no screening)
  double qtol;         // quartets with Q_ab Q_cd below qtol are skipped
  // nuclei
  int natom;
  const double *xyz, *Z;
  // densities (N x N, device) and the output dE/dR (natom x 3, device, accumulated)
  const double *P, *W;
  int N;
  double* grad;
};

cudaError_t mmdg_launch_rhf_gradient(const GradArgs& a, cudaStream_t st);
