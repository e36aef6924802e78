// pairs.cuh -- primitive-pair construction kernel shared by capi.cu and noalloc.cu.
#pragma once
#include <cuda_runtime.h>

struct PairBuildArgs {
  int npair;
  const int *pa, *pb, *prb;
  // optional primitive subset: pair pr builds the primitive pairs
  // keep[prb[pr] .. prb[pr] + prc[pr]) (index ka * Kb + kb); null: all Ka * Kb
  const int *keep, *prc;
  const long long* eoff;
  const int *L, *nprim, *poff;
  const double *center, *exps, *coefs;
  double4_32a* pP;
  float4* pPf;
  double* E64;
  float* E32;
};


// One thread per shell pair: primitive-pair data and E' tables (defined in capi.cu).
__global__ void k_build_pairs(PairBuildArgs a);

// Boys interpolation table on the host (defined in capi.cu), written into t64
// (kBoysTabSize doubles).
void mmdg_fill_boys_table(double* t64);

// Record the failure text returned by mmdg_last_error (defined in capi.cu).
int mmdg_internal_fail(int code, const char* msg);
