// noalloc.cu -- ERI tensor of a small molecule without any memory allocation.
//
// mmdg_eri_tensor needs a context whose primitive-pair data, E' tables and Boys
// table live in cudaMalloc'd buffers.  Some callers cannot allocate device memory:
// host frameworks that own the whole GPU memory pool and forbid outside
// allocations, code that must not synchronise the device (cudaMalloc and cudaFree
// may synchronise), and services that cannot recover from an allocation failure in
// the middle of a request.  For them, mmdg_eri_tensor_noalloc keeps every piece of
// scratch in one file-scope __device__ array, g_noalloc_scratch (kNoAllocScratchBytes,
// held by every GPU that loads the library until the process exits), and stages its
// host-side bookkeeping in fixed-size arrays: no cudaMalloc, no cudaFree, no heap.
//
// Set-up: the first call on a device (with that device current) looks up the
// array's device address with cudaGetSymbolAddress -- in host code the symbol name
// is only a host-side stand-in -- and uploads the Boys table into it.  That first
// call should come before any stream capture.  Every later call looks the address
// up again (cheap, no allocation) and repeats the set-up if it changed, as after a
// cudaDeviceReset, which reloads the module with a fresh array.  All calls share
// the array and it keeps the previous call's contents: everything a call reads is
// rewritten by the same call before use, and the output tensor is cleared.  Calls
// that overlap on the GPU (different streams, or several host threads) race on the
// array; callers must serialise them.  The host-side bookkeeping lives in static
// arrays under one mutex (no heap, and about 1 KB of stack), so host threads are
// serialised here.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/mmdg.h"
#include "md_dispatch.cuh"
#include "pairs.cuh"

using namespace mmdg;

namespace {

constexpr int kNA_MaxShell = 64;
constexpr int kNA_MaxPrim = 256;
constexpr int kNA_MaxFunc = 64;
constexpr int kNA_MaxPair = kNA_MaxShell * (kNA_MaxShell + 1) / 2;  // 2080
constexpr int kNA_MaxPrimPair = 4096;
constexpr long long kNA_MaxE = 131072;  // doubles of E' tables
constexpr int kNA_PairClasses = (MMDG_LMAX + 1) * (MMDG_LMAX + 2) / 2;

// scratch layout (byte offsets, each 256-aligned)
constexpr size_t al(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kOffBoys = 0;
constexpr size_t kOffPP = al(kOffBoys + sizeof(double) * kBoysTabSize);
constexpr size_t kOffE = al(kOffPP + sizeof(double4_32a) * kNA_MaxPrimPair);
constexpr size_t kOffCenter = al(kOffE + sizeof(double) * kNA_MaxE);
constexpr size_t kOffExp = al(kOffCenter + sizeof(double) * 3 * kNA_MaxShell);
constexpr size_t kOffCoef = al(kOffExp + sizeof(double) * kNA_MaxPrim);
constexpr size_t kOffInts = al(kOffCoef + sizeof(double) * kNA_MaxPrim);
// int block: L, nprim, poff, func(6x), shmol, shlocal | pa, pb, prb, prc | class lists
constexpr int kIntShell = kNA_MaxShell * (5 + kMaxComp);
constexpr int kIntPair = kNA_MaxPair * 4;
constexpr int kIntLists = kNA_MaxPair;
constexpr size_t kOffEoff = al(kOffInts + sizeof(int) * (kIntShell + kIntPair + kIntLists + 8));
constexpr size_t kOffMol = al(kOffEoff + sizeof(long long) * kNA_MaxPair);
constexpr size_t kOffStamp = kOffMol + 48;  // 8 bytes, inside the molecule slot's spare tail
constexpr unsigned long long kNAStamp = 0x4d4d4447'4e413031ULL;
constexpr size_t kNoAllocScratchBytes = al(kOffMol + 64);

}  // namespace

// The scratch: one array for every call on this device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

std::mutex g_na_mutex;
void* g_na_base[64] = {};        // device address of g_noalloc_scratch per device
double g_na_boys[kBoysTabSize];  // host copy of the Boys table (static storage)
bool g_na_boys_ready = false;

// host staging of one call (static storage, used under g_na_mutex only)
struct NaHost {
  int L[kNA_MaxShell], K[kNA_MaxShell], poff[kNA_MaxShell], shlocal[kNA_MaxShell], shmol[kNA_MaxShell];
  int pa[kNA_MaxPair], pb[kNA_MaxPair], prb[kNA_MaxPair], prc[kNA_MaxPair], pcls[kNA_MaxPair];
  long long eoff[kNA_MaxPair];
  int lists[kNA_MaxPair], lbeg[kNA_PairClasses + 1];
  int ints[kIntShell + kIntPair + kIntLists + 8];
  long long mol[4];
  int moln[2];
};
NaHost g_na_host;
int na_fail(int code, const char* msg) { return mmdg_internal_fail(code, msg); }

int nnz_pair_na(int la, int lb) {
  int n = 0;
  for (int xa = la; xa >= 0; --xa)
    for (int ya = la - xa; ya >= 0; --ya)
      for (int xb = lb; xb >= 0; --xb)
        for (int yb = lb - xb; yb >= 0; --yb)
          n += (xa + xb + 1) * (ya + yb + 1) * ((la - xa - ya) + (lb - xb - yb) + 1);
  return n;
}

}  // namespace

static_assert(kNoAllocScratchBytes == 1738240, "scratch size stated in include/mmdg.h");

extern "C" int mmdg_eri_tensor_noalloc(int nshell, const int* shell_L, const int* shell_nprim,
                                       const double* shell_center, const double* prim_exp,
                                       const double* prim_coef, const int* shell_func, int nfunc, double* out,
                                       void* stream) {
  if (nshell < 1 || nfunc < 1 || !shell_L || !shell_nprim || !shell_center || !prim_exp || !prim_coef ||
      !shell_func || !out)
    return na_fail(MMDG_E_ARG, "mmdg_eri_tensor_noalloc: empty basis or null pointer");
  if (nshell > kNA_MaxShell)
    return na_fail(MMDG_E_ARG, "mmdg_eri_tensor_noalloc: more than 64 shells (scratch limit)");
  if (nfunc > kNA_MaxFunc)
    return na_fail(MMDG_E_ARG, "mmdg_eri_tensor_noalloc: more than 64 basis functions (scratch limit)");
  // ---------------- host bookkeeping in the static staging arrays
  std::lock_guard<std::mutex> lock(g_na_mutex);
  NaHost& H = g_na_host;
  int* L = H.L;
  int* K = H.K;
  int* poff = H.poff;
  int* shlocal = H.shlocal;
  int* shmol = H.shmol;
  int total_prim = 0;
  for (int s = 0; s < nshell; ++s) {
    if (shell_L[s] < 0) return na_fail(MMDG_E_ARG, "mmdg_eri_tensor_noalloc: negative angular momentum");
    if (shell_L[s] > MMDG_LMAX)
      return na_fail(MMDG_E_LMAX, "mmdg_eri_tensor_noalloc: angular momentum above d (l = 2)");
    if (shell_nprim[s] < 1) return na_fail(MMDG_E_ARG, "mmdg_eri_tensor_noalloc: shell without primitives");
    L[s] = shell_L[s];
    K[s] = shell_nprim[s];
    poff[s] = total_prim;
    shlocal[s] = s;
    shmol[s] = 0;
    total_prim += K[s];
    if (total_prim > kNA_MaxPrim)
      return na_fail(MMDG_E_ARG, "mmdg_eri_tensor_noalloc: more than 256 primitives (scratch limit)");
    const int nc = (L[s] + 1) * (L[s] + 2) / 2;
    for (int c = 0; c < MMDG_MAX_COMP; ++c) {
      const int f = shell_func[s * MMDG_MAX_COMP + c];
      if (f >= nfunc || (c >= nc && f >= 0))
        return na_fail(MMDG_E_ARG, "mmdg_eri_tensor_noalloc: bad function index");
    }
  }
  for (int p = 0; p < total_prim; ++p)
    if (!(prim_exp[p] > 0.0) || !std::isfinite(prim_exp[p]) || !std::isfinite(prim_coef[p]))
      return na_fail(MMDG_E_ARG, "mmdg_eri_tensor_noalloc: exponents must be positive and finite");
  for (int x = 0; x < 3 * nshell; ++x)
    if (!std::isfinite(shell_center[x])) return na_fail(MMDG_E_ARG, "mmdg_eri_tensor_noalloc: non-finite centre");
  int* pa = H.pa;
  int* pb = H.pb;
  int* prb = H.prb;
  int* prc = H.prc;
  int* pcls = H.pcls;
  long long* eoff = H.eoff;
  int npair = 0;
  long long npp = 0, ne = 0;
  for (int s1 = 0; s1 < nshell; ++s1)
    for (int s2 = s1; s2 >= 0; --s2) {
      int a = s1, b = s2;
      if (L[a] < L[b]) {
        const int t = a;
        a = b;
        b = t;
      }
      pa[npair] = a;
      pb[npair] = b;
      pcls[npair] = L[a] * (L[a] + 1) / 2 + L[b];
      prb[npair] = (int)npp;
      prc[npair] = K[a] * K[b];
      eoff[npair] = ne;
      npp += K[a] * K[b];
      ne += (long long)K[a] * K[b] * nnz_pair_na(L[a], L[b]);
      ++npair;
    }
  if (npp > kNA_MaxPrimPair)
    return na_fail(MMDG_E_ARG, "mmdg_eri_tensor_noalloc: more than 4096 primitive pairs (scratch limit)");
  if (ne > kNA_MaxE) return na_fail(MMDG_E_ARG, "mmdg_eri_tensor_noalloc: E' tables exceed the scratch limit");
  // class lists, concatenated
  int* lists = H.lists;
  int* lbeg = H.lbeg;
  {
    int n = 0;
    for (int c = 0; c < kNA_PairClasses; ++c) {
      lbeg[c] = n;
      for (int p = 0; p < npair; ++p)
        if (pcls[p] == c) lists[n++] = p;
    }
    lbeg[kNA_PairClasses] = n;
  }
  // ---------------- set-up per device: device address of the scratch, Boys table;
  // the address is looked up on every call and the set-up repeated when it changed
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 64) return na_fail(MMDG_E_CUDA, "mmdg_eri_tensor_noalloc: no device");
  if (!g_na_boys_ready) {
    mmdg_fill_boys_table(g_na_boys);
    g_na_boys_ready = true;
  }
  void* ptr = nullptr;
  e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
  if (e != cudaSuccess || !ptr) return na_fail(MMDG_E_CUDA, "mmdg_eri_tensor_noalloc: cudaGetSymbolAddress failed");
  cudaStream_t st = (cudaStream_t)stream;
  // a stamp written at set-up tells an initialised array from a fresh (zeroed) one,
  // e.g. after cudaDeviceReset reloaded the module at the same address
  unsigned long long stamp = 0;
  e = cudaMemcpyAsync(&stamp, static_cast<char*>(ptr) + kOffStamp, sizeof(stamp), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return na_fail(MMDG_E_CUDA, "mmdg_eri_tensor_noalloc: reading the set-up stamp failed");
  if (g_na_base[dev] != ptr || stamp != kNAStamp) {
    g_na_base[dev] = nullptr;
    e = cudaMemcpy(static_cast<char*>(ptr) + kOffBoys, g_na_boys, sizeof(double) * kBoysTabSize,
                   cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return na_fail(MMDG_E_CUDA, "mmdg_eri_tensor_noalloc: Boys table upload failed");
    // shared-memory limits of the class kernels (attributes, not allocations)
    for (int gi = 0; gi < kNumGroups; ++gi)
      if (kGroupInit[gi]() != cudaSuccess)
        return na_fail(MMDG_E_CUDA, "mmdg_eri_tensor_noalloc: kernel attribute set-up failed");
    static const unsigned long long kStampValue = kNAStamp;
    e = cudaMemcpy(static_cast<char*>(ptr) + kOffStamp, &kStampValue, sizeof(kStampValue), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return na_fail(MMDG_E_CUDA, "mmdg_eri_tensor_noalloc: writing the set-up stamp failed");
    g_na_base[dev] = ptr;
  }
  char* base = static_cast<char*>(g_na_base[dev]);
  // ---------------- stage inputs into the scratch (stream ordered)
  int* ints = H.ints;
  int* iL = ints;
  int* iK = iL + kNA_MaxShell;
  int* iP = iK + kNA_MaxShell;
  int* iF = iP + kNA_MaxShell;
  int* iM = iF + kNA_MaxShell * kMaxComp;
  int* iS = iM + kNA_MaxShell;
  int* ipa = ints + kIntShell;
  int* ipb = ipa + kNA_MaxPair;
  int* iprb = ipb + kNA_MaxPair;
  int* iprc = iprb + kNA_MaxPair;
  int* ilist = ints + kIntShell + kIntPair;
  for (int s = 0; s < nshell; ++s) {
    iL[s] = L[s];
    iK[s] = K[s];
    iP[s] = poff[s];
    iM[s] = shmol[s];
    iS[s] = shlocal[s];
    for (int c = 0; c < kMaxComp; ++c) iF[s * kMaxComp + c] = shell_func[s * MMDG_MAX_COMP + c];
  }
  for (int p = 0; p < npair; ++p) {
    ipa[p] = pa[p];
    ipb[p] = pb[p];
    iprb[p] = prb[p];
    iprc[p] = prc[p];
  }
  for (int p = 0; p < npair; ++p) ilist[p] = lists[p];
  long long* mol = H.mol;  // mol_base (mol_n as int below)
  mol[0] = 0;
  mol[1] = nfunc;
  mol[2] = mol[3] = 0;
  int* moln = H.moln;
  moln[0] = nfunc;
  moln[1] = nshell;
  double* dCenter = reinterpret_cast<double*>(base + kOffCenter);
  double* dExp = reinterpret_cast<double*>(base + kOffExp);
  double* dCoef = reinterpret_cast<double*>(base + kOffCoef);
  int* dInts = reinterpret_cast<int*>(base + kOffInts);
  long long* dEoff = reinterpret_cast<long long*>(base + kOffEoff);
  long long* dMolBase = reinterpret_cast<long long*>(base + kOffMol);
  int* dMolN = reinterpret_cast<int*>(base + kOffMol + 32);
#define NA_TRY(x)                                                                      \
  do {                                                                                 \
    if ((e = (x)) != cudaSuccess) return na_fail(MMDG_E_CUDA, "mmdg_eri_tensor_noalloc: " #x); \
  } while (0)
  NA_TRY(cudaMemcpyAsync(dCenter, shell_center, sizeof(double) * 3 * nshell, cudaMemcpyHostToDevice, st));
  NA_TRY(cudaMemcpyAsync(dExp, prim_exp, sizeof(double) * total_prim, cudaMemcpyHostToDevice, st));
  NA_TRY(cudaMemcpyAsync(dCoef, prim_coef, sizeof(double) * total_prim, cudaMemcpyHostToDevice, st));
  NA_TRY(cudaMemcpyAsync(dInts, ints, sizeof(H.ints), cudaMemcpyHostToDevice, st));
  NA_TRY(cudaMemcpyAsync(dEoff, eoff, sizeof(long long) * npair, cudaMemcpyHostToDevice, st));
  NA_TRY(cudaMemcpyAsync(dMolBase, mol, sizeof(long long), cudaMemcpyHostToDevice, st));
  NA_TRY(cudaMemcpyAsync(dMolN, moln, sizeof(int), cudaMemcpyHostToDevice, st));
  // pageable sources: make sure the copies have consumed the staging arrays before
  // the next call (or another thread, after the mutex) rewrites them
  NA_TRY(cudaStreamSynchronize(st));
  // ---------------- primitive pairs
  double4_32a* dPP = reinterpret_cast<double4_32a*>(base + kOffPP);
  double* dE = reinterpret_cast<double*>(base + kOffE);
  int* dL = dInts;
  int* dK = dL + kNA_MaxShell;
  int* dP = dK + kNA_MaxShell;
  int* dF = dP + kNA_MaxShell;
  int* dM = dF + kNA_MaxShell * kMaxComp;
  int* dS = dM + kNA_MaxShell;
  int* dpa = dInts + kIntShell;
  int* dpb = dpa + kNA_MaxPair;
  int* dprb = dpb + kNA_MaxPair;
  int* dprc = dprb + kNA_MaxPair;
  int* dlist = dInts + kIntShell + kIntPair;
  PairBuildArgs pa_args;
  pa_args.npair = npair;
  pa_args.pa = dpa;
  pa_args.pb = dpb;
  pa_args.prb = dprb;
  pa_args.keep = nullptr;
  pa_args.prc = nullptr;
  pa_args.eoff = dEoff;
  pa_args.L = dL;
  pa_args.nprim = dK;
  pa_args.poff = dP;
  pa_args.center = dCenter;
  pa_args.exps = dExp;
  pa_args.coefs = dCoef;
  pa_args.pP = dPP;
  pa_args.pPf = nullptr;
  pa_args.E64 = dE;
  pa_args.E32 = nullptr;
  k_build_pairs<<<(npair + 127) / 128, 128, 0, st>>>(pa_args);
  NA_TRY(cudaGetLastError());
  // ---------------- the tensor: cleared, then every class
  NA_TRY(cudaMemsetAsync(out, 0, sizeof(double) * (size_t)nfunc * nfunc * nfunc * nfunc, st));
  Geometry g;
  std::memset(&g, 0, sizeof(g));
  g.pP = dPP;
  g.E64 = dE;
  g.pr_begin = dprb;
  g.pr_count = dprc;
  g.e_off = dEoff;
  g.pa = dpa;
  g.pb = dpb;
  g.func = dF;
  g.sh_mol = dM;
  g.sh_local = dS;
  g.mol_base = dMolBase;
  g.mol_n = dMolN;
  g.boys64 = reinterpret_cast<const double*>(base + kOffBoys);
  g.boysdf = nullptr;  // the static scratch holds the FP64 rows only: boys_eval_df uses them
  TensorArgs t{out};
  for (const ClassEntry& ce : kClasses) {
    const int cb = ce.la * (ce.la + 1) / 2 + ce.lb, ck = ce.lc * (ce.lc + 1) / 2 + ce.ld;
    const int nb = lbeg[cb + 1] - lbeg[cb], nk = lbeg[ck + 1] - lbeg[ck];
    if (!nb || !nk) continue;
    ClassLaunch cl{dlist + lbeg[cb], dlist + lbeg[ck], nb, nk, cb == ck, 0.f, 0.f};
    NA_TRY(ce.tensor(g, t, cl, st));
  }
#undef NA_TRY
  return MMDG_OK;
}
