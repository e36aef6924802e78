/*
 * mmdg.h -- C ABI of the GB300-native McMurchie-Davidson two-electron hot path.
 *
 * Plain C: device pointers, host arrays, sizes and an opaque context.  No torch or
 * C++ types cross this boundary; a ctypes/cffi/cgo caller binds it directly.
 * Every entry point returns 0 on success or a negative MMDG_E* code; the text of
 * the last failure on the calling thread is available from mmdg_last_error().
 *
 * Each entry point replaces one interface of jjgoings/McMurchie-Davidson (cited
 * as file:line within that project):
 *
 *   mmdg_set_basis    <- Basis construction (cython/basis.pxi:46-120) and the
 *                        list-of-Basis argument of doERIs/formPT (cython/twoe.pyx:12,
 *                        cython/fock.pyx:13): the function list is grouped into
 *                        shells and turned into primitive-pair data on the GPU.
 *   mmdg_get_screen   <- the Schwarz dict of Molecule.build(direct=True)
 *                        (mmd/molecule.py:95-99): screen[p(p+1)/2+q] = (pq|pq).
 *   mmdg_eri_tensor   <- doERIs (cython/twoe.pyx:12-31) / Molecule.two_electron_integrals
 *                        (mmd/molecule.py:288-293): the full N^4 ERI tensor.
 *   mmdg_fock         <- formPT (cython/fock.pyx:13-87): unsymmetrised two-electron
 *                        Fock update G(P - P_old) with Schwarz x density screening.
 *   mmdg_set_screen   <- the `screen` argument of formPT (cython/fock.pyx:13,46-47).
 *   mmdg_jk_dense     <- the conventional J/K einsums of buildFock (mmd/scf.py:97-98).
 *   mmdg_fock_update  <- G = (G + G^T)/2, F = F_old + G of buildFock (mmd/scf.py:91-94).
 *   mmdg_one_electron <- S, T, V, Mu of cython/onee.pyx:14-192 as assembled by
 *                        Molecule.one_electron_integrals (mmd/molecule.py:235-276).
 *   mmdg_boys         <- boys / the _boys test hook (cython/util.pxi:54-55,
 *                        cython/onee.pyx:195-196).
 *   mmdg_eri_quartets <- ERI(a, b, c, d) (cython/twoe.pyx:36-50) for whole shells:
 *                        every component of listed shell quartets.
 *   mmdg_set_partition <- the bra-pair loop of formPT (cython/fock.pyx:38-44) split
 *                        over GPUs: each rank digests the shell quartets it owns.
 *   mmdg_ao2mo        <- the AO -> MO transform of PostSCF.ao2mo (mmd/postscf.py:26-27).
 */
#ifndef MMDG_H
#define MMDG_H

#ifdef __cplusplus
extern "C" {
#endif

#define MMDG_OK 0
#define MMDG_E_ARG (-1)      /* invalid argument (null pointer, bad size, bad shell data) */
#define MMDG_E_LMAX (-2)     /* angular momentum above the supported maximum (d, l = 2) */
#define MMDG_E_CUDA (-3)     /* a CUDA runtime call failed */
#define MMDG_E_STATE (-4)    /* call order: no basis set yet, or wrong molecule layout */
#define MMDG_E_NOMEM (-5)    /* device allocation failed */

#define MMDG_LMAX 2          /* highest shell angular momentum (Cartesian d) */
#define MMDG_MAX_COMP 6      /* Cartesian components of a d shell */
#define MMDG_NCLASS 21       /* angular classes (la lb|lc ld), la>=lb, lc>=ld, (la,lb)>=(lc,ld) */
#define MMDG_NCOUNT 5        /* per-class counters of a Fock build (mmdg_fock counts) */

typedef struct mmdg_context mmdg_context;

/* Thread-local text of the last failure ("" if none). */
const char* mmdg_last_error(void);

/* Create a context on CUDA device `device` (allocates its Boys tables). */
int mmdg_create(mmdg_context** out, int device);
int mmdg_destroy(mmdg_context* ctx);

/*
 * Set the basis of one or more molecules (host arrays) and build, on the device,
 * the primitive-pair data and the Schwarz table.  Synchronous.
 *
 *   nmol               number of molecules (1 for a single system)
 *   mol_nfunc[nmol]    basis functions N_m of each molecule
 *   nshell             number of shells over all molecules
 *   shell_mol[s]       molecule of shell s (shells of a molecule are contiguous)
 *   shell_L[s]         angular momentum 0..MMDG_LMAX
 *   shell_nprim[s]     primitives (>= 1)
 *   shell_center[3s]   centre, bohr
 *   prim_exp[], prim_coef[]  primitives of all shells, shell after shell; prim_coef is
 *                      the contraction coefficient times the contracted normalisation
 *                      times the primitive normalisation of an x^L Cartesian
 *                      component (the per-component factor 1/sqrt((2l-1)!!(2m-1)!!(2n-1)!!)
 *                      is applied inside)
 *   shell_func[6s+c]   molecule-local function index of Cartesian component c
 *                      (order xx,xy,xz,yy,yz,zz for d; x,y,z for p), or -1 if that
 *                      component is not part of the basis
 */
int mmdg_set_basis(mmdg_context* ctx, int nmol, const int* mol_nfunc, int nshell, const int* shell_mol,
                   const int* shell_L, const int* shell_nprim, const double* shell_center, const double* prim_exp,
                   const double* prim_coef, const int* shell_func);

/* Copy the Schwarz table (pq|pq), packed per molecule as N_m(N_m+1)/2 entries
 * in row order p(p+1)/2+q, to the host array `screen` of length n. */
int mmdg_get_screen(mmdg_context* ctx, double* screen, long long n);

/* Replace the Schwarz table by the caller's values (same layout as mmdg_get_screen),
 * as formPT takes its `screen` dict from the caller (cython/fock.pyx:13,46-47);
 * the per-shell-pair bounds are recomputed from it. */
int mmdg_set_screen(mmdg_context* ctx, const double* screen, long long n);

/* Full ERI tensor of molecule 0: out is a device array of N^4 doubles (C order). */
int mmdg_eri_tensor(mmdg_context* ctx, double* out, void* stream);

/*
 * ERIs of listed shell quartets (the reference's ERI(a, b, c, d) of
 * cython/twoe.pyx:36-50, applied to every Cartesian component of four shells at once).
 *   shells   host array of 4n global shell indices (a, b, c, d) in the order of
 *            mmdg_set_basis; the four shells of a quartet belong to one molecule
 *   out      device array of n * 1296 doubles: block q holds (ab|cd) at
 *            out[q*1296 + ((ca*6 + cb)*6 + cc)*6 + cd] for the components ca of a, cb of
 *            b, ... in the component order of mmdg_set_basis; entries beyond a shell's
 *            component count are zero
 *   precision 0: the FP64 class code (the plain method); 1: the FP32 class code that
 *            mixed-precision Fock builds use for quartets below their threshold (its
 *            results widened to double), for measuring that path's per-ERI error
 * Synchronises `stream` before returning.
 */
int mmdg_eri_quartets(mmdg_context* ctx, long long n, const int* shells, double* out, int precision, void* stream);

/*
 * Sharded direct Fock build: the bra-pair loop of formPT (cython/fock.pyx:38-44)
 * split over `nparts` ranks (one GPU each).  After this call, mmdg_fock and
 * mmdg_fock_graph of this context digest only the shell quartets of part `part`; the
 * parts' G add up to the full G (one all-reduce per build).  pair_owner (host,
 * npairs = the context's shell pairs) gives the owner of every shell pair in
 * canonical order -- per molecule, s1 ascending, then s2 from the molecule's first
 * shell to s1 -- and a shell quartet belongs to the owner of its pair with the larger
 * canonical index s1(s1+1)/2 + s2 (molecule-local shells).  nparts = 1 switches
 * sharding off (pair_owner may be NULL).
 */
int mmdg_set_partition(mmdg_context* ctx, int part, int nparts, const int* pair_owner, long long npairs);

/* Device bytes held by a context (its buffers; the quartet lists once a Fock build
 * has allocated them).  For caches of contexts; no counterpart in the reference. */
int mmdg_device_bytes(mmdg_context* ctx, long long* bytes);

/*
 * Direct two-electron Fock update (formPT semantics).
 *   dP        device, packed per-molecule N_m x N_m blocks: P - P_old (real)
 *   G         device, same layout; overwritten with the unsymmetrised update
 *   tol       screening threshold (acc2e of RHF; reference default 1e-12)
 *   fp32_below  shell quartets whose Schwarz bound Q_ab*Q_cd is below this value are
 *             evaluated in FP32 (0 = all FP64, the plain method)
 *   counts    optional host array of MMDG_NCOUNT*MMDG_NCLASS unsigned long long: per
 *             class the digested function quartets, shell quartets, primitive quartets,
 *             bra-primitive passes and primitive quartets whose Boys function took the
 *             asymptotic branch (filled after a stream synchronisation; pass NULL to
 *             stay asynchronous)
 */
int mmdg_fock(mmdg_context* ctx, const double* dP, double* G, double tol, double fp32_below,
              unsigned long long* counts, void* stream);

/* mmdg_fock with CUDA events around every class launch: class_ms[MMDG_NCLASS]
 * receives each class's device time in ms (synchronises the stream).  Measurement
 * support; no counterpart in the reference. */
int mmdg_fock_timed(mmdg_context* ctx, const double* dP, double* G, double tol, double fp32_below,
                    unsigned long long* counts, float* class_ms, void* stream);

/* FP64 (DFMA) and FP32 (FFMA) throughput of this GPU in TFLOP/s, from independent
 * FMA chains on every SM: the roofline denominators of the ERI kernels.
 * Measurement support; no counterpart in the reference. */
int mmdg_measure_peaks(mmdg_context* ctx, double* fp64_tflops, double* fp32_tflops);

/* The FP64 pipes of this GPU, with `warps_per_sm` warps per SM: res[0] = DFMA
 * TFLOP/s (8 independent FMA chains per thread), res[1] = FP64 tensor-core TFLOP/s
 * (8 independent mma.sync m8n8k4 f64 chains per warp), res[2..4] = the device times
 * (ms) of the DFMA kernel, the tensor-core kernel and one kernel issuing both
 * streams: res[4] near max(res[2], res[3]) means the two overlap, near the sum that
 * they share one resource.  Measurement support; no counterpart in the reference. */
int mmdg_measure_fp64_pipes(mmdg_context* ctx, int warps_per_sm, double* res);

/* Host copy of the Boys interpolation table (no GPU needed): rows (L, k) of
 * F_{L+n}(k/16)/n! (n = 0..6, 8 doubles per row, L = 0..8, k = 0..767) followed by
 * rows k of exp(-k/16)/n! (n = 0..7).  With out = NULL returns the length; else
 * fills out[0..n) and returns the length, or a negative error code.  Test support. */
long long mmdg_boys_table(double* out, long long n);

/* Autotuner hooks (no counterpart in the reference).  mmdg_set_tuning sets the
 * persistent grid of angular class `cls` (0..MMDG_NCLASS-1, the order of the class
 * table: (ss|ss), (ps|ss), (ps|ps), (pp|ss), ...; 0 = one full wave at the kernel's
 * occupancy); mmdg_set_streams spreads the classes (screening and evaluation) over
 * 1..8 concurrent streams (fork/join on events). */
int mmdg_set_tuning(mmdg_context* ctx, int cls, int grid_blocks);
/* Tile of class `cls`'s Fock kernel (no counterpart in the reference): threads per
 * block of the one-thread-per-quartet kernels (64, 128 or 256; the classes whose
 * Hermite tables live in shared memory keep 128) and the largest number of list
 * quartets a warp takes per work item in the warp-cooperative high-L kernels (1..8,
 * whose Boys functions are evaluated together); 0 restores the default. */
int mmdg_set_tile(mmdg_context* ctx, int cls, int block_threads, int item);
int mmdg_set_streams(mmdg_context* ctx, int nstreams);

/* Primitive-pair screening of the next mmdg_set_basis (no counterpart in the
 * reference, which sums every primitive quartet, cython/twoe.pyx:36-50): a primitive
 * pair whose Schwarz factor q = max sqrt((a_i b_j|a_i b_j)) (contraction weights
 * included) satisfies q * q_max < tol is not stored, so no contracted ERI moves by
 * more than (primitive quartets per shell quartet) * tol.  Default 1e-18; 0 keeps
 * every primitive pair. */
int mmdg_set_prim_tol(mmdg_context* ctx, double tol);

/* Analytic RHF nuclear gradient dE/dR (replaces the Forces.forces loops of
 * mmd/forces.py:8-97 with their ERIx/Sx/Tx/VxA/VxB derivative integrals,
 * cython/grad.pyx:11-330): P and W = P F P are the converged density and
 * energy-weighted density (device, N x N, the reference's P = C_occ C_occ^T);
 * atom_xyz (bohr, natom x 3), atom_Z and shell_atom (the atom of every shell of the
 * basis) are host arrays; grad (host, natom x 3) receives dE/dR including the nuclear
 * repulsion (the reference's forces are -grad).  Shell quartets with Schwarz bounds
 * Q_ab Q_cd < qtol are skipped (0: none; the reference skips none).  One molecule per
 * context. */
int mmdg_rhf_gradient(mmdg_context* ctx, const double* P, const double* W, int natom, const double* atom_xyz,
                      const double* atom_Z, const int* shell_atom, double qtol, double* grad, void* stream);

/* mmdg_fock replayed as one CUDA graph: the first call with a given (dP, G, tol,
 * fp32_below) runs the build eagerly and captures its launches (screening, class
 * kernels over all molecules, memsets) into a graph; later calls with the same
 * arguments launch that graph on `stream`.  Used by the batched SCF, where one
 * launch serves every molecule of the batch. */
int mmdg_fock_graph(mmdg_context* ctx, const double* dP, double* G, double tol, double fp32_below, void* stream);

/*
 * Learned initial guess: kernels of the density-block MLP (no counterpart in the
 * reference, which starts every SCF from P = 0, mmd/scf.py:15,23-24).  BF16 weights,
 * FP32 activations and accumulation; all pointers are device pointers.
 *   mmdg_mlp_gemm      C[M,N] = op(A) op(B) + beta C; op transposes when ta/tb != 0
 *                      (A stored K x M / B stored N x K); a_bf16 / b_bf16 mark a
 *                      BF16 operand (at most one)
 *   mmdg_mlp_bias_act  Z += b (per column), Y = silu(Z) (silu != 0) or Y = Z
 *   mmdg_mlp_act_grad  dZ = dY * silu'(Z) (or dY)
 *   mmdg_mlp_colsum    db[c] = sum_r dZ[r, c]
 *   mmdg_mlp_mse       dY = 2 (Y - T) mask / count; *loss += sum ((Y - T) mask)^2 / count
 *   mmdg_mlp_adam      Adam step on FP32 master weights, refreshing their BF16 copy
 *   mmdg_mlp_to_bf16   BF16 copy of FP32 weights
 */
int mmdg_mlp_gemm(int M, int N, int K, const void* A, int lda, int ta, int a_bf16, const void* B, int ldb, int tb,
                  int b_bf16, float* C, int ldc, float beta, void* stream);
int mmdg_mlp_bias_act(float* Z, float* Y, const float* b, long long rows, int cols, int silu, void* stream);
int mmdg_mlp_act_grad(const float* Z, const float* dY, float* dZ, long long n, int silu, void* stream);
int mmdg_mlp_colsum(const float* dZ, float* db, long long rows, int cols, void* stream);
int mmdg_mlp_mse(const float* Y, const float* T, const float* mask, float* dY, double* loss, long long n,
                 float inv_count, void* stream);
int mmdg_mlp_adam(float* w, void* w_bf16, const float* g, float* m, float* v, long long n, float lr, float b1,
                  float b2, float eps, int step, void* stream);
int mmdg_mlp_to_bf16(const float* w, void* w_bf16, long long n, void* stream);

/* AO -> MO transform of an ERI tensor (mmd/postscf.py:26-27, four einsums with the MO
 * coefficients): eri_out[P,Q,R,S] = sum_pqrs C[p,P] C[q,Q] C[r,R] C[s,S] eri_in[p,q,r,s].
 * All device arrays, C order: C is N x N (AO row, MO column), eri_in / eri_out / work
 * are N^4 and distinct; eri_in is left unchanged, work is scratch.  Four FP64 quarter
 * transforms (each contracts the last index and writes the new one first). */
int mmdg_ao2mo(long long N, const double* C, const double* eri_in, double* eri_out, double* work, void* stream);

/* The ERI kernels' reciprocal square root (an FP32 estimate refined by one
 * third-order FP64 step) and CUDA's rsqrt at n points, for x in the normal float
 * range (device arrays).  Test support; no counterpart in the reference. */
int mmdg_rsqrt(mmdg_context* ctx, long long n, const double* x, double* ours, double* cuda, void* stream);

/* Boys function F_m(T) for integer 0 <= m <= 8 at n points (device arrays). */
int mmdg_boys(mmdg_context* ctx, int m, long long n, const double* T, double* out, void* stream);

/* Symmetrised incremental Fock update of packed per-molecule blocks:
 * F_out = F_in + (G + G^T)/2   (mmd/scf.py:91-94). Device arrays; F_out may alias F_in. */
int mmdg_fock_update(mmdg_context* ctx, const double* G, const double* F_in, double* F_out, void* stream);

/* Conventional Coulomb and exchange matrices from a dense ERI tensor
 * (mmd/scf.py:97-98):  J_pq = sum_rs (pq|rs) P_sr,  K_pq = sum_rs (ps|qr) P_sr.
 * All device arrays: T is N^4, P, J, K are N x N. */
int mmdg_jk_dense(mmdg_context* ctx, long long N, const double* T, const double* P, double* J, double* K,
                  void* stream);

/* One-electron integrals S, T, V and the dipole integrals M (3 blocks) of every
 * molecule, packed like mmdg_fock's G (cython/onee.pyx:14-192, assembled as
 * Molecule.one_electron_integrals, mmd/molecule.py:235-276).  Atoms sorted by
 * molecule: atom_mol[natom], atom_xyz[3*natom] (bohr), atom_Z[natom]; origin[3*nmol]
 * is the dipole gauge origin of each molecule.  Outputs are device arrays of
 * sum N_m^2 doubles (M: 3 x that). */
int mmdg_one_electron(mmdg_context* ctx, int natom, const int* atom_mol, const double* atom_xyz,
                      const double* atom_Z, const double* origin, double* S, double* T, double* V, double* M,
                      void* stream);

/*
 * ERI tensor of one small molecule that allocates nothing -- no cudaMalloc, no
 * cudaFree, no host heap.  No counterpart in the reference (it has no device
 * memory to manage); this is mmdg_eri_tensor for callers that cannot allocate:
 * host frameworks that own the whole GPU memory pool and forbid outside
 * allocations, code that must not synchronise the device (cudaMalloc/cudaFree can),
 * and services that cannot recover from an allocation failure mid-request.
 *
 * Same basis arguments as mmdg_set_basis for one molecule (nfunc functions; no
 * context needed) and a caller-owned device output `out` of nfunc^4 doubles.
 * All scratch (Boys table, primitive pairs, E' tables, bookkeeping) lives in one
 * static device array of 1,738,240 bytes that every GPU loading the library holds
 * until the process exits.  Limits: 64 shells, 64 functions, 256 primitives, 4096
 * primitive pairs, 131072 E' coefficients, l <= 2; larger inputs fail with
 * MMDG_E_ARG and a message naming the limit; so do non-finite exponents,
 * coefficients or centres.  The first call on a device (the device current) looks
 * up the array's device address and uploads the Boys table; make that first call
 * before any stream capture.  Later calls look the address up again and read back a
 * set-up stamp kept in the array, repeating the set-up when the array is new (after
 * a cudaDeviceReset).  Every call shares the array: calls that overlap on the GPU
 * (other streams, other threads) race and must be serialised by the caller; host
 * threads are serialised inside.  The call synchronises `stream` twice: after
 * reading the stamp and after staging its inputs.
 */
int mmdg_eri_tensor_noalloc(int nshell, const int* shell_L, const int* shell_nprim, const double* shell_center,
                            const double* prim_exp, const double* prim_coef, const int* shell_func, int nfunc,
                            double* out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MMDG_H */
