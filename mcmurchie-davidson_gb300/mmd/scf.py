"""RHF driver (mmd/scf.py) with the two-electron work on the GPU.

``RHF(doPrint=True, DIIS=True, direct=False, conver=1e-8, acc2e=1e-12)`` keeps the
reference's algorithm step for step (mmd/scf.py:10-80):

* start from P = 0, F = Core (core-Hamiltonian guess);
* direct SCF: incremental Fock build F = F_old + sym(G(P - P_old)) with G from the
  formPT kernel (Schwarz x density screening at ``acc2e``), never reset;
  conventional: F = Core + 2J - K from the ERI tensor;
* 8-deep DIIS on X (FPS - SPF) X, eigensolve of X^T F X, P = C_occ C_occ^T,
  E = tr((Core + F) P) + E_nuc, stop when ||P - P_old||_F < ``conver``.

Every matrix stays on the device (float64): the Fock build and update run in
libmmdg.so, the DIIS products in cuBLAS through torch; the (n+1)^2 DIIS system and
the eigensolve of X^T F X run on the host cores (LAPACK dsyevd up to
HOST_EIGH_MAX_N = 1024 functions, where it beats cuSOLVER; cuSOLVER above).  Extra
keyword arguments (all default to the reference's behaviour):

* ``fp32_below``  Schwarz-bound threshold under which shell quartets run in FP32
  (0: plain FP64 method);
* ``guess``       initial density (N x N array) instead of P = 0, with a full first
  Fock build F = Core + sym(G(P_guess));
* ``guess_fallback``  with a guess: revert to the core guess when the DIIS error
  grows for 3 consecutive iterations;
* ``maxiter``     iteration cap (reference: 100);
* ``polish``      the final energy from one non-incremental Fock build of the
  converged density (second order in the density error); ``polish_fp32_below`` lets
  that build run in FP32 below its own, smaller threshold;
* ``eigensolver``  "dense" (all eigenpairs every iteration, as the reference) or
  "subspace" (occupied orbitals by Chebyshev-filtered subspace iteration between
  iterations, all eigenpairs once at the end; ``OccupiedSubspace``);
* ``process_group``  a torch.distributed group with one rank per GPU: each rank
  digests its share of the shell quartets and one all-reduce of G completes every
  Fock build (``mmd.distributed``); the rest of the SCF is replicated.
"""
from __future__ import annotations

import time

import numpy as np

# dense symmetric eigensolver of the SCF: host LAPACK up to this size, cuSOLVER above
HOST_EIGH_MAX_N = 1024


def host_eigh(A):
    """One symmetric eigensolve on the host cores: LAPACK dsyevd through SciPy (on the
    16-core Grace CPU 0.64 ms at N = 104 against 2.8 ms for numpy.linalg.eigh; 7.4 ms at
    N = 400 and 28 ms at N = 800, where cuSOLVER's syevd takes 11.8 and 31 ms).  Many
    small solves at once (the batched SCF) stay on numpy.linalg.eigh in a thread pool:
    SciPy's wrapper serialises there (1.14 s against 0.45 s for 1024 matrices)."""
    import scipy.linalg
    return scipy.linalg.eigh(A, driver="evd", check_finite=False)


class OccupiedSubspace:
    """The lowest ``nocc`` eigenpairs of the orthogonalised Fock matrix FO by
    Chebyshev-filtered subspace iteration (Y. Zhou, Y. Saad, M. L. Tiago and J. R.
    Chelikowsky, "Self-consistent-field calculations using Chebyshev-filtered subspace
    iteration", J. Comput. Phys., 2006), warm-started from the previous SCF iteration's
    Ritz vectors.

    Between SCF iterations only the occupied orbitals are needed (P = C_occ C_occ^T);
    a dense eigensolve of all N orbitals costs 7-10 ms on the host cores at N = 400,
    one pass here a few dozen GEMMs of N x N x k on the GPU (k = nocc + a buffer) and
    one k x k generalised eigensolve on the host.  One pass:

    1. filters.  p_m(FO) with p_m the degree-m Chebyshev polynomial of the first kind
       mapped onto [a, b] and scaled to 1 at the bottom of the slice (three-term
       recurrence), b an upper bound of the spectrum -- the largest eigenvalue of the
       last dense solve plus ||FO - FO_dense||_F (Weyl's inequality) -- and a the
       cut-off below which the polynomial amplifies.  The occupied spectrum of a
       molecule with heavy atoms is wide (O 1s near -20.6 Eh, the HOMO near -0.5 Eh),
       and one polynomial would amplify the core ~1e12 times more than the HOMO, which
       no Rayleigh-Ritz in FP64 recovers.  So the block is cut into two slices: the
       core (Ritz values whose amplification exceeds the HOMO's by more than
       ``spread``), filtered on [lowest valence value, b] with degree ``core_degree``,
       and the valence + buffer, filtered on [top of the block, b] with degree
       ``degree`` in the complement of the core (each product by FO is projected:
       Z - V_c V_c^T Z);
    2. Rayleigh-Ritz over both slices: columns normalised, H = Y^T FO Y and M = Y^T Y
       solved on the host (H z = theta M z), V = Y Z;
    3. residuals ||FO v - theta v|| of the occupied Ritz pairs; another pass while the
       largest is above ``tol``.

    After ``max_passes`` the caller falls back to the dense solve (``start`` again),
    so a poor warm start (a guess reverted to the core guess) costs time, not
    accuracy."""

    def __init__(self, nocc: int, nbuf: int = 0, degree: int = 10, core_degree: int = 4, tol: float = 1e-8,
                 max_passes: int = 4, spread: float = 1e3):
        self.nocc = int(nocc)
        self.k = int(nocc) + int(nbuf if nbuf > 0 else self.buffer(nocc))
        self.degree = int(degree)
        self.core_degree = int(core_degree)
        self.tol = float(tol)
        self.max_passes = int(max_passes)
        self.log_spread = float(np.log(spread))
        self.V = None
        self.passes = 0
        self.solves = 0
        self.fallbacks = 0

    @staticmethod
    def buffer(nocc: int) -> int:
        return max(8, nocc // 4)

    @staticmethod
    def applicable(n: int, nocc: int) -> bool:
        return n >= 64 and nocc + OccupiedSubspace.buffer(nocc) <= n // 2

    def start(self, FO, w, v):
        """Warm start from a dense solve of FO (device matrix; host eigenpairs w, v)."""
        import torch
        self.V = torch.as_tensor(np.ascontiguousarray(v[:, : self.k]), device=FO.device)
        self.theta = np.array(w[: self.k])
        self.lmin, self.lmax = float(w[0]), float(w[-1])
        self.F_dense = FO.clone()

    @staticmethod
    def _log_cheb(m, t):
        """log |T_m(t)| for |t| >= 1 (0 inside [-1, 1], where |T_m| <= 1)."""
        t = np.abs(np.asarray(t, dtype=float))
        return np.where(t > 1.0, m * np.arccosh(np.maximum(t, 1.0)), 0.0)

    def core_count(self, theta, a, b):
        """Number of lowest Ritz values whose amplification by the valence filter
        exceeds the HOMO's by more than the allowed spread."""
        e, c = 0.5 * (b - a), 0.5 * (b + a)
        lg = self._log_cheb(self.degree, (theta - c) / e)
        over = lg[: self.nocc] - lg[self.nocc - 1] > self.log_spread
        return int(np.argmin(over)) if not over.all() else 0

    @staticmethod
    def _filter(FO, X, a, b, lo, m, Vc=None):
        """p_m(FO) X: Chebyshev filter on [a, b] scaled to 1 at ``lo`` (< a); products by
        FO projected onto the complement of Vc's columns when given."""
        import torch

        def apply(Z):
            FZ = FO @ Z
            if Vc is not None:
                FZ = FZ - Vc @ (Vc.T @ FZ)
            return FZ

        e, c = 0.5 * (b - a), 0.5 * (b + a)
        sigma = e / (lo - c)
        tau = 2.0 / sigma
        Y = (apply(X) - c * X) * (sigma / e)
        for _ in range(2, m + 1):
            s1 = 1.0 / (tau - sigma)
            Yn = apply(Y).sub_(Y, alpha=c).mul_(2.0 * s1 / e).sub_(X, alpha=sigma * s1)
            X, Y, sigma = Y, Yn, s1
        if Vc is not None:
            Y = Y - Vc @ (Vc.T @ Y)
        return Y

    def solve(self, FO):
        """(theta_occ on the host, V_occ on the device) of FO, or None when the passes
        did not converge (then call ``start`` with a dense solve)."""
        import scipy.linalg
        import torch
        if self.V is None:
            return None
        dF = float(torch.linalg.norm(FO - self.F_dense))
        b = self.lmax + dF
        lo = self.lmin - dF
        V, theta = self.V, self.theta
        for _ in range(self.max_passes):
            self.passes += 1
            a = float(theta[-1])
            if not (lo < float(theta[0]) and a < b):
                break
            nc = self.core_count(theta, a, b)
            if nc:
                Vc = V[:, :nc]
                Yc = self._filter(FO, Vc, float(theta[nc]), b, lo, self.core_degree)
                Yv = self._filter(FO, V[:, nc:], a, b, float(theta[nc]) - dF, self.degree, Vc)
                Y = torch.cat((Yc, Yv), dim=1)
            else:
                Y = self._filter(FO, V, a, b, lo, self.degree)
            Y = Y / torch.linalg.norm(Y, dim=0)
            FY = FO @ Y
            HM = torch.stack((Y.T @ FY, Y.T @ Y)).cpu().numpy()
            H = 0.5 * (HM[0] + HM[0].T)
            M = 0.5 * (HM[1] + HM[1].T)
            try:
                theta, Z = scipy.linalg.eigh(H, M, check_finite=False)
            except (np.linalg.LinAlgError, ValueError):
                break
            Zd = torch.as_tensor(Z, device=FO.device)
            V = Y @ Zd
            R = FY @ Zd[:, : self.nocc] - V[:, : self.nocc] * torch.as_tensor(theta[: self.nocc], device=FO.device)
            res = float(torch.linalg.norm(R, dim=0).max())
            if res < self.tol:
                self.V, self.theta = V, theta
                self.solves += 1
                return theta[: self.nocc], V[:, : self.nocc]
        self.fallbacks += 1
        self.V = None
        return None


# an initial guess is abandoned (restart from the core guess) when the DIIS error
# has grown this many iterations in a row
GUESS_FALLBACK_GROWTH = 3


def diis_error_growing(history, times=GUESS_FALLBACK_GROWTH):
    """True where the last ``times`` DIIS errors each grew (history: list of scalars
    or of equally shaped arrays, oldest first); False while the history is shorter."""
    if len(history) < times + 1:
        return np.zeros(np.shape(history[-1]) if history else (), dtype=bool)
    h = np.asarray(history[-(times + 1):], dtype=float)
    return np.all(h[1:] > h[:-1], axis=0)


class SCF(object):
    """SCF methods for the molecule object (mmd/scf.py:8-180)."""

    def RHF(self, doPrint=True, DIIS=True, direct=False, conver=1e-8, acc2e=1e-12, fp32_below=0.0, guess=None,
            guess_fallback=True, maxiter=100, polish=False, process_group=None, polish_fp32_below=0.0,
            eigensolver="dense"):
        """Restricted Hartree-Fock (mmd/scf.py:10-80): core-Hamiltonian start (or the
        density ``guess``, abandoned for the core guess after three growing DIIS
        errors when ``guess_fallback``), DIIS, stop on ||P - P_old||_F < conver.
        ``direct``: incremental formPT-semantics Fock builds with Schwarz x density
        screening at ``acc2e``; ``fp32_below``: shell quartets with Schwarz bound below
        it in FP32; ``polish``: the returned energy from one non-incremental build of
        the final density (FP64, or FP32 below ``polish_fp32_below``), exact to second
        order in the density error -- a density converged to 1e-5 gives the energy to
        ~1e-11 Eh; ``eigensolver="subspace"``: the occupied orbitals of every iteration
        after the first by Chebyshev-filtered subspace iteration on the GPU
        (``OccupiedSubspace``, residuals below conver / 1000), the full set once at the
        end.  Returns the energy (a numpy float64)."""
        state = self.scf_begin(DIIS=DIIS, direct=direct, acc2e=acc2e, fp32_below=fp32_below, guess=guess,
                               guess_fallback=guess_fallback, maxiter=maxiter, process_group=process_group,
                               eigensolver=eigensolver, subspace_tol=min(1e-8, max(1e-12, 1e-3 * conver)))
        t_start = time.perf_counter()
        for step in range(self.maxiter):
            state.iterate()
            if np.abs(self.P_RMS) < conver or step == (self.maxiter - 1):
                if step == (self.maxiter - 1):
                    print("NOT CONVERGED")
                else:
                    self.is_converged = True
                break
        self.iterations = step
        self.scf_time = time.perf_counter() - t_start
        state.finish()
        if polish and self.is_converged:
            self.energy = np.float64(self.polished_energy(polish_fp32_below))
            self.el_energy = self.energy - self.nuc_energy
        if self.is_converged:
            FPS = self.F @ self.P @ self.S
            error = FPS - FPS.T
            self.computeDipole()
            if doPrint:
                print("E(SCF)    = ", "{0:.12f}".format(self.energy.real) + " in " + str(step) + " iterations")
                print("  Convergence:")
                print("    FPS-SPF  = ", np.linalg.norm(error))
                print("    RMS(P)   = ", "{0:.2e}".format(self.P_RMS))
                print("    dE(SCF)  = ", "{0:.2e}".format(self.delta_energy))
                print("  Dipole X = ", "{0:.8f}".format(self.mu[0].real))
                print("  Dipole Y = ", "{0:.8f}".format(self.mu[1].real))
                print("  Dipole Z = ", "{0:.8f}".format(self.mu[2].real))
        return self.energy

    def scf_begin(self, DIIS=True, direct=False, acc2e=1e-12, fp32_below=0.0, guess=None, guess_fallback=True,
                  maxiter=100, build=True, process_group=None, eigensolver="dense", subspace_tol=1e-8):
        """Integrals and the initial state of an RHF run; returns the iteration object."""
        self.is_converged = False
        self.delta_energy = 1e20
        self.P_RMS = 1e20
        self.maxiter = int(maxiter)
        self.direct = direct
        if self.direct:
            self.incFockRst = False
        self.scrTol = acc2e
        self.fp32_below = float(fp32_below)
        if build or not getattr(self, "is_built", False):
            self.build(self.direct)
        self._set_sharding(process_group if direct else None)
        if eigensolver not in ("dense", "subspace"):
            raise ValueError("eigensolver must be 'dense' or 'subspace'")
        sub = None
        if eigensolver == "subspace" and OccupiedSubspace.applicable(self.nbasis, self.nocc):
            sub = OccupiedSubspace(self.nocc, tol=subspace_tol)
        self.subspace = sub
        return _RHFState(self, DIIS, guess, guess_fallback, sub)

    def _set_sharding(self, group):
        """Sharded Fock builds over ``group`` (one GPU per rank), or none."""
        old = getattr(self, "_sharded", None)
        if old is not None:
            old.close()
            self._sharded = None
        if group is not None:
            import torch.distributed as dist
            if dist.get_world_size(group) > 1:
                from .distributed import ShardedFock
                self._sharded = ShardedFock(self.context, group)
                return
        if self.context.nparts > 1:  # a shared context left sharded by another run
            self.context.set_partition(0, 1)

    def _fock_build(self, dP, tol, fp32_below):
        """Unsymmetrised G(dP) of the whole molecule (sharded over ranks if set up)."""
        sh = getattr(self, "_sharded", None)
        if sh is not None:
            return sh.fock(dP, tol=tol, fp32_below=fp32_below)
        return self.context.fock(dP, tol=tol, fp32_below=fp32_below)

    def polished_energy(self, fp32_below=0.0):
        """E(P) = tr((H + F(P)) P) + E_nuc from one non-incremental Fock build of the
        current density (an extension: the reference's energy pairs P with the Fock
        matrix of the previous density, an error first order in the last change of P;
        this one is second order in the density error).  The build is FP64, or FP32
        for shell quartets whose Schwarz bound is below ``fp32_below`` (each such ERI
        is off by at most 5e-7 times its bound, measured)."""
        ctx = self.context
        torch = ctx.torch
        Core = self._dev["Core"]
        P = torch.as_tensor(np.ascontiguousarray(np.real(np.asarray(self.P)), dtype=np.float64), device=Core.device)
        if getattr(self, "direct", False):
            G = self._fock_build(P.reshape(-1), self.scrTol, float(fp32_below)).view(self.nbasis, self.nbasis)
            F = Core + 0.5 * (G + G.T)
        else:
            F = self._conventional_fock(P)
        return float(torch.sum((Core + F) * P.T).item()) + self.nuc_energy

    # ---------------------------------------------------------------- pieces
    def _two_electron(self, P, P_old, symmetrize=True):
        """G(P - P_old) on the GPU (formPT semantics), symmetrised (G + G^T)/2 unless
        the caller does that itself (mmdg_fock_update)."""
        ctx = self.context
        t0 = time.perf_counter()
        dP = (P - P_old).contiguous().view(-1)
        prof = getattr(self, "_fock_profile", None)
        if prof is not None and getattr(self, "_sharded", None) is None:  # per-class times and counts
            G, ms, cnt = ctx.fock_timed(dP, tol=self.scrTol, fp32_below=self.fp32_below)
            prof["class_ms"] = prof.get("class_ms", 0.0) + ms.astype(np.float64)
            prof["counts"] = prof.get("counts", 0) + cnt.astype(np.float64)
            prof["builds"] = prof.get("builds", 0) + 1
        else:
            G = self._fock_build(dP, self.scrTol, self.fp32_below)
        self.fock_builds += 1
        self.fock_time += time.perf_counter() - t0
        G = G.view(self.nbasis, self.nbasis)
        return 0.5 * (G + G.T) if symmetrize else G

    def _conventional_fock(self, P):
        ctx = self.context
        torch = ctx.torch
        J = torch.empty_like(P)
        K = torch.empty_like(P)
        ctx.jk_dense(self._TwoE_dev, P.contiguous(), J, K)
        self.fock_builds += 1
        self._last_jk = (J, K)  # the reference leaves the last J and K on the molecule
        return self._dev["Core"] + 2.0 * J - K

    def _diis(self, F, P, S, X, fockSet, errorSet):
        """DIIS extrapolation (mmd/scf.py:146-180); returns (F_diis, ||error||)."""
        torch = self.context.torch
        FPS = F @ P @ S
        error = X @ (FPS - FPS.T) @ X
        fockSet.append(F)
        errorSet.append(error)
        if len(fockSet) > 8:
            del fockSet[0]
            del errorSet[0]
        n = len(fockSet)
        E = torch.stack(errorSet).reshape(n, -1)
        # the (n+1) x (n+1) DIIS system is solved on the host: one small copy back
        # (which also yields ||error|| from the Gram diagonal) instead of a device
        # solver call and a second synchronisation
        gram = (E @ E.T).cpu().numpy()
        B = -np.ones((n + 1, n + 1))
        B[:n, :n] = gram
        B[n, n] = 0.0
        rhs = np.zeros(n + 1)
        rhs[n] = -1.0
        w = np.linalg.solve(B, rhs)
        wd = torch.as_tensor(w[:n], dtype=torch.float64, device=F.device)
        Fd = torch.tensordot(wd, torch.stack(fockSet), dims=1)
        return Fd, float(np.sqrt(max(gram[n - 1, n - 1], 0.0)))

    # ---------------------------------------------------------------- reference helpers
    def orthoFock(self):
        """FO = X^T F X (mmd/scf.py:102-104)."""
        self.FO = np.dot(self.X.T, np.dot(self.F, self.X))

    def unOrthoFock(self):
        """F = U^T FO U (mmd/scf.py:106-108)."""
        self.F = np.dot(self.U.T, np.dot(self.FO, self.U))

    def orthoDen(self):
        """PO = U P U^T (mmd/scf.py:110-112)."""
        self.PO = np.dot(self.U, np.dot(self.P, self.U.T))

    def unOrthoDen(self):
        """P = X PO X^T (mmd/scf.py:114-116)."""
        self.P = np.dot(self.X, np.dot(self.PO, self.X.T))

    def computeEnergy(self):
        """E = tr((H + F) P) + E_nuc (mmd/scf.py:118-121)."""
        self.el_energy = np.einsum("pq,qp", self.Core + self.F, self.P)
        self.energy = self.el_energy + self.nuc_energy

    def computeDipole(self):
        """Dipole in Debye from P and the dipole integrals about the centre of charge
        (mmd/scf.py:123-129)."""
        self.el_energy = np.einsum("pq,qp", self.Core + self.F, self.P)
        for i in range(3):
            self.mu[i] = -2 * np.trace(np.dot(self.P, self.M[i])) + sum(
                [atom.charge * (atom.origin[i] - self.center_of_charge[i]) for atom in self.atoms])
        self.mu *= 2.541765

    def adj(self, x):
        """Conjugate transpose of a square matrix (mmd/scf.py:131-134)."""
        assert x.shape[0] == x.shape[1]
        return np.conjugate(x).T

    def comm(self, A, B):
        """[A, B] = AB - BA (mmd/scf.py:136-138)."""
        return np.dot(A, B) - np.dot(B, A)

    def buildFock(self):
        """Host-array Fock build from self.P / self.P_old (mmd/scf.py:82-100)."""
        from .integrals.fock import formPT
        if self.direct:
            G = formPT(self.P, self.P_old, self.bfs, self.nbasis, self.screen, self.scrTol)
            G = 0.5 * (G + G.T)
            self.G = G
            self.F = self.F_old + G
        else:
            # J and K are linear in P: a complex density (real-time TDHF) is two real
            # builds; the results are complex like the reference's einsums
            ctx = self.context
            torch = ctx.torch
            P = np.asarray(self.P)
            J = np.zeros(P.shape, dtype=complex)
            K = np.zeros(P.shape, dtype=complex)
            for scale, part in ((1.0, np.real(P)), (1j, np.imag(P))):
                if scale != 1.0 and not np.any(part):
                    continue
                Pd = torch.as_tensor(np.ascontiguousarray(part, dtype=np.float64), device=self._dev["S"].device)
                Jd, Kd = torch.empty_like(Pd), torch.empty_like(Pd)
                ctx.jk_dense(self._dev["TwoE"], Pd, Jd, Kd)
                J += scale * Jd.cpu().numpy()
                K += scale * Kd.cpu().numpy()
            self.J, self.K = J, K
            self.G = 2.0 * self.J - self.K
            self.F = self.Core.astype(complex) + self.G

    def updateFock(self):
        """unOrthoDen, buildFock, orthoFock (mmd/scf.py:140-144)."""
        self.unOrthoDen()
        self.buildFock()
        self.orthoFock()

    def updateDIIS(self, F, P):
        """One DIIS step on host arrays, as the reference's helper (mmd/scf.py:146-180):
        the error X (FPS - SPF) X of (F, P) and the *current* ``self.F`` join the
        8-deep histories ``self.errorSet`` / ``self.fockSet`` (created empty when
        absent), and the returned complex N x N matrix is the history combination
        whose weights minimise the combined error under sum(w) = 1.  The SCF loop
        itself runs the device version of the same step."""
        if getattr(self, "fockSet", None) is None:
            self.fockSet = []
        if getattr(self, "errorSet", None) is None:
            self.errorSet = []
        FPS = np.asarray(F) @ np.asarray(P) @ np.asarray(self.S)
        X = np.asarray(self.X)
        self.fockSet.append(self.F)
        self.errorSet.append(X @ (FPS - self.adj(FPS)) @ X)
        while len(self.fockSet) > 8:
            self.fockSet.pop(0)
            self.errorSet.pop(0)
        n = len(self.fockSet)
        E = np.stack(self.errorSet)
        B = np.full((n + 1, n + 1), -1.0)
        B[:n, :n] = np.einsum("iab,jab->ij", E.conj(), E).real  # Re tr(e_i^H e_j)
        B[n, n] = 0.0
        rhs = np.zeros(n + 1)
        rhs[n] = -1.0
        w = np.linalg.solve(B, rhs)
        assert np.isclose(w[:n].sum(), 1.0)
        return np.tensordot(w[:n], np.stack(self.fockSet), axes=1).astype(complex).reshape(
            self.nbasis, self.nbasis)


class _RHFState:
    """One RHF run on the device; ``iterate()`` is one pass of mmd/scf.py:30-60."""

    def __init__(self, mol, DIIS, guess, guess_fallback, subspace=None):
        self.mol = mol
        self.sub = subspace
        ctx = mol.context
        self.ctx = ctx
        torch = ctx.torch
        self.torch = torch
        dd = mol._dev
        self.Core, self.X, self.S = dd["Core"], dd["X"], dd["S"]
        if not mol.direct:
            mol._TwoE_dev = dd["TwoE"]
        self.DIIS = DIIS
        self.guess_fallback = guess_fallback
        mol.fock_builds = 0
        mol.fock_time = 0.0
        mol.guess_used = guess is not None
        mol.guess_reverted = False
        N = mol.nbasis
        self.P_old = torch.zeros((N, N), dtype=torch.float64, device=self.S.device)
        self.P = self.P_old
        self.F = self.Core.clone()
        if guess is not None:
            Pg = torch.as_tensor(np.asarray(guess, dtype=np.float64), device=self.S.device)
            self.F = self.Core + mol._two_electron(Pg, torch.zeros_like(Pg))
            self.P_old = Pg
            self.P = Pg
        self.fockSet, self.errorSet, self.err_hist = [], [], []
        self.energy = None
        self.FO = None
        self.F_old = None
        self.step = 0
        self.last_dP = None

    def iterate(self):
        """One SCF pass (mmd/scf.py:30-60): Fock build, DIIS, orthogonalised Fock,
        eigensolve, new density, energy and ||P - P_old||."""
        mol, torch = self.mol, self.torch
        X, S, Core = self.X, self.S, self.Core
        if self.step > 0:
            F_old = self.F
            self.F_old = F_old
            energy_old = self.energy
            if mol.direct:
                self.last_dP = (self.P, self.P_old)
                G = mol._two_electron(self.P, self.P_old, symmetrize=False)
                F = torch.empty_like(F_old)
                mol.context.fock_update(G, F_old, F)  # F = F_old + (G + G^T) / 2
                self.F = F
            else:
                self.F = mol._conventional_fock(self.P)
            self.P_old = self.P
            if self.DIIS:
                F_diis, derr = mol._diis(self.F, self.P, S, X, self.fockSet, self.errorSet)
                self.FO = X.T @ F_diis @ X
                eh = self.err_hist
                eh.append(derr)
                if mol.guess_used and self.guess_fallback and not mol.guess_reverted and diis_error_growing(eh):
                    # the initial guess misbehaves: restart from the core guess
                    mol.guess_reverted = True
                    self.P_old = torch.zeros_like(self.P)
                    self.F = Core.clone()
                    self.fockSet.clear()
                    self.errorSet.clear()
                    self.FO = X.T @ self.F @ X
                    if self.sub is not None:
                        self.sub.V = None  # dense solve, then a fresh warm start
        if not self.DIIS or self.step == 0:
            self.FO = X.T @ self.F @ X
        occ = self.sub.solve(self.FO) if self.sub is not None and self.step > 0 else None
        if occ is not None:  # occupied orbitals only (subspace iteration)
            self.E, self.CO, self.C = None, None, None
            Cocc = X @ occ[1]
        else:
            self._dense_solve()
            Cocc = self.C[:, : mol.nocc]
        self.P = Cocc @ Cocc.T
        self.energy = float(torch.sum((Core + self.F) * self.P.T).item()) + mol.nuc_energy
        if self.step > 0:
            mol.delta_energy = self.energy - energy_old
            mol.P_RMS = float(torch.linalg.norm(self.P - self.P_old).item())
        mol.energy = np.float64(self.energy)
        self.step += 1

    def _dense_solve(self):
        """All eigenpairs of FO (host LAPACK up to HOST_EIGH_MAX_N, cuSOLVER above);
        restarts the subspace iteration's warm start when one is in use."""
        torch = self.torch
        if self.FO.shape[0] <= HOST_EIGH_MAX_N:
            # up to ~1000 functions LAPACK on the host cores beats cuSOLVER's syevd
            w, v = host_eigh(self.FO.cpu().numpy())
            E = torch.from_numpy(w).to(self.FO.device)
            CO = torch.from_numpy(v).to(self.FO.device)
            if self.sub is not None:
                self.sub.start(self.FO, w, v)
        else:
            E, CO = torch.linalg.eigh(self.FO)
            if self.sub is not None:
                self.sub.start(self.FO, E.cpu().numpy(), CO.cpu().numpy())
        self.E, self.CO = E, CO
        self.C = self.X @ CO

    def finish(self):
        """Results back to the reference's attribute names (host arrays), with the
        reference's types: P, P_old, F, FO, C and CO complex128 (mmd/scf.py:15,24 start
        them complex; the imaginary parts are zero for RHF), the orbital energies MO
        real.  The energy stays a real float64 (the reference's carries a zero
        imaginary part).  Like the reference's loop, the molecule also keeps F_old
        (the Fock matrix before the last build) and, after a conventional run, the
        last build's J and K (complex128)."""
        mol = self.mol
        if self.E is None:  # the last iteration solved for the occupied orbitals only
            self._dense_solve()
        cplx = lambda t: t.cpu().numpy().astype(np.complex128)
        mol.P = cplx(self.P)
        mol.P_old = cplx(self.P_old)
        mol.F = cplx(self.F)
        mol.FO = cplx(self.FO)
        mol.C = cplx(self.C)
        mol.CO = cplx(self.CO)
        mol.MO = self.E.cpu().numpy()
        mol.energy = np.float64(self.energy)
        mol.el_energy = mol.energy - mol.nuc_energy
        if self.F_old is not None:
            mol.F_old = cplx(self.F_old)
        jk = getattr(mol, "_last_jk", None)
        if not mol.direct and jk is not None:
            mol.J, mol.K = cplx(jk[0]), cplx(jk[1])
