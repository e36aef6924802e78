"""Batched RHF: many closed-shell molecules in lockstep, one Fock launch for all.

Every molecule runs the reference's RHF (mmd/scf.py:10-80: core guess, direct
incremental Fock builds at acc2e, 8-deep DIIS, eigensolve, convergence on
||P - P_old||_F); what is batched is the two-electron work.  All molecules share
one device context (``nmol`` > 1): the screening and the class kernels of a Fock
build cover every molecule in one launch per class, replayed as one CUDA graph
(``mmdg_fock_graph``).  A molecule that has converged keeps P fixed, so its density
difference is zero and the screening removes all its quartets.

The small dense algebra is batched too: padded (B, Nmax, Nmax) tensors on the GPU
for the products and DIIS, and the eigensolves on the host cores in a thread pool
(LAPACK releases the GIL; cuSOLVER's batched path is slow for these sizes).
"""
from __future__ import annotations

import ctypes
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import _native
from .integrals.shells import shells_from_bfs
from .molecule import Molecule
from .scf import diis_error_growing


def _openblas_controls():
    """(get, set) thread-count functions of the OpenBLAS that numpy loaded, or None."""
    try:
        with open("/proc/self/maps") as f:
            paths = sorted({ln.split()[-1] for ln in f if "openblas" in ln.lower() and ln.split()[-1].startswith("/")})
    except OSError:
        return None
    for path in paths:
        try:
            lib = ctypes.CDLL(path)
        except OSError:
            continue
        for pre, suf in (("scipy_openblas", "64_"), ("scipy_openblas", ""), ("openblas", "64_"), ("openblas", "")):
            g, s = f"{pre}_get_num_threads{suf}", f"{pre}_set_num_threads{suf}"
            if hasattr(lib, g) and hasattr(lib, s):
                get, set_ = getattr(lib, g), getattr(lib, s)
                get.restype = ctypes.c_int
                set_.argtypes = [ctypes.c_int]
                return get, set_
    return None


class _single_threaded_blas:
    """Context manager: numpy's OpenBLAS on one thread (no-op if it cannot be found)."""

    def __enter__(self):
        self.ctl = _openblas_controls()
        if self.ctl:
            self.prev = self.ctl[0]()
            self.ctl[1](1)
        return self

    def __exit__(self, *exc):
        if self.ctl:
            self.ctl[1](self.prev)
        return False


class BatchRHF:
    """RHF of many molecules in lockstep through one device context: one Fock build
    (a CUDA graph of every class's screening and evaluation launch) serves the whole
    batch per iteration; the dense algebra runs on padded (B, Nmax, Nmax) tensors, the
    eigensolves on the host cores; molecules that converge drop out of the
    eigensolves.  ``run`` returns the energies (mmd/scf.py:10-80 per molecule)."""

    def __init__(self, geometries, basis="6-31g", acc2e=1e-12, fp32_below=0.0, graph=True, tuning=None):
        torch = _native._torch()
        self.torch = torch
        self.mols = [Molecule(g, basis) for g in geometries]
        self.B = len(self.mols)
        self.N = np.array([m.nbasis for m in self.mols])
        self.nocc = np.array([m.nocc for m in self.mols])
        self.Nmax = int(self.N.max())
        self.acc2e = acc2e
        self.fp32_below = fp32_below
        self.graph = graph
        self.ctx = _native.Context([shells_from_bfs(m.bfs) for m in self.mols])
        if tuning is not None:
            tuning.apply(self.ctx)
        dev = f"cuda:{self.ctx.device}"
        self.dev = dev
        # packed <-> padded index maps
        base = self.ctx.base
        pk, pd = [], []
        for b, n in enumerate(self.N):
            i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
            pk.append(base[b] + (i * n + j).ravel())
            pd.append(b * self.Nmax * self.Nmax + (i * self.Nmax + j).ravel())
        self.pk = torch.as_tensor(np.concatenate(pk), device=dev)
        self.pd = torch.as_tensor(np.concatenate(pd), device=dev)
        self._one_electron()

    # ------------------------------------------------------------ set-up
    def _pad(self, packed):
        torch = self.torch
        out = torch.zeros(self.B * self.Nmax * self.Nmax, dtype=torch.float64, device=self.dev)
        out[self.pd] = packed[self.pk]
        return out.view(self.B, self.Nmax, self.Nmax)

    def _pack(self, padded):
        torch = self.torch
        out = torch.empty(self.ctx.nn, dtype=torch.float64, device=self.dev)
        out[self.pk] = padded.reshape(-1)[self.pd]
        return out

    def _one_electron(self):
        torch = self.torch
        nn = self.ctx.nn
        S = torch.empty(nn, dtype=torch.float64, device=self.dev)
        T, V = torch.empty_like(S), torch.empty_like(S)
        M = torch.empty(3 * nn, dtype=torch.float64, device=self.dev)
        atom_mol, xyz, Z, org = [], [], [], []
        for b, m in enumerate(self.mols):
            for a in m.atoms:
                atom_mol.append(b)
                xyz.extend(a.origin)
                Z.append(float(a.charge))
            org.extend(m.center_of_charge)
        atom_mol = np.array(atom_mol, dtype=np.int32)
        xyz, Z, org = (np.ascontiguousarray(x, dtype=np.float64) for x in (xyz, Z, org))
        p = _native._ptr
        _native.check(_native.lib().mmdg_one_electron(self.ctx._h, len(atom_mol), p(atom_mol), p(xyz), p(Z), p(org),
                                                       ctypes.c_void_p(S.data_ptr()), ctypes.c_void_p(T.data_ptr()),
                                                       ctypes.c_void_p(V.data_ptr()), ctypes.c_void_p(M.data_ptr()),
                                                       _native.stream_ptr()), "mmdg_one_electron")
        self.S = self._pad(S)
        self.Core = self._pad(T + V)
        self.nuc = np.zeros(self.B)
        for b, m in enumerate(self.mols):
            at = m.atoms
            for i in range(len(at)):
                for j in range(i):
                    self.nuc[b] += at[i].charge * at[j].charge / np.linalg.norm(at[i].origin - at[j].origin)
        # X = S^-1/2 per molecule (padding: zero rows/columns)
        Sh = self.S.cpu().numpy()
        X = np.zeros_like(Sh)
        for b, n in enumerate(self.N):
            w, U = np.linalg.eigh(Sh[b, :n, :n])
            X[b, :n, :n] = (U * (1.0 / np.sqrt(w))) @ U.T
        self.X = torch.as_tensor(X, device=self.dev)
        # large level shift on the padded diagonal of X^T F X keeps padding unoccupied
        pad = np.ones((self.B, self.Nmax))
        for b, n in enumerate(self.N):
            pad[b, :n] = 0.0
        self.pad_shift = torch.as_tensor(pad * 1e6, device=self.dev)

    # ------------------------------------------------------------ iteration pieces
    def fock(self, dP_padded):
        """Unsymmetrised G of every molecule for a padded density difference (packed result)."""
        torch = self.torch
        dP = self._pack(dP_padded)
        if not hasattr(self, "_dP_buf"):
            self._dP_buf = torch.empty_like(dP)
            self._G_buf = torch.empty_like(dP)
        self._dP_buf.copy_(dP)
        if self.graph:
            _native.check(_native.lib().mmdg_fock_graph(self.ctx._h, ctypes.c_void_p(self._dP_buf.data_ptr()),
                                                         ctypes.c_void_p(self._G_buf.data_ptr()),
                                                         float(self.acc2e), float(self.fp32_below),
                                                         _native.stream_ptr()), "mmdg_fock_graph")
        else:
            self.ctx.fock(self._dP_buf, self._G_buf, tol=self.acc2e, fp32_below=self.fp32_below)
        return self._G_buf

    def _eigh(self, FO, active=None):
        """Eigenpairs of every (active) molecule's block, on the host cores: one LAPACK
        call per molecule in a thread pool, with numpy's OpenBLAS held to one thread
        meanwhile (16 solves in parallel beat 16 threads inside each small solve:
        0.13 s against 0.45 s for 1024 matrices of 13..104 on 16 Grace cores).
        Converged (inactive) molecules are skipped; their slots return zeros."""
        FOh = FO.cpu().numpy()
        E = np.zeros((self.B, self.Nmax))
        C = np.zeros_like(FOh)

        def one(b):
            n = self.N[b]
            w, v = np.linalg.eigh(FOh[b, :n, :n])
            E[b, :n] = w
            C[b, :n, :n] = v

        todo = range(self.B) if active is None else np.flatnonzero(active)
        with _single_threaded_blas(), ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
            list(ex.map(one, todo))
        return self.torch.as_tensor(E, device=self.dev), self.torch.as_tensor(C, device=self.dev)

    def _density(self, CO):
        C = self.X @ CO
        mask = (self.torch.arange(self.Nmax, device=self.dev)[None, :] <
                self.torch.as_tensor(self.nocc, device=self.dev)[:, None]).to(C.dtype)
        Cocc = C * mask[:, None, :]
        return Cocc @ Cocc.transpose(1, 2)

    def run(self, conver=1e-8, maxiter=100, DIIS=True, guess=None, guess_fallback=True, polish=False,
            polish_fp32_below=0.0):
        """RHF of every molecule; returns the energies (numpy, Eh).

        ``polish``: after convergence, one non-incremental Fock build of the converged
        densities (FP64, or FP32 below ``polish_fp32_below``) and the energy
        E(P) = tr((H + F(P)) P) + E_nuc from it
        (returned; the SCF's own last energies stay in ``energies_raw``).  This
        removes what the incremental builds accumulate (screening drops, FP32
        quartets) from the energy and leaves only the density's own convergence
        error, which enters the energy to second order.

        ``guess``: optional list of initial densities (N_m x N_m); the first Fock
        matrix is then Core + sym(G(P_guess)), and a molecule whose DIIS error grows
        three iterations in a row restarts from the core guess (its stale DIIS
        entries get zero weight)."""
        torch = self.torch
        B, Nm = self.B, self.Nmax
        X, S, Core = self.X, self.S, self.Core
        P_old = torch.zeros((B, Nm, Nm), dtype=torch.float64, device=self.dev)
        P = P_old.clone()
        F = Core.clone()
        self.reverted = np.zeros(B, dtype=bool)
        if guess is not None:
            Pg = np.zeros((B, Nm, Nm))
            for b, g in enumerate(guess):
                n = self.N[b]
                Pg[b, :n, :n] = g
            P = torch.as_tensor(Pg, device=self.dev)
            P_old = P.clone()
            G = self._pad(self.fock(P))
            F = Core + 0.5 * (G + G.transpose(1, 2))
        valid_from = np.zeros(B, dtype=int)  # first usable DIIS slot (by global step) per molecule
        revert = None
        err_hist = []
        hist_steps = []
        hist_F, hist_E = [], []
        done = np.zeros(B, dtype=bool)
        energy = np.zeros(B)
        E_old = np.zeros(B)
        self.iterations = np.zeros(B, dtype=int)
        self.fock_builds = 0
        for step in range(maxiter):
            active = torch.as_tensor(~done, device=self.dev)[:, None, None]
            if step > 0:
                F_old = F
                G = self.fock(P - P_old)
                self.fock_builds += 1
                Gp = self._pad(G)
                F = torch.where(active, F_old + 0.5 * (Gp + Gp.transpose(1, 2)), F_old)
                P_old = P
                if DIIS:
                    FPS = F @ P @ S
                    err = X @ (FPS - FPS.transpose(1, 2)) @ X
                    hist_F.append(F)
                    hist_E.append(err)
                    hist_steps.append(step)
                    if len(hist_F) > 8:
                        hist_F.pop(0)
                        hist_E.pop(0)
                        hist_steps.pop(0)
                    n = len(hist_F)
                    Ev = torch.stack(hist_E, 1).reshape(B, n, -1)
                    Bm = torch.full((B, n + 1, n + 1), -1.0, dtype=torch.float64, device=self.dev)
                    Bm[:, :n, :n] = Ev @ Ev.transpose(1, 2)
                    Bm[:, n, n] = 0.0
                    # slots from before a molecule's restart: decoupled, huge diagonal -> zero weight
                    stale = torch.as_tensor(np.array(hist_steps)[None, :] < valid_from[:, None], device=self.dev)
                    if bool(stale.any()):
                        sf = stale.to(Bm.dtype)
                        keep = 1.0 - sf
                        Bm[:, :n, :n] = Bm[:, :n, :n] * keep[:, :, None] * keep[:, None, :]
                        Bm[:, :n, :n] += torch.diag_embed(sf * 1e30)
                    if guess is not None and guess_fallback:
                        en = torch.linalg.norm(err.reshape(B, -1), dim=1).cpu().numpy()
                        err_hist.append(en)
                        grow = diis_error_growing(err_hist) & ~self.reverted & ~done
                        if grow.any():
                            idx = np.flatnonzero(grow)
                            self.reverted[idx] = True
                            valid_from[idx] = step + 1
                            rm = torch.zeros(B, dtype=torch.bool, device=self.dev)
                            rm[torch.as_tensor(idx, device=self.dev)] = True
                            revert = rm[:, None, None]
                    rhs = torch.zeros((B, n + 1), dtype=torch.float64, device=self.dev)
                    rhs[:, n] = -1.0
                    # converged (frozen) molecules: a well-posed dummy system
                    eye = torch.eye(n + 1, dtype=torch.float64, device=self.dev).expand(B, -1, -1)
                    Bm = torch.where(active, Bm, eye)
                    # the B small (n+1)^2 systems are solved on the host (LAPACK), like the
                    # eigensolves: no dependence on torch's CUDA linear-algebra library
                    w = torch.as_tensor(np.linalg.solve(Bm.cpu().numpy(), rhs.cpu().numpy()[..., None])[..., 0],
                                        device=self.dev)
                    Fd = torch.einsum("bi,bijk->bjk", w[:, :n], torch.stack(hist_F, 1))
                    FO = X.transpose(1, 2) @ Fd @ X
                    if revert is not None:  # restart from the core guess: F = Core, P_old = 0
                        F = torch.where(revert, Core, F)
                        P_old = torch.where(revert, torch.zeros_like(P_old), P_old)
                        FO = torch.where(revert, X.transpose(1, 2) @ Core @ X, FO)
                        revert = None
                else:
                    FO = X.transpose(1, 2) @ F @ X
            else:
                FO = X.transpose(1, 2) @ F @ X
            FO = FO + torch.diag_embed(self.pad_shift)
            _, CO = self._eigh(FO, ~done)
            Pn = self._density(CO)
            P = torch.where(active, Pn, P)
            e = (torch.sum((Core + F) * P.transpose(1, 2), dim=(1, 2))).cpu().numpy() + self.nuc
            if step > 0:
                rms = torch.linalg.norm((P - P_old).reshape(B, -1), dim=1).cpu().numpy()
                newly = (~done) & (rms < conver)
                energy = np.where(~done, e, energy)
                self.iterations[newly] = step
                done |= newly
            else:
                energy = e
            E_old = energy
            if done.all():
                break
        self.energies_raw = energy
        self.converged = done
        self.P = P
        if polish:
            dP = self._pack(P)
            G = torch.empty_like(dP)
            self.ctx.fock(dP, G, tol=self.acc2e, fp32_below=float(polish_fp32_below))
            Gp = self._pad(G)
            Fp = Core + 0.5 * (Gp + Gp.transpose(1, 2))
            energy = (torch.sum((Core + Fp) * P.transpose(1, 2), dim=(1, 2))).cpu().numpy() + self.nuc
            self.fock_builds += 1
        self.energies = energy
        return energy


def per_molecule_fock_rate(geometries, basis, densities, acc2e=1e-12):
    """Fock builds/s launching every molecule separately (one context each)."""
    import time
    torch = _native._torch()
    ctxs, dPs = [], []
    for g, P in zip(geometries, densities):
        m = Molecule(g, basis)
        ctx = _native.Context(shells_from_bfs(m.bfs))
        ctxs.append(ctx)
        dPs.append(torch.as_tensor(np.ascontiguousarray(P), device="cuda").reshape(-1))
    for c, d in zip(ctxs, dPs):
        c.fock(d, tol=acc2e)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for c, d in zip(ctxs, dPs):
        c.fock(d, tol=acc2e)
    torch.cuda.synchronize()
    return len(ctxs) / (time.perf_counter() - t0)
