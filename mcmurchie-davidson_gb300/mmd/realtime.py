"""Real-time TDHF with Magnus propagators, behind the reference's ``mmd.realtime`` API.

``RealTime(mol, numsteps, stepsize, field, pulse)`` with ``Magnus2``, ``Magnus4``,
``addField`` and ``reset`` keeps the attributes and results of mmd/realtime.py:6-197
(``time``, ``dipole``, ``Energy``, ``shape``; the molecule's ``P``, ``PO``, ``F``,
``FO`` and ``energy`` after the run).  The propagators are the explicit Magnus
integrators of Blanes and Casas, *A concise introduction to geometric numerical
integration* (CRC Press 2016), Eq. (4.61) (second order) and Eq. (4.62) (fourth
order), evaluated exactly as the reference sequences them (mmd/realtime.py:32-153):
each stage adds the dipole field at its time to the Fock matrix, exponentiates, moves
the density of the step start and rebuilds the Fock matrix from it.

Everything between the ground-state SCF and the end of the run stays on the GPU as
complex128 tensors: the exponentials (scaled Taylor series, squared back), the
similarity transforms, and the Fock rebuild ``F = H + 2J - K`` from the device ERI
tensor with the ``mmdg_jk_dense`` kernel (real and imaginary parts of the density in
two launches; J and K are linear in P).  One propagation step -- field values read
from a precomputed table by a device step counter, dipole and energy written into
device records -- is captured once as a CUDA graph and replayed for every step, so a
step costs one graph launch instead of some 300 kernel launches from Python.  Like
the reference (whose ``reset`` runs ``RHF(doPrint=False)``), the rebuild is the
conventional one.
"""
from __future__ import annotations

import numpy as np


class RealTime:
    """Class for real-time routines (mmd/realtime.py:6-19)."""

    def __init__(self, mol, numsteps=1000, stepsize=0.1, field=0.0001, pulse=None):
        self.mol = mol
        self.field = field
        self.stepsize = stepsize
        self.numSteps = numsteps
        self.time = np.arange(0, self.numSteps) * self.stepsize
        self.pulse = pulse if pulse else (lambda t: 0.0)
        self.reset()

    def reset(self):
        """Ground state again and empty property records (mmd/realtime.py:21-31)."""
        self.mol.RHF(doPrint=False)
        self.dipole = []
        self.angmom = []
        self.Energy = []
        self.shape = []

    def addField(self, time, direction="x"):
        """Dipole field of the pulse envelope at ``time`` added to the host Fock matrix,
        then orthogonalised (mmd/realtime.py:155-197); the propagators do the same on
        the device."""
        self.mol.F = self.mol.F + self.field * self.pulse(time) * self.mol.M[_axis(direction)]
        self.mol.orthoFock()

    def Magnus2(self, direction="x"):
        """Second-order Magnus propagation along ``direction`` (mmd/realtime.py:32-74)."""
        self._run(2, direction)

    def Magnus4(self, direction="x"):
        """Fourth-order Magnus propagation along ``direction`` (mmd/realtime.py:76-153)."""
        self._run(4, direction)

    # ------------------------------------------------------------------ device run
    def _run(self, order, direction):
        self.reset()
        mol = self.mol
        ax = _axis(direction)
        ctx = mol.context
        torch = ctx.torch
        dev = mol._dev["S"].device
        c128 = torch.complex128
        X = mol._dev["X"].to(c128)
        Us = torch.as_tensor(mol.U, device=dev).to(c128)
        Core = mol._dev["Core"].to(c128)
        Mdir = mol._dev["M"][ax].to(c128)
        Mreal = mol._dev["M"][ax]
        TwoE = mol._dev["TwoE"]
        N = mol.nbasis
        eye = torch.eye(N, dtype=c128, device=dev)
        nuc_mu = float(sum(a.charge * (a.origin[ax] - mol.center_of_charge[ax]) for a in mol.atoms))
        dt, h = self.stepsize, -1j * self.stepsize
        # field x envelope at every stage time of every step, known in advance
        frac = (0.0, 1.0) if order == 2 else (0.0, 0.5, 0.5, 1.0, 0.5, 1.0)
        fall = torch.as_tensor([[self.field * self.pulse(t + f * dt) for f in frac] for t in self.time],
                               dtype=torch.float64, device=dev)
        self.shape = [self.pulse(t) for t in self.time]
        # static state and records
        P = torch.as_tensor(np.asarray(mol.P, dtype=complex), device=dev)
        F = torch.as_tensor(np.asarray(mol.F, dtype=complex), device=dev)
        PO = Us @ P @ Us.T
        kidx = torch.zeros(1, dtype=torch.int64, device=dev)
        dips = torch.zeros(len(self.time), dtype=torch.float64, device=dev)
        ens = torch.zeros(len(self.time), dtype=torch.float64, device=dev)
        Pr, Pi = torch.empty((N, N), dtype=torch.float64, device=dev), torch.empty((N, N), dtype=torch.float64,
                                                                                   device=dev)
        Jr, Kr = torch.empty_like(Pr), torch.empty_like(Pr)
        Ji, Ki = torch.empty_like(Pr), torch.empty_like(Pr)
        # scaling for the Taylor exponential: 2^-s |A|_1 <= 1/4 with a 4x margin over
        # the largest Magnus exponent expected (a few times |h F_O|)
        FO0 = X.T @ F @ X
        norm = float(torch.linalg.matrix_norm(h * FO0, ord=1).item()) * 4.0
        sq = max(0, int(np.ceil(np.log2(max(norm, 1e-300) / 0.25))))

        def expm(A):
            """exp(A): degree-12 Taylor series of A / 2^sq (Horner), squared sq times;
            truncation below (1/4)^13 / 13! = 2e-18 relative."""
            B = A * (0.5 ** sq)
            E = eye
            for k in range(12, 0, -1):
                E = eye + (B @ E) * (1.0 / k)
            for _ in range(sq):
                E = E @ E
            return E

        def rebuild(POn):
            """unOrthoDen + buildFock + orthoFock (mmd/scf.py:82-117) into the state."""
            Pn = X @ POn @ X.T
            Pr.copy_(Pn.real)
            Pi.copy_(Pn.imag)
            ctx.jk_dense(TwoE, Pr, Jr, Kr)
            ctx.jk_dense(TwoE, Pi, Ji, Ki)
            Fn = Core + 2.0 * torch.complex(Jr, Ji) - torch.complex(Kr, Ki)
            return Pn, Fn

        def ortho(Fm):
            return X.T @ Fm @ X

        def move(A, PO0):
            Um = expm(A)
            return Um @ PO0 @ Um.conj().T

        def comm(A, B):
            return A @ B - B @ A

        def step():
            fv = fall.index_select(0, kidx).reshape(-1)
            # dipole of the step's starting density (computeDipole, mmd/scf.py:146-152)
            dip = (-2.0 * torch.sum(P.real * Mreal.T) + nuc_mu) * 2.541765
            PO0 = PO.clone()
            if order == 2:
                k1 = h * ortho(F + fv[0] * Mdir)
                Pn, Fn = rebuild(move(k1, PO0))
                L = 0.5 * (k1 + h * ortho(Fn + fv[1] * Mdir))
                POn = move(L, PO0)
                Pn, Fn = rebuild(POn)
            else:
                k1 = h * ortho(F + fv[0] * Mdir)
                Q1 = k1
                Pn, Fn = rebuild(move(0.5 * Q1, PO0))
                k2 = h * ortho(Fn + fv[1] * Mdir)
                Q2 = k2 - k1
                Pn, Fn = rebuild(move(0.5 * Q1 + 0.25 * Q2, PO0))
                k3 = h * ortho(Fn + fv[2] * Mdir)
                Q3 = k3 - k2
                Pn, Fn = rebuild(move(Q1 + Q2, PO0))
                k4 = h * ortho(Fn + fv[3] * Mdir)
                Q4 = k4 - 2.0 * k2 + k1
                C12 = comm(Q1, Q2)
                Pn, Fn = rebuild(move(0.5 * Q1 + 0.25 * Q2 + (1.0 / 3.0) * Q3 - (1.0 / 24.0) * Q4
                                      - (1.0 / 48.0) * C12, PO0))
                k5 = h * ortho(Fn + fv[4] * Mdir)
                Q5 = k5 - k2
                Pn, Fn = rebuild(move(Q1 + Q2 + (2.0 / 3.0) * Q3 + (1.0 / 6.0) * Q4 - (1.0 / 6.0) * C12, PO0))
                k6 = h * ortho(Fn + fv[5] * Mdir)
                Q6 = k6 - 2.0 * k2 + k1
                L = Q1 + Q2 + (2.0 / 3.0) * Q5 + (1.0 / 6.0) * Q6 - (1.0 / 6.0) * comm(Q1, Q2 - Q3 + Q5 + 0.5 * Q6)
                POn = move(L, PO0)
                Pn, Fn = rebuild(POn)
            # energy of the step's final density (computeEnergy, mmd/scf.py:141-144)
            E = torch.sum((Core + Fn) * Pn.T).real + mol.nuc_energy
            dips.index_copy_(0, kidx, dip.reshape(1))
            ens.index_copy_(0, kidx, E.reshape(1))
            PO.copy_(POn)
            P.copy_(Pn)
            F.copy_(Fn)
            kidx.add_(1)

        # one propagation step captured as a CUDA graph and replayed for every step;
        # the warm-up run (allocator, library handles) works on a copy of the state
        saved = (P.clone(), F.clone(), PO.clone())
        side = torch.cuda.Stream(device=dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):
            step()
        torch.cuda.current_stream(dev).wait_stream(side)
        P.copy_(saved[0])
        F.copy_(saved[1])
        PO.copy_(saved[2])
        kidx.zero_()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            step()
        for _ in self.time:
            graph.replay()
        self.dipole = dips.cpu().tolist()
        self.Energy = ens.cpu().tolist()
        mol.PO = PO.cpu().numpy()
        mol.P = P.cpu().numpy()
        mol.F = F.cpu().numpy()
        mol.FO = ortho(F).cpu().numpy()
        mol.energy = np.complex128(self.Energy[-1]) if self.Energy else mol.energy


def _axis(direction):
    d = direction.lower()
    if d not in ("x", "y", "z"):
        raise ValueError("direction must be 'x', 'y' or 'z'")
    return "xyz".index(d)
