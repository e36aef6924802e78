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
complex128 tensors: the exponentials (``torch.linalg.matrix_exp``), the similarity
transforms, and the Fock rebuild ``F = H + 2J - K`` from the device ERI tensor with
the ``mmdg_jk_dense`` kernel (real and imaginary parts of the density in two
launches; J and K are linear in P).  Like the reference (whose ``reset`` runs
``RHF(doPrint=False)``), the rebuild is the conventional one.
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
        self._run(2, direction)

    def Magnus4(self, direction="x"):
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
        M3 = mol._dev["M"]
        TwoE = mol._dev["TwoE"]
        N = mol.nbasis
        nuc_mu = np.array([sum(a.charge * (a.origin[i] - mol.center_of_charge[i]) for a in mol.atoms)
                           for i in range(3)])
        Jr, Kr = torch.empty((N, N), dtype=torch.float64, device=dev), torch.empty((N, N), dtype=torch.float64,
                                                                                  device=dev)

        def jk(P):
            out = []
            for part in (P.real.contiguous(), P.imag.contiguous()):
                ctx.jk_dense(TwoE, part, Jr, Kr)
                out.append((Jr.clone(), Kr.clone()))
            (jr, kr), (ji, ki) = out
            return torch.complex(jr, ji), torch.complex(kr, ki)

        def rebuild(PO):
            """unOrthoDen + buildFock + orthoFock (mmd/scf.py:82-117)."""
            P = X @ PO @ X.T
            J, K = jk(P)
            F = Core + 2.0 * J - K
            return P, F

        def ortho(F):
            return X.T @ F @ X

        def field_at(t):
            return self.field * self.pulse(t)

        def move(A, PO0):
            Um = torch.linalg.matrix_exp(A)
            return Um @ PO0 @ Um.conj().T

        def comm(A, B):
            return A @ B - B @ A

        P = torch.as_tensor(np.asarray(mol.P, dtype=complex), device=dev)
        F = torch.as_tensor(np.asarray(mol.F, dtype=complex), device=dev)
        PO = Us @ P @ Us.T
        h = -1j * self.stepsize
        dt = self.stepsize
        for t in self.time:
            # dipole of the current density (computeDipole, mmd/scf.py:146-152)
            mu = (-2.0 * torch.einsum("pq,qp->", P.real, M3[ax])).item() + nuc_mu[ax]
            self.dipole.append(float(np.real(mu * 2.541765)))
            self.shape.append(self.pulse(t))
            PO0 = PO
            if order == 2:
                k1 = h * ortho(F + field_at(t) * Mdir)
                PO = move(k1, PO0)
                P, F = rebuild(PO)
                L = 0.5 * (k1 + h * ortho(F + field_at(t + dt) * Mdir))
                PO = move(L, PO0)
                P, F = rebuild(PO)
            else:
                k1 = h * ortho(F + field_at(t) * Mdir)
                Q1 = k1
                PO = move(0.5 * Q1, PO0)
                P, F = rebuild(PO)
                k2 = h * ortho(F + field_at(t + 0.5 * dt) * Mdir)
                Q2 = k2 - k1
                PO = move(0.5 * Q1 + 0.25 * Q2, PO0)
                P, F = rebuild(PO)
                k3 = h * ortho(F + field_at(t + 0.5 * dt) * Mdir)
                Q3 = k3 - k2
                PO = move(Q1 + Q2, PO0)
                P, F = rebuild(PO)
                k4 = h * ortho(F + field_at(t + dt) * Mdir)
                Q4 = k4 - 2.0 * k2 + k1
                C12 = comm(Q1, Q2)
                PO = move(0.5 * Q1 + 0.25 * Q2 + (1.0 / 3.0) * Q3 - (1.0 / 24.0) * Q4 - (1.0 / 48.0) * C12, PO0)
                P, F = rebuild(PO)
                k5 = h * ortho(F + field_at(t + 0.5 * dt) * Mdir)
                Q5 = k5 - k2
                PO = move(Q1 + Q2 + (2.0 / 3.0) * Q3 + (1.0 / 6.0) * Q4 - (1.0 / 6.0) * C12, PO0)
                P, F = rebuild(PO)
                k6 = h * ortho(F + field_at(t + dt) * Mdir)
                Q6 = k6 - 2.0 * k2 + k1
                L = Q1 + Q2 + (2.0 / 3.0) * Q5 + (1.0 / 6.0) * Q6 - (1.0 / 6.0) * comm(Q1, Q2 - Q3 + Q5 + 0.5 * Q6)
                PO = move(L, PO0)
                P, F = rebuild(PO)
            # energy of the step's final density (computeEnergy, mmd/scf.py:141-144)
            E = torch.einsum("pq,qp->", Core + F, P).item() + mol.nuc_energy
            self.Energy.append(float(np.real(E)))
        mol.PO = PO.cpu().numpy()
        mol.P = P.cpu().numpy()
        mol.F = F.cpu().numpy()
        mol.FO = ortho(F).cpu().numpy()
        mol.energy = np.complex128(E)


def _axis(direction):
    d = direction.lower()
    if d not in ("x", "y", "z"):
        raise ValueError("direction must be 'x', 'y' or 'z'")
    return "xyz".index(d)
