"""AO -> MO integral transform and MP2 on the GPU, behind the reference's
``mmd.postscf.PostSCF`` API (mmd/postscf.py:13-73).

``PostSCF(mol)`` requires a converged conventional RHF (the device ERI tensor) and
runs ``ao2mo``: the 4-index transform (pq|rs) -> (PQ|RS) as four FP64 quarter
transforms over one index each (the project's kernel, mmdg_ao2mo), the
spin-orbital antisymmetrised integrals <AB||CD> (spin orbital 2p + sigma, the
ordering of the reference's Kronecker products; built on first use), the spin-orbital
core Hamiltonian ``Hp`` and orbital energies ``fs`` -- the attributes the reference
sets, as host arrays.  ``MP2`` evaluates the reference's sums (spatial, and spin-orbital from
<ij||ab>) as vectorised device reductions instead of Python loops.

``CIS`` and ``TDHF`` (mmd/postscf.py:249-400) build the singles matrices A and B from
device blocks of <AB||CD> and diagonalise on the GPU: CIS energies and oscillator
strengths from one symmetric eigensolve; TDHF by the reference's three algorithms
('hermitian': sqrt(A-B)(A+B)sqrt(A-B), the square root from a symmetric
eigendecomposition; 'reduced': the non-symmetric (A-B)(A+B); 'full': the
non-symmetric [[A, B], [-B^T, -A^T]]).  The determinant-string paths (CIS with
``bitstring=True``, CISD, FCI) build Slater-determinant Hamiltonians from bit
strings, not integral contractions, and are not provided.
"""
from __future__ import annotations

import sys

import numpy as np

from . import _native


class PostSCF:
    """Post-SCF methods on a converged RHF molecule (mmd/postscf.py:13-19)."""

    def __init__(self, mol):
        self.mol = mol
        if not self.mol.is_converged:
            sys.exit("SCF not converged, skipping Post-SCF")
        if "TwoE" not in getattr(mol, "_dev", {}):
            raise ValueError("PostSCF needs the ERI tensor: run mol.RHF(direct=False) first")
        self.ao2mo()

    def ao2mo(self):
        """(pq|rs) -> (PQ|RS), spin blocking and antisymmetrisation (mmd/postscf.py:21-41)."""
        mol = self.mol
        torch = mol.context.torch
        dev = mol._dev["S"].device
        N = mol.nbasis
        C = torch.as_tensor(np.real(np.asarray(mol.C)), dtype=torch.float64, device=dev)
        # the four quarter transforms in libmmdg.so (mmdg_ao2mo): each contracts the
        # last index and writes the new one first, pqrs -> Spqr -> RSpq -> QRSp -> PQRS
        mo = _native.ao2mo(C, mol._dev["TwoE"].reshape(-1)).view(N, N, N, N)
        self._mo = mo
        mol.single_bar = mo.cpu().numpy()
        mol.norb = 2 * N
        # the (2N)^4 spin-orbital tensor is built when first used (MP2(spin_orbital=True)
        # or mol.double_bar), not here: it is 16x the spatial one
        self._double_bar = None
        mol._double_bar = None
        mol._double_bar_build = lambda: self._spin_tensor().cpu().numpy()
        Core = mol._dev["Core"]
        h = C.T @ Core @ C
        mol.Hp = np.kron(h.cpu().numpy(), np.eye(2))
        mol.fs = np.kron(np.diag(np.real(np.asarray(mol.MO))), np.eye(2))

    def _spin_block(self, A, B, C, D):
        """Block <AB||CD> of the spin-orbital integrals for index ranges A..D (spin
        orbital 2p + sigma, mmd/postscf.py:31-35): <AB|CD> = (ac|bd) d(sA,sC) d(sB,sD),
        antisymmetrised in C, D."""
        torch = self.mol.context.torch
        dev = self._mo.device
        idx = [torch.arange(r.start, r.stop, device=dev) for r in (A, B, C, D)]
        sp = [i // 2 for i in idx]
        sg = [i % 2 for i in idx]
        phys = self._mo.permute(0, 2, 1, 3)                             # <ab|cd> = (ac|bd)

        def coulomb(c, d):
            blk = phys[sp[0]][:, sp[1]][:, :, sp[c]][:, :, :, sp[d]]
            s_ac = (sg[0][:, None] == sg[c][None, :]).to(blk.dtype)
            s_bd = (sg[1][:, None] == sg[d][None, :]).to(blk.dtype)
            return blk * s_ac[:, None, :, None] * s_bd[None, :, None, :]

        return coulomb(2, 3) - coulomb(3, 2).permute(0, 1, 3, 2)

    def _spin_tensor(self):
        """The whole (2N)^4 spin-orbital tensor (device, cached)."""
        if self._double_bar is None:
            n = range(0, 2 * self._mo.shape[0])
            self._double_bar = self._spin_block(n, n, n, n)
        return self._double_bar

    def MP2(self, spin_orbital=False):
        """MP2 energy from the RHF reference (mmd/postscf.py:44-73)."""
        mol = self.mol
        torch = mol.context.torch
        dev = self._mo.device
        if spin_orbital:
            e = torch.as_tensor(np.diag(mol.fs).copy(), dtype=torch.float64, device=dev)
            o, v = slice(0, mol.nelec), slice(mol.nelec, mol.norb)
            d = e[o][:, None, None, None] + e[o][None, :, None, None] - e[v][None, None, :, None] - e[v][None, None, None, :]
            num = self._spin_block(range(o.start, o.stop), range(o.start, o.stop), range(v.start, v.stop),
                                   range(v.start, v.stop)) ** 2
            mol.emp2 = np.complex128(0.25 * float((num / d).sum().item()) + mol.energy)
        else:
            e = torch.as_tensor(np.real(np.asarray(mol.MO)), dtype=torch.float64, device=dev)
            no = mol.nocc
            iajb = self._mo[:no, no:, :no, no:]
            d = e[:no][:, None, None, None] - e[no:][None, :, None, None] + e[:no][None, None, :, None] - \
                e[no:][None, None, None, :]
            num = iajb * (2.0 * iajb - iajb.permute(0, 3, 2, 1))
            mol.emp2 = np.complex128(float((num / d).sum().item()) + mol.energy)
        print("E(MP2) = ", mol.emp2.real)

    def _singles(self, with_b=False):
        """The singles matrices of mmd/postscf.py:262-266 and 349-355 on the device:
        A[ia,jb] = (e_a - e_i) d_ij d_ab + <aj||ib>, B[ia,jb] = <ab||ij>."""
        mol = self.mol
        torch = mol.context.torch
        dev = self._mo.device
        no, nv = mol.nelec, mol.norb - mol.nelec
        occ, vir = range(0, no), range(no, mol.norb)
        e = torch.as_tensor(np.diag(mol.fs).copy(), dtype=torch.float64, device=dev)
        A = self._spin_block(vir, occ, occ, vir).permute(2, 0, 1, 3).reshape(no * nv, no * nv)
        A = A + torch.diag((e[no:][None, :] - e[:no][:, None]).reshape(-1))
        if not with_b:
            return A
        B = self._spin_block(vir, vir, occ, occ).permute(2, 0, 3, 1).reshape(no * nv, no * nv)
        return A, B

    def CIS(self, bitstring=False):
        """Configuration interaction singles from the RHF reference (mmd/postscf.py:249-322):
        excitation energies (eV) in ``mol.cis_omega``, oscillator strengths
        f = 2/3 w |<0|mu|n>|^2 in ``mol.cis_oscil``."""
        if bitstring:
            raise NotImplementedError("PostSCF.CIS(bitstring=True) builds a determinant Hamiltonian; "
                                      "not part of this implementation")
        mol = self.mol
        torch = mol.context.torch
        no, nv = mol.nelec, mol.norb - mol.nelec
        nOV = no * nv
        if nOV > 5000:
            print("Number determinants: ", nOV)
            sys.exit("CIS too expensive. Quitting.")
        A = self._singles()
        print("Diagonalizing Hamiltonian...")
        w, V = torch.linalg.eigh(A)
        # MO dipole integrals, spin-blocked (mmd/postscf.py:295-299)
        C = torch.as_tensor(np.real(np.asarray(mol.C)), dtype=torch.float64, device=A.device)
        Mmo = C.T @ mol._dev["M"].to(torch.float64) @ C
        sp = torch.arange(mol.norb, device=A.device)
        Ms = Mmo[:, sp // 2][:, :, sp // 2] * (sp[:, None] % 2 == sp[None, :] % 2).to(torch.float64)
        D = Ms[:, :no, no:].reshape(3, nOV)
        td = D @ V                                                    # (3, states)
        f = (2.0 / 3.0) * w * (td * td).sum(0)
        mol.cis_omega = (w * 27.211399).cpu().numpy()
        mol.cis_oscil = f.cpu().numpy()
        print("\nConfiguration Interaction Singles (CIS)")
        print("------------------------------")
        print("# Determinants: ", nOV)
        print("nOcc * nVirt:   ", nOV)
        for state in range(min(nOV, 30)):
            print("CIS state %2s (eV): %12.4f (f=%6.4f)" % (state + 1, mol.cis_omega[state], mol.cis_oscil[state]))

    def TDHF(self, alg="hermitian"):
        """Time-dependent Hartree-Fock (RPA) excitation energies in eV, ``mol.tdhf_omega``
        (mmd/postscf.py:325-400), by the algorithm ``alg`` names."""
        mol = self.mol
        torch = mol.context.torch
        A, B = self._singles(with_b=True)
        nOV = A.shape[0]
        if alg == "hermitian":
            # principal square root of the symmetric positive-definite A - B
            lam, U = torch.linalg.eigh(A - B)
            root = (U * lam.sqrt()) @ U.T
            H = root @ (A + B) @ root
            w = torch.linalg.eigvalsh(0.5 * (H + H.T)).sqrt()
        elif alg == "reduced":
            H = (A - B) @ (A + B)
            w = torch.sort(torch.linalg.eigvals(H).sqrt().real).values
        elif alg == "full":
            H = torch.cat([torch.cat([A, B], 1), torch.cat([-B.T, -A.T], 1)], 0)
            lam = torch.linalg.eigvals(H)
            w = torch.sort(lam.real).values[nOV:]
        else:
            raise ValueError("alg must be 'hermitian', 'reduced' or 'full'")
        mol.tdhf_omega = (w * 27.211399).cpu().numpy()
        print("\nTime-dependent Hartree-Fock (TDHF)")
        print("------------------------------")
        print("Algorithm:        ", alg)
        print("Matrix shape:     ", len(H))
        print("2 * nOcc * nVirt: ", 2 * nOV)
        for state in range(min(nOV, 10)):
            print("TDHF state %2s (eV): %12.4f" % (state + 1, mol.tdhf_omega[state]))

    def _absent(self, name):
        raise NotImplementedError(f"PostSCF.{name} is not part of this implementation (determinant-string method)")

    def CISD(self, *a, **k):
        self._absent("CISD")

    def FCI(self, *a, **k):
        self._absent("FCI")
