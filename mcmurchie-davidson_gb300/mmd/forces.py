"""Analytic RHF nuclear forces on the GPU, behind the reference's ``Forces`` mixin.

``mol.forces()`` sets ``atom.forces`` (not mass weighted, -dE/dR) for every atom, as
mmd/forces.py:8-97 does, and ``mol._forces`` collects them (mmd/molecule.py:47-53).
The reference assembles, per atom and direction, full derivative matrices dS, dT, dV
and a derivative ERI tensor (N^4) from the Cython integrals of cython/grad.pyx; here
one call of ``mmdg_rhf_gradient`` computes the derivative integrals on the GPU shell
pair by shell pair and shell quartet by shell quartet and contracts them at once with
P and W = P F P, so nothing of size N^4 is formed.
"""
from __future__ import annotations

import ctypes
import sys

import numpy as np

from . import _native


# Schwarz screening of the two-electron derivative terms: a derivative integral is at
# most ~2 sqrt(exponent) times the integral bound Q_ab Q_cd, and the density factor at
# most a few units, so skipped quartets change a force by < 1e-12 each at 1e-16
GRADIENT_SCHWARZ_TOL = 1e-16


class Forces:
    """Nuclear gradient methods for the molecule object (mmd/forces.py:6-97)."""

    def forces(self, qtol=GRADIENT_SCHWARZ_TOL):
        """Compute the nuclear forces of the converged RHF state.  ``qtol``: shell
        quartets with Q_ab Q_cd below it are skipped (0 keeps all, as the reference)."""
        if not self.is_converged:
            sys.exit("Need to converge SCF before computing gradient")
        ctx = self.context
        torch = ctx.torch
        dev = f"cuda:{ctx.device}"
        P = np.ascontiguousarray(np.real(np.asarray(self.P)), dtype=np.float64)
        F = np.ascontiguousarray(np.real(np.asarray(self.F)), dtype=np.float64)
        Pd = torch.as_tensor(P, device=dev)
        Wd = (Pd @ torch.as_tensor(F, device=dev) @ Pd).contiguous()
        ss = ctx.sets[0]
        bf_atom = np.asarray(self.bf_atom)
        first = np.array([row[row >= 0][0] for row in ss.func])
        shell_atom = np.ascontiguousarray(bf_atom[first], dtype=np.int32)
        natom = len(self.atoms)
        xyz = np.ascontiguousarray(np.array([a.origin for a in self.atoms], dtype=np.float64).reshape(-1))
        Z = np.ascontiguousarray(np.array([float(a.charge) for a in self.atoms]))
        grad = np.zeros(3 * natom)
        lib = _native.lib()
        _native.check(lib.mmdg_rhf_gradient(ctx._h, ctypes.c_void_p(Pd.data_ptr()), ctypes.c_void_p(Wd.data_ptr()),
                                            natom, _native._ptr(xyz), _native._ptr(Z), _native._ptr(shell_atom),
                                            float(qtol), _native._ptr(grad), _native.stream_ptr()),
                      "mmdg_rhf_gradient")
        grad = grad.reshape(natom, 3)
        for a, atom in enumerate(self.atoms):
            atom.forces = -grad[a]
        return -grad
