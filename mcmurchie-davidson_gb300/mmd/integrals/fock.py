"""Direct Fock digestion on the GPU, behind the reference's ``mmd.integrals.fock`` API.

``formPT(P, P_old, bfs, nbasis, screen, tol)`` keeps the signature and result of
cython/fock.pyx:13-87: the unsymmetrised two-electron update G(P - P_old), with
the same Schwarz x density screening, degeneracy factors and Coulomb/exchange
scatter pattern, returned as a complex array (the caller symmetrises).
"""
from __future__ import annotations

import numpy as np

from .twoe import context_for


def _screen_array(screen, N):
    if isinstance(screen, dict):
        return np.fromiter((screen[i] for i in range(N * (N + 1) // 2)), dtype=np.float64, count=N * (N + 1) // 2)
    return np.ascontiguousarray(screen, dtype=np.float64)


def formPT(P, P_old, bfs, nbasis, screen, tol):
    """Two-electron Fock contribution G(P - P_old), unsymmetrised, as a complex N x N
    array (cython/fock.pyx:13-87): the reference's Schwarz x density screening of
    every function quartet at ``tol``, degeneracy factors and scatter, computed by
    the GPU class kernels (a complex density difference is two real builds)."""
    N = int(nbasis)
    ctx = context_for(bfs)
    torch = ctx.torch
    if screen is not None and screen is not getattr(ctx, "_user_screen_obj", None):
        ctx.set_screen(_screen_array(screen, N))
        ctx._user_screen_obj = screen
    dP = np.asarray(P) - np.asarray(P_old)
    parts = [np.real(dP)]
    if np.iscomplexobj(dP) and np.any(np.imag(dP) != 0):
        parts.append(np.imag(dP))
    G = np.zeros((N, N), dtype=complex)
    for k, part in enumerate(parts):
        d = torch.as_tensor(np.ascontiguousarray(part, dtype=np.float64), device=f"cuda:{ctx.device}").reshape(-1)
        g = ctx.fock(d, tol=float(tol)).reshape(N, N).cpu().numpy()
        G += g if k == 0 else 1j * g
    return G
