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
    """The Schwarz table as a flat array screen[p(p+1)/2+q], read at call time like the
    reference's per-quartet ``screen[ij]`` lookups (fock.pyx:46-48), so values edited
    in place are seen.  A dict whose keys are 0..n-1 in insertion order (how
    ``Molecule.build`` makes it) is read through ``values()``; its key order is
    verified once per dict object and length, any other dict key by key."""
    n = N * (N + 1) // 2
    if not isinstance(screen, dict):
        return np.ascontiguousarray(screen, dtype=np.float64).reshape(-1)
    if len(screen) == n:
        memo = _KEY_ORDER_OK.get(id(screen))
        if memo is None or memo[0] is not screen or memo[1] != n:
            ok = next(iter(screen)) == 0 and next(reversed(screen)) == n - 1 and \
                all(a == b for a, b in zip(screen, range(n)))
            memo = (screen, n, ok)
            _KEY_ORDER_OK.clear()  # one dict remembered at a time
            _KEY_ORDER_OK[id(screen)] = memo
        if memo[2] and next(reversed(screen)) == n - 1:
            return np.fromiter(screen.values(), dtype=np.float64, count=n)
    return np.fromiter(map(screen.__getitem__, range(n)), dtype=np.float64, count=n)


_KEY_ORDER_OK: dict = {}


def formPT(P, P_old, bfs, nbasis, screen, tol):
    """Two-electron Fock contribution G(P - P_old), unsymmetrised, as a complex N x N
    array (cython/fock.pyx:13-87): the reference's Schwarz x density screening of
    every function quartet at ``tol``, degeneracy factors and scatter, computed by
    the GPU class kernels (a complex density difference is two real builds).  The
    Schwarz table is re-uploaded to the device whenever its contents differ from
    the last upload (``screen=None`` keeps the table the device computed)."""
    N = int(nbasis)
    ctx = context_for(bfs)
    torch = ctx.torch
    if screen is not None:
        arr = _screen_array(screen, N)
        last = getattr(ctx, "_user_screen_arr", None)
        if last is None or last.shape != arr.shape or not np.array_equal(last, arr):
            ctx.set_screen(arr)
            ctx._user_screen_arr = arr
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
