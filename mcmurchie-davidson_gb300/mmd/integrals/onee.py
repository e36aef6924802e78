"""One-electron integrals behind the reference's ``mmd.integrals.onee`` API.

``S(a, b)``, ``T(a, b)``, ``V(a, b, C)`` and ``Mu(a, b, C, direction)`` keep the
signatures of cython/onee.pyx:14-69; they evaluate the pair on the GPU
(``mmdg_one_electron``).  ``Molecule`` computes whole matrices in one launch.
``RxDel`` is importable but raises (no consumer of the angular-momentum integrals).
``_boys(n, T)`` is the Boys-function test hook (cython/onee.pyx:195-196), served
by the GPU Boys kernel for integer orders 0..8 (the orders the ERI path uses).
"""
from __future__ import annotations

import ctypes

import numpy as np

from .. import _native
from .shells import shells_from_bfs


def _pair_matrices(a, b, C=None, origin=None):
    ctx = _native.Context(shells_from_bfs([a, b]))
    torch = ctx.torch
    dev = f"cuda:{ctx.device}"
    S = torch.empty(4, dtype=torch.float64, device=dev)
    T, V = torch.empty_like(S), torch.empty_like(S)
    M = torch.empty(12, dtype=torch.float64, device=dev)
    C = np.zeros(3) if C is None else np.asarray(C, dtype=np.float64)
    xyz = np.ascontiguousarray(C.reshape(3))
    Z = np.array([-1.0])  # the kernel returns -Z*V; Z = -1 yields +V, the sign of onee.V
    org = np.ascontiguousarray(np.zeros(3) if origin is None else np.asarray(origin, dtype=np.float64))
    _native.check(_native.lib().mmdg_one_electron(ctx._h, 1, _native._ptr(np.zeros(1, dtype=np.int32)),
                                                   _native._ptr(xyz), _native._ptr(Z), _native._ptr(org),
                                                   ctypes.c_void_p(S.data_ptr()), ctypes.c_void_p(T.data_ptr()),
                                                   ctypes.c_void_p(V.data_ptr()), ctypes.c_void_p(M.data_ptr()),
                                                   _native.stream_ptr()), "mmdg_one_electron")
    out = (S.cpu().numpy().reshape(2, 2), T.cpu().numpy().reshape(2, 2), V.cpu().numpy().reshape(2, 2),
           M.cpu().numpy().reshape(3, 2, 2))
    ctx.close()
    return out


def S(a, b):
    """Overlap (onee.pyx:14-23)."""
    return float(_pair_matrices(a, b)[0][0, 1])


def T(a, b):
    """Kinetic energy (onee.pyx:47-56)."""
    return float(_pair_matrices(a, b)[1][0, 1])


def V(a, b, C):
    """Nuclear attraction of a unit positive charge at C, without the -Z factor (onee.pyx:60-69)."""
    return float(_pair_matrices(a, b, C=C)[2][0, 1])


def Mu(a, b, C, direction):
    """Dipole integral about origin C (onee.pyx:27-36)."""
    k = {"x": 0, "y": 1, "z": 2}[direction.lower()]
    return float(_pair_matrices(a, b, origin=C)[3][k, 0, 1])


def RxDel(a, b, C, direction):
    """Angular-momentum integral (onee.pyx:36-46): importable under the reference's
    name, but not evaluated here -- nothing in the reference reads ``Molecule.L``, and
    it is no part of the two-electron path this package serves."""
    raise NotImplementedError("RxDel: the angular-momentum integrals are not implemented on the GPU path")


def _boys(n, T):
    """F_n(T) on the GPU for integer n in 0..8."""
    if float(n) != int(n) or not (0 <= int(n) <= 8):
        raise ValueError("the GPU Boys kernel serves integer orders 0..8 (the orders of (dd|dd) and below)")
    ctx = _native.scratch_context()
    torch = ctx.torch
    t = torch.tensor([float(T)], dtype=torch.float64, device="cuda")
    return float(ctx.boys(int(n), t).item())
