"""Seeded synthetic water clusters (the workloads of the two-electron hot path).

No dataset is involved: every cluster is generated from a seed.  A monomer with
the reference's water geometry (Angstrom; the same geometry as the reference's
tests/test002.py and README sample input) is centred on its centroid, rotated
rigidly by a uniform random unit quaternion (Shoemake's method), and placed on a
simple-cubic lattice of spacing ``spacing`` (default 3.0 Angstrom) with a uniform
jitter of +-``jitter`` (0.3 Angstrom) per Cartesian component.  Sites are filled
in row-major order of a 4 x 4 x ceil(n/16) lattice, so n=16 is the 4x4x1 sheet
and n=32 the 4x4x2 slab.  If any O-O distance falls below ``min_oo`` (2.5
Angstrom) the whole cluster is redrawn from the same generator stream.

This module has no package-relative imports so that fixture scripts can load it
by file path.
"""
from __future__ import annotations

import numpy as np

WATER = np.array([
    [0.000000000, -0.075791844, 0.000000000],   # O
    [0.866811829, 0.601435779, 0.000000000],    # H
    [-0.866811829, 0.601435779, 0.000000000],   # H
])
WATER_SYMBOLS = ("O", "H", "H")


def random_rotation(rng: np.random.Generator) -> np.ndarray:
    """Uniform random rotation matrix from a Shoemake unit quaternion."""
    u1, u2, u3 = rng.random(3)
    a, b = np.sqrt(1.0 - u1), np.sqrt(u1)
    w = a * np.sin(2 * np.pi * u2)
    x = a * np.cos(2 * np.pi * u2)
    y = b * np.sin(2 * np.pi * u3)
    z = b * np.cos(2 * np.pi * u3)
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
        [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
        [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
    ])


def water_cluster_coords(n: int, seed: int, spacing: float = 3.0, jitter: float = 0.3,
                         min_oo: float = 2.5, max_tries: int = 1000) -> tuple[list[str], np.ndarray]:
    """Symbols and Angstrom coordinates (3n x 3) of a seeded (H2O)_n cluster."""
    if n < 1:
        raise ValueError("n must be >= 1")
    rng = np.random.default_rng(seed)
    mono = WATER - WATER.mean(axis=0)
    nz = (n + 15) // 16
    sites = np.array([[ix, iy, iz] for iz in range(nz) for iy in range(4) for ix in range(4)], dtype=float)[:n]
    for _ in range(max_tries):
        coords = []
        for s in sites:
            R = random_rotation(rng)
            shift = s * spacing + rng.uniform(-jitter, jitter, 3)
            coords.append(mono @ R.T + shift)
        coords = np.concatenate(coords)
        oxy = coords[0::3]
        d = np.linalg.norm(oxy[:, None, :] - oxy[None, :, :], axis=-1)
        d[np.diag_indices(n)] = np.inf
        if n == 1 or d.min() >= min_oo:
            return list(WATER_SYMBOLS) * n, coords
    raise RuntimeError("could not place cluster")


def geometry_string(symbols, coords, charge: int = 0, multiplicity: int = 1) -> str:
    lines = [f"{charge} {multiplicity}"]
    for s, (x, y, z) in zip(symbols, coords):
        lines.append(f"{s} {x:.10f} {y:.10f} {z:.10f}")
    return "\n" + "\n".join(lines) + "\n"


def water_cluster(n: int, seed: int, **kw) -> str:
    """Geometry string (the format ``Molecule(geometry, basis)`` reads) of a seeded (H2O)_n."""
    sym, xyz = water_cluster_coords(n, seed, **kw)
    return geometry_string(sym, xyz)


WATER_STO3G_GEOMETRY = geometry_string(WATER_SYMBOLS, WATER)
