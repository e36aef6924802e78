"""RT-TDHF (mmd.realtime) on the GPU against the reference's own trajectories
(tests/golden/rt_trajectories.npz, made by tests/golden/make_golden_rt.py) and the
reference's tests/test011.py energy-conservation check."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "rt_trajectories.npz")
H2 = """
0 1
H 0.0 0.0 0.74
H 0.0 0.0 0.00
"""
WATER = """
0 1
O    0.000000      -0.075791844    0.000000
H    0.866811829    0.601435779    0.000000
H   -0.866811829    0.601435779    0.000000
"""


def pulse(t):
    return np.exp(-((t - 1.0) ** 2) / 0.25)


@pytest.mark.parametrize("name,geom", [("h2", H2), ("water", WATER)])
@pytest.mark.parametrize("order,direction", [(2, "z"), (4, "z"), (4, "x")])
def test_magnus_trajectories_match_reference(built_lib, name, geom, order, direction):
    from mmd.molecule import Molecule
    from mmd.realtime import RealTime
    g = np.load(GOLDEN)
    mol = Molecule(geometry=geom, basis="sto-3g")
    rt = RealTime(mol, numsteps=int(g["steps"]), stepsize=float(g["dt"]), field=float(g["field"]), pulse=pulse)
    getattr(rt, f"Magnus{order}")(direction=direction)
    key = f"{name}_m{order}{direction}"
    assert np.abs(np.array(rt.shape) - g[key + "_shape"]).max() < 1e-15  # libm exp may differ by an ulp
    assert np.abs(np.array(rt.dipole) - g[key + "_dipole"]).max() < 1e-9
    assert np.abs(np.array(rt.Energy) - g[key + "_energy"]).max() < 1e-9


@pytest.mark.parametrize("order", [2, 4])
def test_field_free_propagation_conserves_energy(built_lib, order):
    """The reference's tests/test011.py: no pulse, 100 steps of 0.2, H2 / STO-3G."""
    from mmd.molecule import Molecule
    from mmd.realtime import RealTime
    mol = Molecule(geometry=H2, basis="sto-3g")
    rt = RealTime(mol, numsteps=100, stepsize=0.2, field=0.0001, pulse=None)
    e0 = rt.mol.energy.real
    getattr(rt, f"Magnus{order}")(direction="z")
    np.testing.assert_allclose(e0 * np.ones_like(rt.Energy), rt.Energy)


def test_host_buildfock_with_a_complex_density(built_lib):
    """mol.buildFock (conventional) for a complex Hermitian density equals the
    reference's einsums (mmd/scf.py:96-100) on the same ERI tensor."""
    from mmd.molecule import Molecule
    mol = Molecule(geometry=WATER, basis="sto-3g")
    mol.RHF(doPrint=False)
    rng = np.random.default_rng(2)
    N = mol.nbasis
    A = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    mol.P = 0.1 * (A + A.conj().T)
    mol.buildFock()
    T = mol.TwoE.astype(complex)
    J = np.einsum("pqrs,sr->pq", T, mol.P)
    K = np.einsum("psqr,sr->pq", T, mol.P)
    assert np.abs(mol.F - (mol.Core + 2 * J - K)).max() < 1e-12
