"""Analytic RHF forces on the GPU (mmd.forces, mmdg_rhf_gradient) against the
reference's own forces (tests/golden/forces.json, made by
tests/golden/make_golden_forces.py from its Cython derivative integrals), the
reference's tests/test001.py pin, central finite differences of the GPU RHF energy
(d shells), and the vanishing net torque of an isolated cluster."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "forces.json")


def _cases():
    with open(GOLDEN) as f:
        return json.load(f)["cases"]


@pytest.mark.parametrize("case", _cases(), ids=lambda c: f"{c['name']}_{c['basis']}")
def test_forces_match_reference(built_lib, case):
    from mmd.molecule import Molecule
    mol = Molecule(geometry=case["geometry"], basis=case["basis"])
    mol.RHF(doPrint=False, conver=1e-12)
    assert abs(mol.energy.real - case["energy"]) < 1e-10
    mol.forces()
    ref = np.array(case["forces"])
    assert np.abs(mol._forces - ref).max() < 1e-9, np.abs(mol._forces - ref).max()


def test_reference_pin_test001(built_lib):
    from mmd.molecule import Molecule
    mol = Molecule(geometry="\n0 1\nH 0.0 0.0 0.74\nH 0.0 0.0 0.00\n", basis="sto-3g")
    mol.RHF(doPrint=False)
    np.testing.assert_allclose(mol.energy.real, -1.11675930740, atol=1e-12)
    mol.forces()
    ref = np.array([[0.0, 0.0, -0.027679601], [0.0, 0.0, 0.027679601]])
    np.testing.assert_allclose(mol._forces, ref, atol=1e-9)


def _geom(sym, xyz):
    return "\n0 1\n" + "\n".join(f"{s} {x:.12f} {y:.12f} {z:.12f}" for s, (x, y, z) in zip(sym, xyz)) + "\n"


def test_forces_equal_finite_differences_with_d_shells(built_lib):
    from mmd.molecule import Molecule
    sym = ["O", "H", "H"]
    xyz = np.array([[0.0, -0.07, 0.01], [0.80, 0.62, 0.03], [-0.88, 0.56, -0.02]])
    mol = Molecule(geometry=_geom(sym, xyz), basis="6-31gss")
    mol.RHF(doPrint=False, conver=1e-12)
    f = mol.forces()
    h = 1e-4  # Angstrom
    for atom, d in ((0, 1), (1, 0), (2, 2)):
        E = []
        for s in (+1, -1):
            x = xyz.copy()
            x[atom, d] += s * h
            E.append(float(Molecule(geometry=_geom(sym, x), basis="6-31gss").RHF(doPrint=False, conver=1e-12)))
        dEdx = (E[0] - E[1]) / (2 * h / 0.52917721092)
        assert abs(-dEdx - f[atom, d]) < 2e-7, (atom, d, -dEdx, f[atom, d])


def test_cluster_forces_have_no_net_force_or_torque(built_lib):
    from mmd.clusters import water_cluster
    from mmd.molecule import Molecule
    mol = Molecule(water_cluster(3, seed=4), "6-31gss")
    mol.RHF(doPrint=False, conver=1e-10)
    f = mol.forces()
    R = np.array([a.origin for a in mol.atoms])
    assert np.abs(f.sum(axis=0)).max() < 1e-10
    assert np.abs(np.cross(R, f).sum(axis=0)).max() < 1e-7


def test_schwarz_screened_forces_equal_unscreened(built_lib):
    """Skipping shell quartets with Q_ab Q_cd < 1e-16 (the default) changes no force
    component by more than 1e-11 on a spread-out (H2O)6 cluster."""
    from mmd.clusters import water_cluster
    from mmd.molecule import Molecule
    mol = Molecule(water_cluster(6, seed=8), "6-31g")
    mol.RHF(doPrint=False, conver=1e-10)
    f_all = mol.forces(qtol=0.0).copy()
    f_scr = mol.forces()
    assert np.abs(f_scr - f_all).max() < 1e-11
