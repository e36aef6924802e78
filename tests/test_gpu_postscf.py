"""AO->MO transform and MP2 on the GPU (mmd.postscf) against the reference's own MP2
energies (tests/golden/mp2.json, made by tests/golden/make_golden_mp2.py), the
reference's tests/test014.py and test016.py pins, and a numpy transform of the same
integrals and orbitals."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "mp2.json")


def _cases():
    with open(GOLDEN) as f:
        return json.load(f)["cases"]


@pytest.mark.parametrize("case", _cases(), ids=lambda c: f"{c['name']}_{c['basis']}")
def test_mp2_matches_reference(built_lib, case):
    from mmd.molecule import Molecule
    from mmd.postscf import PostSCF
    mol = Molecule(geometry=case["geometry"], basis=case["basis"])
    mol.RHF(doPrint=False, conver=1e-12)
    assert abs(mol.energy.real - case["energy"]) < 1e-10
    PostSCF(mol).MP2()
    assert abs(mol.emp2.real - case["emp2_spatial"]) < 1e-10
    PostSCF(mol).MP2(spin_orbital=True)
    assert abs(mol.emp2.real - case["emp2_spin"]) < 1e-10


def test_ao2mo_equals_numpy_transform(built_lib):
    from mmd.molecule import Molecule
    from mmd.postscf import PostSCF
    water = _cases()[1]
    mol = Molecule(geometry=water["geometry"], basis=water["basis"])
    mol.RHF(doPrint=False, conver=1e-10)
    PostSCF(mol)
    C = np.real(mol.C)
    ref = np.einsum("pqrs,pP,qQ,rR,sS->PQRS", mol.TwoE, C, C, C, C, optimize=True)
    assert np.abs(mol.single_bar - ref).max() < 1e-12
    # spin blocking as the reference's Kronecker products (mmd/postscf.py:31-35)
    spin_block = np.kron(np.kron(ref, np.eye(2)).transpose(), np.eye(2))
    dbl = spin_block.transpose(0, 2, 1, 3) - spin_block.transpose(0, 2, 3, 1)
    assert np.abs(mol.double_bar - dbl).max() < 1e-12
    assert np.abs(mol.Hp - np.kron(np.einsum("uj,vi,uv", C, C, mol.Core), np.eye(2))).max() < 1e-12
    assert np.abs(mol.fs - np.kron(np.diag(np.real(mol.MO)), np.eye(2))).max() == 0.0


def test_reference_pins_test014_test016(built_lib):
    from mmd.molecule import Molecule
    from mmd.postscf import PostSCF
    methane = """
0 1
C    0.000000    0.000000    0.000000
H    0.626425042   -0.626425042   -0.626425042
H    0.626425042    0.626425042    0.626425042
H   -0.626425042    0.626425042   -0.626425042
H   -0.626425042   -0.626425042    0.626425042
"""
    mol = Molecule(geometry=methane, basis="3-21G")
    mol.RHF(direct=False, doPrint=False)
    PostSCF(mol).MP2()
    np.testing.assert_allclose(mol.energy.real, -39.9768654272)
    np.testing.assert_allclose(mol.emp2.real, -40.076963354817)
    he2 = """
0 1
He   0.0 0.0 0.0
He   0.0 0.0 0.75
"""
    mol = Molecule(geometry=he2, basis="cc-pvDZ")
    mol.RHF(doPrint=False)
    PostSCF(mol).MP2()
    spatial = mol.emp2.real
    PostSCF(mol).MP2(spin_orbital=True)
    assert np.allclose(spatial, mol.emp2.real)
    assert np.allclose(-5.29648041091, mol.energy.real)
    assert np.allclose(-5.3545864180140, spatial)
