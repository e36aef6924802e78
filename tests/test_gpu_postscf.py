"""AO->MO transform, MP2, CIS and TDHF on the GPU (mmd.postscf) against the
reference's own results (tests/golden/mp2.json and excited.json, made by the
make_golden_mp2.py and make_golden_excited.py scripts beside them), the reference's
tests/test014.py, test016.py, test019.py and test020.py pins, and a numpy transform
of the same integrals and orbitals."""
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


EXCITED = os.path.join(os.path.dirname(__file__), "golden", "excited.json")


def test_cis_matches_reference(built_lib):
    """CIS energies and oscillator strengths against the reference's own CIS
    (tests/golden/excited.json, made by tests/golden/make_golden_excited.py) and the
    Gaussian 16 pins of the reference's tests/test019.py."""
    from mmd.molecule import Molecule
    from mmd.postscf import PostSCF
    with open(EXCITED) as f:
        gold = json.load(f)["cis"]
    mol = Molecule(geometry=gold["geometry"], basis=gold["basis"])
    mol.RHF(doPrint=False, conver=1e-12)
    PostSCF(mol).CIS()
    assert mol.cis_omega.shape == (160,)
    assert np.abs(mol.cis_omega - np.asarray(gold["omega"])).max() < 1e-8      # eV
    assert np.abs(mol.cis_oscil - np.asarray(gold["oscil"])).max() < 1e-10
    gau_ref = [6.5822, 6.5822, 6.5822, 7.7597, 7.8156, 7.8156, 7.8156, 8.4377, 8.4377,
               8.4377, 9.0903, 9.0903, 9.0903, 9.3334, 10.5493]
    assert np.allclose(np.asarray(gau_ref), mol.cis_omega[:15])
    with pytest.raises(NotImplementedError):
        PostSCF(mol).CIS(bitstring=True)


def test_tdhf_matches_reference(built_lib):
    """TDHF by the three algorithms against the reference's own results and the
    tests/test020.py pins and consistency checks."""
    from mmd.molecule import Molecule
    from mmd.postscf import PostSCF
    with open(EXCITED) as f:
        gold = json.load(f)["tdhf"]
    mol = Molecule(geometry=gold["geometry"], basis=gold["basis"])
    mol.RHF(doPrint=False, conver=1e-12)
    post = PostSCF(mol)
    for alg in ("hermitian", "reduced", "full"):
        post.TDHF(alg=alg)
        assert mol.tdhf_omega.shape == (40,)
        assert np.abs(mol.tdhf_omega - np.asarray(gold[alg])).max() < 1e-8
    mol = Molecule(geometry=gold["geometry"], basis=gold["basis"])
    mol.RHF()
    PostSCF(mol).TDHF()
    gau_ref = [7.7597, 7.7597, 7.7597, 8.1564, 8.1564, 8.1564, 9.5955, 9.5955, 9.5955, 9.6540]
    assert np.allclose(np.asarray(gau_ref), mol.tdhf_omega[:10])
    ref_omega = mol.tdhf_omega
    PostSCF(mol).TDHF(alg="reduced")
    assert np.allclose(mol.tdhf_omega, ref_omega)
    PostSCF(mol).TDHF(alg="full")
    assert np.allclose(mol.tdhf_omega, ref_omega)
    with pytest.raises(ValueError):
        PostSCF(mol).TDHF(alg="davidson")
