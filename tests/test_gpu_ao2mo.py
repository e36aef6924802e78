"""The AO -> MO transform kernel (mmdg_ao2mo; the four einsums of mmd/postscf.py:26-27)
against the same contraction in float64 torch, on sizes that do and do not fill
the kernel's 64-wide tiles, and its use by PostSCF (MP2 energies are pinned to the
reference in test_gpu_postscf.py)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N", [7, 13, 64, 70])
def test_ao2mo_kernel_matches_the_four_einsums(N):
    import torch
    from mmd import _native
    g = torch.Generator(device="cpu").manual_seed(N)
    A = torch.randn(N, N, N, N, generator=g, dtype=torch.float64)
    eri = (A + A.permute(1, 0, 2, 3) + A.permute(0, 1, 3, 2) + A.permute(2, 3, 0, 1)).cuda()
    C = torch.randn(N, N, generator=g, dtype=torch.float64).cuda()
    ref = torch.einsum("pqrs,pP,qQ,rR,sS->PQRS", eri, C, C, C, C)
    src = eri.clone()
    got = _native.ao2mo(C, eri.reshape(-1)).view(N, N, N, N)
    assert torch.equal(eri, src)  # the input is left unchanged
    scale = ref.abs().max().item()
    assert (got - ref).abs().max().item() < 1e-13 * scale


def test_postscf_uses_the_kernel_and_keeps_the_mo_integrals_symmetric():
    from mmd.molecule import Molecule
    from mmd.postscf import PostSCF
    mol = Molecule("\n0 1\nO 0.0 -0.075791844 0.0\nH 0.866811829 0.601435779 0.0\nH -0.866811829 0.601435779 0.0\n",
                   "6-31g")
    mol.RHF(doPrint=False, conver=1e-10)
    ps = PostSCF(mol)
    mo = mol.single_bar
    assert np.abs(mo - mo.transpose(1, 0, 2, 3)).max() < 1e-12
    assert np.abs(mo - mo.transpose(2, 3, 0, 1)).max() < 1e-12
    # (PQ|RS) from the device AO tensor and C by numpy
    C = np.real(np.asarray(mol.C))
    ref = np.einsum("pqrs,pP,qQ,rR,sS->PQRS", mol.TwoE, C, C, C, C, optimize=True)
    assert np.abs(mo - ref).max() < 1e-12
    assert ps is not None
