"""Learned initial guess: host-side geometry logic (CPU) and the GPU MLP kernels'
gradients against the CPU oracle; the trained network's gain over the core guess."""
import os

import numpy as np
import pytest


def _water_mol(n=3, seed=7):
    from mmd.clusters import water_cluster
    from mmd.molecule import Molecule
    return Molecule(water_cluster(n, seed=seed), "6-31g")


def _rotated(mol, R):
    from mmd.molecule import Molecule
    lines = [f"{0} {1}"]
    for a in mol.atoms:
        x = R @ (a.origin * 0.52917721092)
        lines.append(f"{'O' if a.charge == 8 else 'H'} {x[0]:.12f} {x[1]:.12f} {x[2]:.12f}")
    return Molecule("\n" + "\n".join(lines) + "\n", "6-31g")


def test_pair_features_are_rotation_invariant():
    from mmd import guess as G
    from mmd.clusters import random_rotation
    m = _water_mol()
    R = random_rotation(np.random.default_rng(1))
    p1, f1, _, _, _ = G.molecule_samples(m)
    p2, f2, _, _, _ = G.molecule_samples(_rotated(m, R))
    assert p1 == p2
    assert np.abs(f1 - f2).max() < 1e-5


def test_block_targets_round_trip():
    """targets (local frames) -> assemble (lab frame) reproduces every block within the cutoff."""
    from mmd import guess as G
    m = _water_mol(2)
    rng = np.random.default_rng(2)
    A = rng.standard_normal((m.nbasis, m.nbasis))
    P = A + A.T
    pairs, F, Y, M, (Z, R, off) = G.molecule_samples(m, P)
    Pa = G.assemble(Y, Z, R, off, pairs, m.nbasis)
    assert np.abs(Pa - P).max() < 1e-5  # float32 targets; both waters are within 8 Angstrom


def test_rotated_targets_are_invariant():
    from mmd import guess as G
    from mmd.clusters import random_rotation
    m = _water_mol(2, seed=5)
    R = random_rotation(np.random.default_rng(3))
    # density of the rotated molecule = the rotated density (p blocks rotate, s do not)
    rng = np.random.default_rng(4)
    A = rng.standard_normal((m.nbasis, m.nbasis))
    P = A + A.T
    Z, X, off = G.molecule_layout(m)
    T = np.zeros((m.nbasis, m.nbasis))
    for a, z in enumerate(Z):
        n = G.NFUNC[int(z)]
        T[off[a]:off[a] + n, off[a]:off[a] + n] = G.block_transform(int(z), R)
    Prot = T @ P @ T.T
    _, _, Y1, _, _ = G.molecule_samples(m, P)
    _, _, Y2, _, _ = G.molecule_samples(_rotated(m, R), Prot)
    assert np.abs(Y1 - Y2).max() < 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("B", [300, 5000])  # 5000 rows: the split-K weight-gradient GEMMs
def test_mlp_kernels_gradients_match_cpu_oracle(B):
    import torch
    import mlp_oracle as O
    from mmd import guess as G
    net = G.DensityMLP(seed=3)
    rng = np.random.default_rng(9)
    X = rng.standard_normal((B, G.NIN)).astype(np.float32)
    T = rng.standard_normal((B, G.NOUT)).astype(np.float32)
    M = (rng.random((B, G.NOUT)) < 0.6).astype(np.float32)
    # the oracle uses the same BF16-rounded weights the kernels read
    W = [w.float().cpu().numpy().astype(np.float64) for w in net.Wb]
    b = [x.cpu().numpy().astype(np.float64) for x in net.b]
    loss_o, grads_o = O.loss_and_grads(W, b, X.astype(np.float64), T.astype(np.float64), M.astype(np.float64))
    acts = net.forward(torch.tensor(X, device="cuda"))
    loss, dY = net.loss_grad(acts[-1][2], torch.tensor(T, device="cuda"), torch.tensor(M, device="cuda"))
    grads = net.backward(acts, dY)
    assert abs(loss.item() - loss_o) < 1e-4 * abs(loss_o)
    Y_o = O.forward(W, b, X.astype(np.float64))[-1][2]
    assert np.abs(acts[-1][2].cpu().numpy() - Y_o).max() < 1e-4 * np.abs(Y_o).max()
    for (dW, db), (dWo, dbo) in zip(grads, grads_o):
        assert np.abs(dW.cpu().numpy() - dWo).max() < 2e-3 * np.abs(dWo).max()
        assert np.abs(db.cpu().numpy() - dbo).max() < 2e-3 * np.abs(dbo).max()


@pytest.mark.gpu
def test_learned_guess_gains_over_core_guess():
    """The committed network (trained by mmd.guess_train on 20k clusters) cuts the SCF
    iterations of held-out (H2O)8 clusters at conver 1e-8; converged tightly and
    polished by an FP64 build, both guesses give the same energies."""
    from mmd import guess as G
    from mmd.batch import BatchRHF
    from mmd.clusters import water_cluster
    from mmd.molecule import Molecule
    assert os.path.exists(G.WEIGHTS)
    net = G.DensityMLP.load()
    geoms = [water_cluster(8, seed=900000 + k) for k in range(8)]
    gs = [G.predict_density(net, Molecule(g, "6-31g")) for g in geoms]
    core = BatchRHF(geoms, "6-31g")
    core.run(conver=1e-8)
    learned = BatchRHF(geoms, "6-31g")
    learned.run(conver=1e-8, guess=gs)
    assert core.converged.all() and learned.converged.all()
    assert not learned.reverted.any()
    assert learned.iterations.mean() < 0.8 * core.iterations.mean()
    Ec = core.run(conver=1e-10, polish=True)
    El = learned.run(conver=1e-10, guess=gs, polish=True)
    assert np.abs(El - Ec).max() < 1e-9


def test_fallback_rule_counts_three_growths():
    from mmd.scf import diis_error_growing as grow
    assert not grow([])
    assert not grow([1.0, 2.0, 3.0])          # only two growths so far
    assert grow([1.0, 2.0, 3.0, 4.0])
    assert not grow([1.0, 2.0, 1.5, 4.0])
    assert grow([9.0, 1.0, 2.0, 3.0, 4.0])    # only the last three steps count
    h = [np.array([1.0, 5.0]), np.array([2.0, 4.0]), np.array([3.0, 3.0]), np.array([4.0, 6.0])]
    assert grow(h).tolist() == [True, False]  # per molecule


@pytest.mark.gpu
def test_guess_fallback_restart_reaches_core_energy(monkeypatch):
    """Restart machinery of the fallback: molecule 0 is made to revert at its fourth
    DIIS step (F = Core, P_old = 0, its older DIIS entries get zero weight) while
    molecule 1 keeps its learned guess; both reach the core-guess energies."""
    import mmd.batch as batch
    from mmd import guess as G
    from mmd.clusters import water_cluster
    from mmd.molecule import Molecule
    geoms = [water_cluster(3, seed=11 + k) for k in range(2)]
    Ec = batch.BatchRHF(geoms, "6-31g").run(conver=1e-10, polish=True)
    net = G.DensityMLP.load()
    gs = [G.predict_density(net, Molecule(g, "6-31g")) for g in geoms]
    calls = []

    def forced(history, times=3):
        calls.append(1)
        return np.array([len(calls) == 4, False])

    monkeypatch.setattr(batch, "diis_error_growing", forced)
    br = batch.BatchRHF(geoms, "6-31g")
    E = br.run(conver=1e-10, guess=gs, polish=True)
    assert br.reverted.tolist() == [True, False]
    assert br.converged.all()
    assert np.abs(E - Ec).max() < 1e-9


@pytest.mark.gpu
def test_embedded_guess_for_631gss_converges_faster_to_the_same_energy():
    """The 6-31G network's prediction embedded in 6-31G** (polarisation functions
    zero) is a valid density there, cuts the direct SCF iterations of a held-out
    (H2O)8, and the polished energies agree with the core-guess run."""
    from mmd import guess as G
    from mmd.clusters import water_cluster
    from mmd.molecule import Molecule
    net = G.DensityMLP.load()
    geom = water_cluster(8, seed=900123)
    m = Molecule(geom, "6-31gss")
    P0 = G.predict_density(net, m)
    assert P0.shape == (m.nbasis, m.nbasis)
    core = Molecule(geom, "6-31gss")
    Ec = core.RHF(doPrint=False, direct=True, conver=1e-9, polish=True)
    learned = Molecule(geom, "6-31gss")
    El = learned.RHF(doPrint=False, direct=True, conver=1e-9, guess=P0, polish=True)
    assert abs(np.trace(P0 @ learned.S) - learned.nocc) < 0.05 * learned.nocc
    assert not learned.guess_reverted
    assert learned.iterations < core.iterations
    assert abs(El - Ec) < 1e-9


def test_embedding_places_631g_blocks_on_the_shared_functions():
    from mmd import guess as G
    from mmd.clusters import water_cluster
    from mmd.molecule import Molecule
    geom = water_cluster(2, seed=3)
    small, big = Molecule(geom, "6-31g"), Molecule(geom, "6-31gss")
    rng = np.random.default_rng(0)
    A = rng.standard_normal((small.nbasis, small.nbasis))
    Ps = A + A.T
    P = G.embed_density(small, big, Ps)
    keep = [k for k, b in enumerate(big.bfs) if sum(int(x) for x in b.shell) <= 1 and
            not (big.atoms[big.bf_atom[k]].charge == 1 and sum(int(x) for x in b.shell) == 1)]
    assert len(keep) == small.nbasis
    assert np.array_equal(P[np.ix_(keep, keep)], Ps)
    rest = np.setdiff1d(np.arange(big.nbasis), keep)
    assert not P[rest].any() and not P[:, rest].any()
    with pytest.raises(ValueError):
        G.embed_density(small, Molecule(geom, "sto-3g"), Ps)


def test_631gss_targets_are_rotation_invariant_with_d_functions():
    """6-31G** layout (d sextet on O, p on H): a rotated molecule with the rotated
    density (P_new = T(R^T)^T P T(R^T) per atom block) gives the same local-frame
    targets, and assemble() inverts pair_targets()."""
    from mmd import guess as G
    from mmd.clusters import random_rotation
    gb = G.B631GSS
    m = _water_mol(2, seed=5)
    from mmd.molecule import Molecule
    m = Molecule(m.geometry_input, "6-31gss")
    R = random_rotation(np.random.default_rng(3))
    rng = np.random.default_rng(4)
    A = rng.standard_normal((m.nbasis, m.nbasis))
    P = A + A.T
    Z, X, off = G.molecule_layout(m, gb)
    T = np.zeros((m.nbasis, m.nbasis))
    for a, z in enumerate(Z):
        n = gb.nfunc[int(z)]
        T[off[a]:off[a] + n, off[a]:off[a] + n] = G.block_transform(int(z), R.T, gb)
    Prot = T.T @ P @ T
    rot = Molecule(_rotated(m, R).geometry_input, "6-31gss")
    pairs, _, Y1, _, (Zs, Rs, offs) = G.molecule_samples(m, P, gb)
    _, _, Y2, _, _ = G.molecule_samples(rot, Prot, gb)
    assert np.abs(Y1 - Y2).max() < 1e-4 * np.abs(Y1).max()
    Pa = G.assemble(Y1, Zs, Rs, offs, pairs, m.nbasis, gb)
    assert np.abs(Pa - P).max() < 1e-4 * np.abs(P).max()


@pytest.mark.gpu
def test_631gss_network_gains_over_core_guess():
    """The committed 6-31G** network (mmd.guess_train --basis 6-31gss, 8000 clusters)
    is the one network_for() picks for a 6-31G** molecule; on held-out (H2O)8 it cuts
    the batched SCF iterations and the polished energies match the core-guess ones."""
    from mmd import guess as G
    from mmd.batch import BatchRHF
    from mmd.clusters import water_cluster
    from mmd.molecule import Molecule
    geoms = [water_cluster(8, seed=900000 + k) for k in range(4)]
    net = G.network_for(Molecule(geoms[0], "6-31gss"))
    assert net.gb is G.B631GSS
    gs = [G.predict_density(net, Molecule(g, "6-31gss")) for g in geoms]
    core = BatchRHF(geoms, "6-31gss")
    core.run(conver=1e-8)
    learned = BatchRHF(geoms, "6-31gss")
    learned.run(conver=1e-8, guess=gs)
    assert learned.converged.all() and not learned.reverted.any()
    assert learned.iterations.mean() < 0.8 * core.iterations.mean()
    Ec = core.run(conver=1e-10, polish=True)
    El = learned.run(conver=1e-10, guess=gs, polish=True)
    assert np.abs(El - Ec).max() < 1e-9
