"""Batched launch (many molecules in one context / one graph), the CUDA-graph replay
and the autotuner, against the single-molecule path."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _geoms():
    from mmd.clusters import water_cluster
    return [water_cluster(n, seed=100 + k) for k, n in enumerate((1, 2, 3, 2, 1, 3))]


def test_batched_fock_equals_single_molecule_builds():
    import torch
    from mmd import _native
    from mmd.integrals.shells import shells_from_bfs
    from mmd.molecule import Molecule
    mols = [Molecule(g, "6-31g") for g in _geoms()]
    sets = [shells_from_bfs(m.bfs) for m in mols]
    batch = _native.Context(sets)
    rng = np.random.default_rng(4)
    dens = []
    for m in mols:
        A = rng.standard_normal((m.nbasis, m.nbasis)) * 0.3
        dens.append(A + A.T)
    dP = torch.tensor(np.concatenate([d.ravel() for d in dens]), device="cuda")
    G = batch.fock(dP, tol=1e-12).cpu().numpy()
    off = 0
    for s, d in zip(sets, dens):
        n = s.nfunc
        g1 = _native.Context(s).fock(torch.tensor(d.ravel(), device="cuda"), tol=1e-12).cpu().numpy()
        assert np.abs(G[off:off + n * n] - g1).max() < 1e-12
        off += n * n


def test_fock_graph_replay_and_tuning():
    import ctypes
    import torch
    from mmd import _native, autotune
    from mmd.integrals.shells import shells_from_bfs
    from mmd.molecule import Molecule
    sets = [shells_from_bfs(Molecule(g, "6-31g").bfs) for g in _geoms()]
    ctx = _native.Context(sets)
    rng = np.random.default_rng(5)
    dP = torch.tensor(rng.standard_normal(ctx.nn), device="cuda")
    ref = ctx.fock(dP, tol=1e-12).clone()
    tun = autotune.autotune(ctx, dP, tol=1e-12, reps=1, use_cache=False)
    assert tun.streams in (1, 2, 4, 8)
    assert torch.max(torch.abs(ctx.fock(dP, tol=1e-12) - ref)).item() < 1e-12
    G = torch.empty_like(dP)
    for k in range(3):  # capture, then replays with new contents of the same buffers
        dP.copy_(torch.tensor(rng.standard_normal(ctx.nn), device="cuda"))
        _native.check(_native.lib().mmdg_fock_graph(ctx._h, ctypes.c_void_p(dP.data_ptr()),
                                                     ctypes.c_void_p(G.data_ptr()), 1e-12, 0.0,
                                                     _native.stream_ptr()), "mmdg_fock_graph")
        eager = ctx.fock(dP, tol=1e-12)
        torch.cuda.synchronize()
        assert torch.max(torch.abs(G - eager)).item() < 1e-12


def test_batched_rhf_energies_match_single_molecule_rhf():
    from mmd.batch import BatchRHF
    from mmd.molecule import Molecule
    geoms = _geoms()
    br = BatchRHF(geoms, "6-31g")
    E = br.run(conver=1e-10)
    assert br.converged.all()
    for g, e in zip(geoms, E):
        m = Molecule(g, "6-31g")
        e1 = m.RHF(doPrint=False, direct=True, conver=1e-10)
        assert abs(e - e1) < 1e-10, (e, e1)


def test_every_tile_gives_the_same_fock_build():
    """mmdg_set_tile: 64/128/256 threads per block for the one-thread-per-quartet
    kernels and 1..8 quartets per warp work item for the high-L kernels change the
    schedule, not the result (water 6-31G**: every class present)."""
    import torch
    from mmd import _native, autotune
    from mmd.flop_model import CLASSES, fock_kernel
    from mmd.molecule import Molecule
    mol = Molecule("\n0 1\nO 0.0 -0.075791844 0.0\nH 0.866811829 0.601435779 0.0\nH -0.866811829 0.601435779 0.0\n",
                   "6-31gss")
    ctx = mol.context
    rng = np.random.default_rng(8)
    A = rng.standard_normal((mol.nbasis, mol.nbasis))
    dP = torch.tensor((A + A.T).ravel(), device="cuda")
    ref = ctx.fock(dP, tol=1e-12).clone()
    warp = [fock_kernel(c) == "warp" for c in CLASSES]
    try:
        for k in range(4):
            tiles = [autotune.ITEMS[k] if w else (autotune.BLOCKS[k] if k < 3 else 0) for w in warp]
            autotune.Tuning(tiles=tiles, streams=1).apply(ctx)
            assert torch.max(torch.abs(ctx.fock(dP, tol=1e-12) - ref)).item() < 1e-12, tiles
    finally:
        autotune.Tuning(streams=_native.DEFAULT_STREAMS_SINGLE).apply(ctx)
    with pytest.raises(_native.MMDGError):
        _native.check(_native.lib().mmdg_set_tile(ctx._h, 0, 96, 0), "mmdg_set_tile")
