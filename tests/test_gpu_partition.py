"""The sharded Fock build on one GPU (mmdg_set_partition): each part of a shell-pair
partition digests only its shell quartets.  The parts are run one after another on
the same GPU (no kernel waits on another), and checked against the oracle's formPT
restricted to the same quartets and, summed, against the unsharded build -- what one
all-reduce of G per build gives the ranks of a multi-GPU run (cython/fock.pyx:38-44
is the loop that is split)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _case(name):
    from mmd.clusters import water_cluster
    from mmd.molecule import Molecule
    if name == "water_631gss":
        d = np.load(os.path.join(GOLDEN, "mol_water_631gss.npz"))
        return Molecule(str(d["geometry"]), "6-31gss")
    return Molecule(water_cluster(2, seed=16), "6-31g")


@pytest.mark.parametrize("name", ["water_631gss", "w2_631g"])
@pytest.mark.parametrize("world", [2, 3])
def test_partition_parts_match_oracle_parts_and_add_up(name, world):
    import torch
    import oracle as O
    from mmd.distributed import function_shells, partition_shell_pairs
    from mmd.integrals.shells import shells_from_bfs
    from test_gpu_benchsize import oracle_bfs
    mol = _case(name)
    ctx = mol.context
    N = mol.nbasis
    ss = shells_from_bfs(mol.bfs)
    owner = partition_shell_pairs(ss, world)
    rng = np.random.default_rng(world)
    A = rng.standard_normal((N, N)) * 0.2
    P = A + A.T
    dP = torch.tensor(P.ravel(), device="cuda")
    full = ctx.fock(dP, tol=1e-12).cpu().numpy()
    scr = ctx.screen()
    ob = oracle_bfs(mol)
    fs = function_shells(ss)
    total = np.zeros_like(full)
    try:
        for r in range(world):
            ctx.set_partition(r, world, owner)
            g = ctx.fock(dP, tol=1e-12).cpu().numpy()
            go = O.formPT_part(P, np.zeros_like(P), ob, N, scr, 1e-12, func_shell=fs, owner=owner, part=r)
            assert np.abs(g).max() > 0.0
            assert np.abs(g - go.ravel()).max() < 1e-12, (r, np.abs(g - go.ravel()).max())
            total += g
    finally:
        ctx.set_partition(0, 1)
    assert np.abs(total - full).max() < 1e-12
    # sharding off again: the full build (G accumulates by FP64 atomics, so repeated
    # builds agree to rounding, not bit for bit)
    assert np.abs(ctx.fock(dP, tol=1e-12).cpu().numpy() - full).max() < 1e-13


def test_sharded_fock_builds_a_direct_rhf_on_one_rank_group():
    """RHF(direct=True, process_group=g) on a one-rank gloo group runs unsharded and
    gives the plain energy; the partitioned context is left unsharded afterwards."""
    import socket
    import torch.distributed as dist
    from mmd.molecule import Molecule
    d = np.load(os.path.join(GOLDEN, "mol_water_631g.npz"))
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=0, world_size=1)
    try:
        E1 = Molecule(str(d["geometry"]), "6-31g").RHF(doPrint=False, direct=True, conver=1e-10,
                                                        process_group=dist.group.WORLD)
    finally:
        dist.destroy_process_group()
    E0 = Molecule(str(d["geometry"]), "6-31g").RHF(doPrint=False, direct=True, conver=1e-10)
    assert abs(E1 - E0) < 1e-12
