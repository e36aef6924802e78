"""The sharded Fock build's partition (mmd.distributed), on the CPU.

The reference builds G in one loop over canonical bra pairs ij (cython/fock.pyx:38-44);
the sharded build gives every shell quartet to the owner of its shell pair with the
larger canonical index.  Checked here: every shell quartet has exactly one owner,
the ranks' loads are balanced, and two gloo ranks on 127.0.0.1, each computing its
partial G with the oracle's formPT restricted to its quartets, reproduce the full
formPT after one all-reduce(sum) -- the exchange step of the multi-GPU build.
"""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
WATER = "\n0 1\nO 0.000000 -0.075791844 0.000000\nH 0.866811829 0.601435779 0.000000\nH -0.866811829 0.601435779 0.000000\n"


def _shells(geom, basis):
    from mmd.integrals.shells import shells_from_bfs
    from mmd.molecule import Molecule
    return shells_from_bfs(Molecule(geom, basis).bfs)


def test_every_shell_quartet_has_one_owner_and_loads_balance():
    from mmd.clusters import water_cluster
    from mmd.distributed import canonical_pairs, pair_weights, partition_shell_pairs, quartet_owner
    ss = _shells(water_cluster(2, seed=16), "6-31gss")
    pairs = canonical_pairs(ss)
    n = len(pairs)
    assert n == ss.nshell * (ss.nshell + 1) // 2
    assert np.array_equal(pairs[:, 0] * (pairs[:, 0] + 1) // 2 + pairs[:, 1], np.arange(n))
    w = pair_weights(ss)
    for world in (1, 2, 3, 8):
        owner = partition_shell_pairs(ss, world)
        assert owner.min() >= 0 and owner.max() < world
        c1, c2 = np.tril_indices(n)  # every unordered pair of shell pairs once
        own = quartet_owner(owner, c1, c2)
        counts = np.bincount(own, minlength=world)
        assert counts.sum() == n * (n + 1) // 2
        load = np.bincount(own, weights=w[c1] * w[c2], minlength=world)
        assert load.max() <= 1.05 * load.mean() + 1e-9, (world, load)


def test_batched_partition_keeps_molecules_apart():
    from mmd.distributed import canonical_pairs, partition_shell_pairs
    sets = [_shells(WATER, "6-31g"), _shells(WATER, "sto-3g")]
    pairs = canonical_pairs(sets)
    n0 = sets[0].nshell * (sets[0].nshell + 1) // 2
    assert len(pairs) == n0 + sets[1].nshell * (sets[1].nshell + 1) // 2
    assert pairs[n0:].min() >= sets[0].nshell  # second molecule: its own shells only
    assert len(partition_shell_pairs(sets, 2)) == len(pairs)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    for p in (ROOT, os.path.join(ROOT, "mcmurchie-davidson_gb300"), os.path.join(ROOT, "oracle")):
        sys.path.insert(0, p)
    import torch
    import torch.distributed as dist
    import oracle as O
    from mmd.distributed import function_shells, partition_shell_pairs
    from mmd.integrals.shells import shells_from_bfs
    from mmd.molecule import Molecule
    dist.init_process_group("gloo", rank=rank, world_size=world)
    d = np.load(os.path.join(ROOT, "tests", "golden", "mol_water_631gss.npz"))
    mol = Molecule(str(d["geometry"]), "6-31gss")
    ss = shells_from_bfs(mol.bfs)
    owner = partition_shell_pairs(ss, world)  # the product's partition, the same on every rank
    bfs = []
    for atom in mol.atoms:
        for momentum, prims in mol.basis_data[atom.charge]:
            ex = [e for e, c in prims]
            co = [c for e, c in prims]
            for shell in mol.momentum2shell(momentum):
                bfs.append(O.Basis(atom.origin, shell, len(ex), ex, co))
    N = len(bfs)
    P, Po = d["formPT0_P"], d["formPT0_Pold"]
    part = O.formPT_part(P, Po, bfs, N, d["screen"], 1e-12, func_shell=function_shells(ss), owner=owner, part=rank)
    G = torch.tensor(part)
    dist.all_reduce(G, op=dist.ReduceOp.SUM)  # the one exchange step per Fock build
    full = O.formPT(P, Po, bfs, N, d["screen"], 1e-12).real if rank == 0 else None
    q.put((rank, float(np.abs(part).max()), G.numpy(), full, d["formPT0_G"]))
    dist.destroy_process_group()


def test_two_gloo_ranks_partial_fock_all_reduce_equals_formPT():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted((q.get(timeout=300) for _ in procs), key=lambda t: t[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    full = out[0][3]
    for rank, pmax, G, _, ref in out:
        assert pmax > 0.0  # every rank did part of the work
        assert np.max(np.abs(G - full)) < 1e-12  # all-reduced partial G == full formPT
        assert np.max(np.abs(G - ref)) < 1e-12   # == the reference's own recorded call
