"""Sharded direct Fock build: one GPU per rank, one all-reduce of G per build.

The reference builds G(P - P_old) in one loop over the canonical bra pairs ij
(cython/fock.pyx:38-44) and everything inside it; that loop is the unit that
shards.  Here the unit is the shell pair: every shell quartet {P, Q} belongs to
the owner of its pair with the larger canonical index (s1(s1+1)/2 + s2, s1 >= s2,
molecule-local shells), each rank digests only the quartets it owns into a partial
G on its own GPU (``mmdg_set_partition`` filters the screening lists), and one
all-reduce(sum) of the N x N partial G gives every rank the full G.  DIIS, the
eigensolve and the energy stay replicated, so the ranks stay in lockstep.

The partition itself (``partition_shell_pairs``) is host logic, shared by the GPU
path and the tests, which also run it on CPU ranks with the oracle's formPT.
"""
from __future__ import annotations

import heapq

import numpy as np


def _sets(shells):
    return list(shells) if isinstance(shells, (list, tuple)) else [shells]


def canonical_pairs(shells):
    """(s1, s2) global shell indices of every shell pair in canonical order: per
    molecule, s1 ascending, then s2 from the molecule's first shell to s1."""
    out = []
    base = 0
    for ss in _sets(shells):
        for s1 in range(ss.nshell):
            for s2 in range(s1 + 1):
                out.append((base + s1, base + s2))
        base += ss.nshell
    return np.array(out, dtype=np.int64).reshape(-1, 2)


def _ncart(l):
    return (l + 1) * (l + 2) // 2


def pair_weights(shells):
    """Work proxy of every canonical shell pair: primitive pairs x Cartesian function
    pairs (a shell quartet costs about the product of its two pairs' weights)."""
    w = []
    for ss in _sets(shells):
        K, L = ss.nprim.astype(np.float64), ss.L
        for s1 in range(ss.nshell):
            for s2 in range(s1 + 1):
                w.append(K[s1] * K[s2] * _ncart(int(L[s1])) * _ncart(int(L[s2])))
    return np.array(w, dtype=np.float64)


def partition_shell_pairs(shells, world: int) -> np.ndarray:
    """Owner rank (0..world-1) of every canonical shell pair (order of
    ``canonical_pairs``).  Pair k owns the shell quartets it forms with the pairs
    k' <= k of its molecule; its load is w_k * sum_{k' <= k} w_k'.  Longest load first
    onto the least-loaded rank (LPT)."""
    world = int(world)
    if world < 1:
        raise ValueError("world must be >= 1")
    w = pair_weights(shells)
    load = np.empty_like(w)
    k = 0
    for ss in _sets(shells):
        n = ss.nshell * (ss.nshell + 1) // 2
        load[k:k + n] = w[k:k + n] * np.cumsum(w[k:k + n])
        k += n
    owner = np.zeros(len(w), dtype=np.int32)
    if world == 1:
        return owner
    heap = [(0.0, r) for r in range(world)]
    for idx in np.argsort(-load, kind="stable"):
        tot, r = heapq.heappop(heap)
        owner[idx] = r
        heapq.heappush(heap, (tot + load[idx], r))
    return owner


def quartet_owner(owner: np.ndarray, canon1, canon2):
    """Owner of the shell quartet of two pairs given by canonical index (one molecule)."""
    return owner[np.maximum(canon1, canon2)]


def function_shells(shells) -> np.ndarray:
    """Shell index of every basis function of a single molecule's ShellSet."""
    ss = _sets(shells)[0]
    fs = np.full(ss.nfunc, -1, dtype=np.int64)
    for s, row in enumerate(ss.func):
        for f in row:
            if f >= 0:
                fs[f] = s
    return fs


class ShardedFock:
    """The Fock build of one rank: partial G of the owned shell quartets on this rank's
    GPU, then ``all_reduce(sum)`` over ``group`` (NCCL for CUDA tensors), so every
    rank returns the full unsymmetrised G."""

    def __init__(self, ctx, group=None):
        import torch.distributed as dist
        self.ctx = ctx
        self.group = group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)
        self.owner = partition_shell_pairs(ctx.sets, self.world)
        ctx.set_partition(self.rank, self.world, self.owner)

    def fock(self, dP, G=None, tol: float = 1e-12, fp32_below: float = 0.0):
        import torch.distributed as dist
        G = self.ctx.fock(dP, G, tol=tol, fp32_below=fp32_below)
        if self.world > 1:
            dist.all_reduce(G, op=dist.ReduceOp.SUM, group=self.group)
        return G

    def close(self):
        """Back to unsharded builds on this context."""
        self.ctx.set_partition(0, 1, None)
