#!/usr/bin/env python3
"""Reference energies of held-out seeded (H2O)8 / 6-31G clusters, from the reference.

The combined form (learned guess + FP32 below a Schwarz threshold + FP64 polish) and
the batched SCF are checked against these: the reference's own conventional RHF
(mmd/scf.py:10-80 with the ERI tensor of its compiled Cython doERIs,
cython/twoe.pyx:12-31) converged to conver = 1e-12, on the clusters
``water_cluster(8, seed=900000 + k)`` for k = 0..7 -- the first eight of the 64
held-out molecules of bench.py's combined-form benchmark (never in the guess
network's training data).  One molecule per process (each ~10 minutes of the
reference's Cython).

Runs only here, with $MMD_REFERENCE naming the reference tree (make_golden.py's
shimmed, compiled copy of the reference); writes h2o8_631g_reference.json.
"""
from __future__ import annotations

import json
import multiprocessing as mp
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as MG  # noqa: E402

SEEDS = [900000 + k for k in range(8)]


def _one(seed):
    MG._prepare_reference()  # the copy exists already: only puts it on sys.path
    from mmd.molecule import Molecule
    clusters = MG._load_clusters()
    geom = clusters.water_cluster(8, seed=seed)
    t0 = time.time()
    mol = Molecule(geometry=geom, basis="6-31g")
    mol.RHF(doPrint=False, conver=1e-12)
    return {"seed": seed, "energy": float(mol.energy.real), "nbasis": int(mol.nbasis),
            "converged": bool(mol.is_converged), "seconds": time.time() - t0}


def main():
    MG._prepare_reference()  # lay out the shimmed, compiled reference once, before the workers
    with mp.get_context("spawn").Pool(len(SEEDS)) as pool:
        res = pool.map(_one, SEEDS)
    out = {"source": "the reference's conventional RHF (compiled Cython doERIs, mmd/scf.py RHF, conver 1e-12)",
           "workload": "water_cluster(8, seed) / 6-31G", "conver": 1e-12, "molecules": res}
    with open(os.path.join(HERE, "h2o8_631g_reference.json"), "w") as f:
        json.dump(out, f, indent=1)
    for r in res:
        print(r)


if __name__ == "__main__":
    main()
