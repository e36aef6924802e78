#!/usr/bin/env python3
"""Inputs of one full-size reference formPT call on (H2O)2 / 6-31G**: the anchor of the
CPU baseline's extrapolation.

bench.py times the reference's compiled Cython formPT (cython/fock.pyx:13-87) on the
water monomer and extrapolates per-candidate and per-surviving-quartet costs to the
benchmark's (H2O)16.  This fixture lets the bench also time one whole formPT call of a
cluster -- the first call of the reference's own direct RHF (mmd/scf.py:10-80) on
``water_cluster(2, seed=16)``, the benchmark generator's (H2O)2 -- and compare it with
what the extrapolation predicts.  Stored: the geometry, the reference's Schwarz table
(Molecule.build(direct=True), mmd/molecule.py:90-102) and the density P of that call
(P_old = 0).

Runs only here, with $MMD_REFERENCE naming the reference tree (make_golden.py's
shimmed, compiled copy); writes h2o2_631gss_formpt.npz.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as MG  # noqa: E402


class _Stop(Exception):
    pass


def main():
    MG._prepare_reference()
    import mmd.scf as scf_mod
    from mmd.molecule import Molecule
    clusters = MG._load_clusters()
    geom = clusters.water_cluster(2, seed=16)
    mol = Molecule(geometry=geom, basis="6-31gss")
    orig = scf_mod.formPT
    rec = {}

    def first_call(P, P_old, bfs, nbasis, screen, tol):
        t0 = time.time()
        G = orig(P, P_old, bfs, nbasis, screen, tol)
        rec.update(P=np.array(P).real.copy(), P_old=np.array(P_old).real.copy(), G=np.array(G).real.copy(),
                   seconds=time.time() - t0, tol=tol)
        raise _Stop()

    scf_mod.formPT = first_call
    try:
        mol.RHF(doPrint=False, direct=True)
    except _Stop:
        pass
    finally:
        scf_mod.formPT = orig
    N = mol.nbasis
    screen = np.array([mol.screen[i] for i in range(N * (N + 1) // 2)])
    assert not np.any(rec["P_old"]), "the first formPT call of a direct RHF has P_old = 0"
    np.savez_compressed(os.path.join(HERE, "h2o2_631gss_formpt.npz"), geometry=geom, screen=screen, P=rec["P"],
                        G=rec["G"], seconds_here=rec["seconds"], tol=rec["tol"])
    print(f"(H2O)2/6-31G** N={N}: first formPT {rec['seconds']:.1f} s here")


if __name__ == "__main__":
    main()
