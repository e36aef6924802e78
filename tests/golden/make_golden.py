#!/usr/bin/env python3
"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs only where the reference tree is present (its path in $MMD_REFERENCE, which
is required).  It lays out a shimmed, compiled copy of the reference package
with ``oracle/build_ref.py --full`` (the same three shims), imports it, and dumps
the reference's own outputs:

* ``boys_test012.json``  the 50 literature Boys values of the reference's
                          tests/test012.py:12-69, parsed from that file's text;
* ``boys_grid.npz``       reference ``_boys`` (SciPy hyp1f1) and mpmath values on a
                          grid of m = 0..16 and T in [0, 1e4];
* ``eri_functions.npz``   contracted ERIs ``twoe.ERI`` for random quartets of
                          s/p/d functions (the carbon 6-31G** shells of the
                          reference's tests/test013.py:14-24, all Cartesian
                          components, on three centres) -- every angular class
                          (ss|ss) .. (dd|dd);
* ``mol_<name>.npz``      per molecule: nbasis, S/T/V, nuclear repulsion, RHF
                          energies (conventional at conver 1e-8 and 1e-12; direct
                          where affordable), the ERI tensor (small cases) or a
                          sampled set of its entries, the Schwarz table and one
                          or two recorded ``formPT`` calls (inputs and output).

The fixtures are committed; this script is committed beside them so they can be
regenerated.  Nothing on the GPU machine runs it.
"""
from __future__ import annotations

import importlib.util
import json
import os
import re
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REFERENCE = os.environ.get("MMD_REFERENCE", "")
REFCOPY = os.environ.get("MMD_REFCOPY", "/tmp/mmd_golden_ref")


def _load_clusters():
    path = os.path.join(REPO, "mcmurchie-davidson_gb300", "mmd", "clusters.py")
    spec = importlib.util.spec_from_file_location("_clusters_for_golden", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _prepare_reference():
    if not REFERENCE or not os.path.isdir(os.path.join(REFERENCE, "cython")):
        raise SystemExit("set MMD_REFERENCE to the reference tree (the directory holding cython/ and mmd/)")
    if not os.path.isdir(os.path.join(REFCOPY, "mmd", "integrals")):
        subprocess.check_call([sys.executable, os.path.join(REPO, "oracle", "build_ref.py"),
                               "--reference", REFERENCE, "--full", REFCOPY])
    # the 6-31G file the reference lacks: same derivation as the package's copy
    src = os.path.join(REPO, "mcmurchie-davidson_gb300", "mmd", "basis", "6-31g.gbs")
    dst = os.path.join(REFCOPY, "mmd", "basis", "6-31g.gbs")
    with open(src) as f, open(dst, "w") as g:
        g.write(f.read())
    sys.path.insert(0, REFCOPY)


WATER = """
0 1
O    0.000000      -0.075791844    0.000000
H    0.866811829    0.601435779    0.000000
H   -0.866811829    0.601435779    0.000000
"""
H2 = """
0 1
H 0.0 0.0 0.74
H 0.0 0.0 0.00
"""
METHANE = """
0 1
C    0.000000    0.000000    0.000000
H    0.626425042   -0.626425042   -0.626425042
H    0.626425042    0.626425042    0.626425042
H   -0.626425042    0.626425042   -0.626425042
H   -0.626425042   -0.626425042    0.626425042
"""
HELIUM = """
0 1
He    0.000000    0.000000    0.000000
"""
FORMALDEHYDE = """
0 1
C          0.0000000000        0.0000000000       -0.5265526741
O          0.0000000000        0.0000000000        0.6555124750
H          0.0000000000       -0.9325664988       -1.1133424527
H          0.0000000000        0.9325664988       -1.1133424527
"""


def boys_fixtures():
    from mmd.integrals.onee import _boys
    import mpmath as mp
    text = open(os.path.join(REFERENCE, "tests", "test012.py")).read()
    vals = [(float(m), float(t), float(v)) for m, t, v in
            re.findall(r"boys\(\s*([0-9.Ee+-]+)\s*,\s*([0-9.Ee+-]+)\s*\)\s*,\s*([0-9.Ee+-]+)", text)]
    with open(os.path.join(HERE, "boys_test012.json"), "w") as f:
        json.dump({"source": "reference tests/test012.py:12-69", "values": vals}, f, indent=1)
    mp.mp.dps = 40
    ms = np.arange(0, 17)
    Ts = np.concatenate([[0.0, 1e-12, 1e-9, 1e-6, 1e-3], np.linspace(0.01, 60, 241), [75.0, 100.0, 200.0, 500.0, 1e3, 1e4]])
    ref = np.array([[_boys(int(m), float(T)) for T in Ts] for m in ms])
    exact = np.array([[float(mp.hyp1f1(m + mp.mpf(1) / 2, m + mp.mpf(3) / 2, -mp.mpf(float(T))) / (2 * m + 1))
                       for T in Ts] for m in ms])
    np.savez_compressed(os.path.join(HERE, "boys_grid.npz"), m=ms, T=Ts, reference=ref, mpmath=exact)
    print("boys: %d literature values, grid %s" % (len(vals), ref.shape))


def eri_fixtures():
    from mmd.integrals.twoe import Basis, ERI
    # carbon 6-31G** shells of the reference's tests/test013.py:14-24
    Se = [3047.5249000, 457.3695100, 103.9486900, 29.2101550, 9.2866630, 3.1639270]
    Sc = [0.0018347, 0.0140373, 0.0688426, 0.2321844, 0.4679413, 0.3623120]
    Pe = [7.8682724, 1.8812885, 0.5442493]
    Pc = [0.0689991, 0.3164240, 0.7443083]
    De, Dc = [0.8000000], [1.0000000]
    centres = [[0.0, 0.0, 0.0], [2.0, 0.0, 0.0], [0.31, -1.17, 0.74]]
    comps = {0: [(0, 0, 0)], 1: [(1, 0, 0), (0, 1, 0), (0, 0, 1)],
             2: [(2, 0, 0), (1, 1, 0), (1, 0, 1), (0, 2, 0), (0, 1, 1), (0, 0, 2)]}
    shells = [(0, Se, Sc), (1, Pe, Pc), (2, De, Dc)]
    origin, shell, L, nprim, exps, coefs, bfs = [], [], [], [], [], [], []
    for c in centres:
        for l, e, co in shells:
            for lmn in comps[l]:
                b = Basis(np.array(c), np.array(lmn), len(e), np.array(e, float), np.array(co, float))
                bfs.append(b)
                origin.append(c)
                shell.append(lmn)
                L.append(l)
                nprim.append(len(e))
                exps.append(np.pad(np.array(e, float), (0, 6 - len(e))))
                coefs.append(np.pad(np.array(co, float), (0, 6 - len(e))))
    nf = len(bfs)
    rng = np.random.default_rng(2024)
    Larr = np.array(L)
    quartets = []
    # every class (la lb|lc ld), 60 random quartets each
    for la in range(3):
        for lb in range(3):
            for lc in range(3):
                for ld in range(3):
                    pools = [np.flatnonzero(Larr == x) for x in (la, lb, lc, ld)]
                    for _ in range(60):
                        quartets.append([rng.choice(p) for p in pools])
    quartets = np.array(quartets, dtype=np.int64)
    t0 = time.time()
    vals = np.array([ERI(bfs[i], bfs[j], bfs[k], bfs[l]) for i, j, k, l in quartets])
    np.savez_compressed(os.path.join(HERE, "eri_functions.npz"), origin=np.array(origin), shell=np.array(shell),
                        nprim=np.array(nprim), exps=np.array(exps), coefs=np.array(coefs),
                        quartets=quartets, eri=vals)
    print("eri: %d functions, %d quartets, %.1fs" % (nf, len(quartets), time.time() - t0))


def _record_formPT(mol, calls):
    import mmd.scf as scf_mod
    orig = scf_mod.formPT
    rec = []

    def wrapper(P, P_old, bfs, nbasis, screen, tol):
        G = orig(P, P_old, bfs, nbasis, screen, tol)
        if len(rec) < calls:
            rec.append((np.array(P).real.copy(), np.array(P_old).real.copy(), np.array(G).real.copy(),
                        float(np.abs(np.imag(P)).max()), float(np.abs(np.imag(P_old)).max())))
        return G
    scf_mod.formPT = wrapper
    try:
        mol.RHF(doPrint=False, direct=True)
    finally:
        scf_mod.formPT = orig
    return rec


def molecule_fixture(name, geometry, basis, *, tensor="full", direct=False, formpt_calls=0, sample=20000):
    from mmd.molecule import Molecule
    t0 = time.time()
    out = {"name": name, "geometry": geometry, "basis": basis}
    mol = Molecule(geometry=geometry, basis=basis)
    mol.RHF(doPrint=False)
    out.update(nbasis=mol.nbasis, nocc=mol.nocc, S=mol.S, T=mol.T, V=mol.V, nuc_energy=mol.nuc_energy,
               energy_conv=mol.energy.real, P_conv=np.array(mol.P).real)
    TwoE = np.asarray(mol.TwoE)
    N = mol.nbasis
    if tensor == "full":
        out["TwoE"] = TwoE
    else:
        rng = np.random.default_rng(7)
        idx = rng.integers(0, N, size=(sample, 4))
        out["TwoE_idx"] = idx
        out["TwoE_val"] = TwoE[idx[:, 0], idx[:, 1], idx[:, 2], idx[:, 3]]
    mol2 = Molecule(geometry=geometry, basis=basis)
    mol2.RHF(doPrint=False, conver=1e-12)
    out["energy_conv_1e12"] = mol2.energy.real
    if direct:
        mol3 = Molecule(geometry=geometry, basis=basis)
        rec = _record_formPT(mol3, formpt_calls)
        out["energy_direct"] = mol3.energy.real
        out["screen"] = np.array([mol3.screen[i] for i in range(N * (N + 1) // 2)])
        for c, (P, Po, G, ip, ipo) in enumerate(rec):
            out[f"formPT{c}_P"] = P
            out[f"formPT{c}_Pold"] = Po
            out[f"formPT{c}_G"] = G
            out[f"formPT{c}_imag"] = np.array([ip, ipo])
    np.savez_compressed(os.path.join(HERE, f"mol_{name}.npz"), **out)
    print("%s/%s N=%d E=%.12f (%.1fs)" % (name, basis, N, out["energy_conv"], time.time() - t0))


def main():
    _prepare_reference()
    clusters = _load_clusters()
    boys_fixtures()
    eri_fixtures()
    molecule_fixture("h2_sto3g", H2, "sto-3g", direct=True, formpt_calls=2)
    molecule_fixture("water_sto3g", WATER, "sto-3g", direct=True, formpt_calls=3)
    molecule_fixture("methane_sto3g", METHANE, "sto-3g", direct=True, formpt_calls=2)
    molecule_fixture("helium_ccpvtz", HELIUM, "cc-pvtz", direct=True, formpt_calls=1)
    molecule_fixture("formaldehyde_sto3g", FORMALDEHYDE, "sto-3g")
    molecule_fixture("water_dz", WATER, "dz")
    molecule_fixture("water_321g", WATER, "3-21g")
    molecule_fixture("water_631g", WATER, "6-31g", direct=True, formpt_calls=2)
    molecule_fixture("water_631gss", WATER, "6-31gss", tensor="sample", direct=True, formpt_calls=2)
    molecule_fixture("water_631ppgss", WATER, "6-31ppgss", tensor="sample")
    molecule_fixture("w2_631g", clusters.water_cluster(2, seed=11), "6-31g", tensor="sample")
    molecule_fixture("w3_631g", clusters.water_cluster(3, seed=12), "6-31g", tensor="sample")


if __name__ == "__main__":
    main()
