"""The oracle pinned against the reference's golden vectors (CPU only).

* Boys function: the 48 literature values of the reference's tests/test012.py
  (its own places=12 check plus relative 1e-9; the literature values are only
  good to ~7e-10 relative) and an mpmath grid (relative 5e-15);
* contracted ERIs of every angular class, the full water/STO-3G tensor and the
  Schwarz tables: the compiled reference, run to make the fixtures;
* formPT: the reference's own recorded calls (inputs and unsymmetrised output);
* the excited-state chain (RHF, spin-orbital integrals, CIS, TDHF): the reference's
  own excitation energies.
"""
import json
import os

import numpy as np
import pytest

import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_boys_literature_values():
    with open(os.path.join(GOLDEN, "boys_test012.json")) as f:
        vals = json.load(f)["values"]
    assert len(vals) == 48  # every assertAlmostEqual(boys(...)) of tests/test012.py
    for m, T, ref in vals:
        got = O.boys(m, T)
        # the reference's own check: assertAlmostEqual(places=12), i.e. |diff| < 5e-13
        assert round(got - ref, 12) == 0, (m, T, got, ref)
        # relative: the literature values themselves carry up to 7e-10 relative error
        # (e.g. F_25(6.4); the oracle agrees with mpmath there to 1e-15)
        assert abs(got - ref) <= 1e-9 * abs(ref), (m, T, got, ref)


def test_boys_mpmath_grid(golden):
    g = golden("boys_grid.npz")
    for im, m in enumerate(g["m"]):
        for iT, T in enumerate(g["T"]):
            ex = g["mpmath"][im, iT]
            assert abs(O.boys(m, T) - ex) <= 5e-15 * abs(ex), (m, T)


def test_boys_reference_agrees_with_mpmath(golden):
    # the reference's own values (SciPy 1.18 hyp1f1) deviate from mpmath by up to
    # 1e-13 relative for m <= 8 (the orders of (dd|dd)) and 3e-12 for m <= 16
    g = golden("boys_grid.npz")
    rel = np.abs(g["reference"] - g["mpmath"]) / np.abs(g["mpmath"])
    assert rel[:9].max() < 2e-13
    assert rel.max() < 5e-12


def _functions(g):
    bfs = []
    for o, s, k, e, c in zip(g["origin"], g["shell"], g["nprim"], g["exps"], g["coefs"]):
        bfs.append(O.Basis(o, s, int(k), e[:k], c[:k]))
    return bfs


def test_eri_every_class(golden):
    g = golden("eri_functions.npz")
    bfs = _functions(g)
    q, ref = g["quartets"], g["eri"]
    # a deterministic subset keeps the CPU suite fast (all 81 orderings covered)
    sel = np.arange(0, len(q), 3)
    got = np.array([O.ERI(*(bfs[i] for i in q[k])) for k in sel])
    assert np.max(np.abs(got - ref[sel])) < 1e-13


@pytest.mark.parametrize("name", ["h2_sto3g", "water_sto3g", "methane_sto3g"])
def test_eri_tensor_small(golden, name):
    d = golden(f"mol_{name}.npz")
    N = int(d["nbasis"])
    T = O.doERIs(N, np.zeros((N, N, N, N)), _raw_bfs(d))
    assert np.max(np.abs(T - d["TwoE"])) < 1e-13


def _raw_bfs(d):
    """Oracle Basis objects from the molecule's basis file (raw contraction coefficients)."""
    from mmd.molecule import Molecule
    m = Molecule(str(d["geometry"]), str(d["basis"]))
    out = []
    for atom in m.atoms:
        for momentum, prims in m.basis_data[atom.charge]:
            exps = [e for e, c in prims]
            coefs = [c for e, c in prims]
            for shell in m.momentum2shell(momentum):
                out.append(O.Basis(atom.origin, shell, len(exps), exps, coefs))
    return out


@pytest.mark.parametrize("name", ["water_sto3g", "methane_sto3g", "water_631g", "helium_ccpvtz"])
def test_screen_table(golden, name):
    d = golden(f"mol_{name}.npz")
    scr = O.screen_table(_raw_bfs(d))
    assert np.max(np.abs(scr - d["screen"])) < 1e-13


@pytest.mark.parametrize("name", ["h2_sto3g", "water_sto3g", "methane_sto3g", "water_631g"])
def test_formPT_records(golden, name):
    d = golden(f"mol_{name}.npz")
    bfs = _raw_bfs(d)
    N = int(d["nbasis"])
    k = 0
    while f"formPT{k}_G" in d:
        assert np.all(d[f"formPT{k}_imag"] == 0.0)
        G = O.formPT(d[f"formPT{k}_P"], d[f"formPT{k}_Pold"], bfs, N, d["screen"], 1e-12)
        assert np.max(np.abs(G.real - d[f"formPT{k}_G"])) < 1e-13
        k += 1
    assert k >= 1


def test_excited_state_oracle_matches_reference():
    """The CPU restatement of the reference's RHF -> CIS / TDHF chain (oracle/
    postscf_oracle.py), started from the golden integrals of water 3-21G and STO-3G,
    reproduces the reference's own excitation energies (tests/golden/excited.json)."""
    import postscf_oracle as X
    with open(os.path.join(GOLDEN, "excited.json")) as f:
        gold = json.load(f)
    for case, key in ((("cis",), "mol_water_321g.npz"), (("tdhf",), "mol_water_sto3g.npz")):
        d = np.load(os.path.join(GOLDEN, key))
        C, e = X.rhf(d["S"], d["T"], d["V"], d["TwoE"], int(d["nocc"]))
        A, B = X.singles(e, X.spin_integrals(C, d["TwoE"]), 2 * int(d["nocc"]))
        if case[0] == "cis":
            assert np.abs(X.cis(A) - np.asarray(gold["cis"]["omega"])).max() < 1e-9   # eV
        else:
            for alg in ("hermitian", "reduced", "full"):
                assert np.abs(X.tdhf(A, B, alg) - np.asarray(gold["tdhf"][alg])).max() < 1e-9


def test_mp2_oracle_matches_reference():
    """MP2 (spatial and spin-orbital) of the CPU restatement from the golden integrals
    equals the reference's own MP2 energies (tests/golden/mp2.json) for water STO-3G
    and 6-31G."""
    import postscf_oracle as X
    with open(os.path.join(GOLDEN, "mp2.json")) as f:
        cases = {(c["name"], c["basis"]): c for c in json.load(f)["cases"]}
    for key, fixture in ((("water", "sto-3g"), "mol_water_sto3g.npz"), (("water", "6-31g"), "mol_water_631g.npz")):
        d, c = np.load(os.path.join(GOLDEN, fixture)), cases[key]
        nocc = int(d["nocc"])
        C, e = X.rhf(d["S"], d["T"], d["V"], d["TwoE"], nocc)
        assert abs(X.mp2_spatial(C, e, d["TwoE"], nocc) + c["energy"] - c["emp2_spatial"]) < 1e-10
        dbl = X.spin_integrals(C, d["TwoE"])
        assert abs(X.mp2_spin(e, dbl, 2 * nocc) + c["energy"] - c["emp2_spin"]) < 1e-10


# ------------------------------------------------------------------ partial / fast oracle forms
def _shell_lists(bfs_mol):
    """Function-index lists of the shells of a Molecule's basis (the product's grouping)."""
    from mmd.integrals.shells import shells_from_bfs
    ss = shells_from_bfs(bfs_mol)
    return [[int(f) for f in row if f >= 0] for row in ss.func], ss


def test_memoised_shell_eri_equals_per_function_eri_bitwise(golden):
    """oracle eri_shell (memoised E and R, whole shells) gives exactly ERI() of every
    component quartet: the same recursions and summation order, evaluated once."""
    from mmd.molecule import Molecule
    d = golden("mol_water_631gss.npz")
    bfs = _raw_bfs(d)
    shells, _ = _shell_lists(Molecule(str(d["geometry"]), "6-31gss").bfs)
    rng = np.random.default_rng(3)
    picks = [tuple(int(x) for x in rng.integers(0, len(shells), 4)) for _ in range(24)]
    picks += [(5, 5, 5, 5), (5, 4, 5, 2)]  # the d shell of O: (dd|dd) and (dp|ds)
    for q in picks:
        fl = [shells[s] for s in q]
        v = O.eri_shell(bfs, *fl)
        for x, i in enumerate(fl[0]):
            for y, j in enumerate(fl[1]):
                for z, k in enumerate(fl[2]):
                    for w, l in enumerate(fl[3]):
                        assert v[x, y, z, w] == O.ERI(bfs[i], bfs[j], bfs[k], bfs[l]), (q, x, y, z, w)


def test_ranged_unique_eris_equal_doERIs(golden):
    d = golden("mol_water_sto3g.npz")
    bfs = _raw_bfs(d)
    N = len(bfs)
    T = O.doERIs(N, np.zeros((N, N, N, N)), bfs)
    i, j, k, l = O.unique_index(N)
    npair = N * (N + 1) // 2
    parts = [O.eri_unique(bfs, a, b) for a, b in ((0, 9), (9, 20), (20, npair))]
    assert np.array_equal(np.concatenate(parts), T[i, j, k, l])
    assert np.max(np.abs(T[i, j, k, l] - d["TwoE"][i, j, k, l])) < 1e-13
    # formPT from the table of those ERIs equals formPT recomputing them, bit for bit
    k0 = 0
    while f"formPT{k0}_G" in d:
        P, Po = d[f"formPT{k0}_P"], d[f"formPT{k0}_Pold"]
        Gt = O.formPT_table(P, Po, T[i, j, k, l], N, d["screen"], 1e-12)
        assert np.array_equal(Gt, O.formPT(P, Po, bfs, N, d["screen"], 1e-12).real)
        k0 += 1


def test_shell_blocked_unique_eris_equal_the_per_function_ones(golden):
    """parallel_eri_unique_shells (every shell quartet once, components scattered to
    their canonical positions) against the per-function unique ERIs of doERIs order:
    water/6-31G** with its d shell, equal to 1e-15 (blocks that hold a canonical
    quartet in another function order differ in the last bits only); a shell list
    missing a function is refused."""
    from mmd.integrals.shells import shells_from_bfs
    from mmd.molecule import Molecule
    d = golden("mol_water_631gss.npz")
    bfs = _raw_bfs(d)
    shells = [[int(f) for f in row if f >= 0] for row in
              shells_from_bfs(Molecule(str(d["geometry"]), str(d["basis"])).bfs).func]
    ref = O.parallel_eri_unique(bfs, nproc=2)
    got = O.parallel_eri_unique_shells(bfs, shells, nproc=2)
    assert got.shape == ref.shape
    assert np.max(np.abs(got - ref)) < 1e-15
    with pytest.raises(ValueError):
        O.parallel_eri_unique_shells(bfs, shells[:-1], nproc=2)


def test_partial_formPT_adds_up_to_formPT(golden):
    """formPT restricted to ij ranges, or to the shell quartets of each part of a
    shell-pair partition, adds up to the full formPT (the reference's records)."""
    from mmd.distributed import function_shells, partition_shell_pairs
    from mmd.molecule import Molecule
    d = golden("mol_water_631g.npz")
    bfs = _raw_bfs(d)
    N = int(d["nbasis"])
    P, Po = d["formPT0_P"], d["formPT0_Pold"]
    ref = d["formPT0_G"]
    npair = N * (N + 1) // 2
    G = sum(O.formPT_part(P, Po, bfs, N, d["screen"], 1e-12, a, b) for a, b in ((0, 30), (30, 61), (61, npair)))
    assert np.max(np.abs(G - ref)) < 1e-13
    _, ss = _shell_lists(Molecule(str(d["geometry"]), "6-31g").bfs)
    fs = function_shells(ss)
    for world in (2, 3):
        owner = partition_shell_pairs(ss, world)
        parts = [O.formPT_part(P, Po, bfs, N, d["screen"], 1e-12, func_shell=fs, owner=owner, part=r)
                 for r in range(world)]
        assert all(np.abs(p).max() > 0 for p in parts)
        assert np.max(np.abs(sum(parts) - ref)) < 1e-13


def test_oracle_formPT_matches_the_reference_call_on_h2o2():
    """The oracle's formPT against the reference's own first formPT call of its direct
    RHF on (H2O)2 / 6-31G** (813,450 candidate quartets; fixture made by
    tests/golden/make_golden_h2o2_formpt.py), run over ij ranges in processes."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                    "mcmurchie-davidson_gb300"))
    from mmd.molecule import Molecule
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "h2o2_631gss_formpt.npz"))
    mol = Molecule(str(g["geometry"]), "6-31gss")
    bfs = []
    for atom in mol.atoms:
        for momentum, prims in mol.basis_data[atom.charge]:
            ex = [e for e, c in prims]
            co = [c for e, c in prims]
            for shell in mol.momentum2shell(momentum):
                bfs.append(O.Basis(atom.origin, shell, len(ex), ex, co))
    N = len(bfs)
    assert np.abs(O.screen_table(bfs) - g["screen"]).max() < 1e-13
    G = O.parallel_formPT(g["P"], np.zeros((N, N)), bfs, N, g["screen"], float(g["tol"]))
    assert np.abs(G - g["G"]).max() < 1e-12
