"""Parity at the benchmark's own sizes: the GPU path against the oracle on the
seeded water clusters of the workload (6-31G**, Cartesian d).

* (H2O)2 and (H2O)4: the full ERI tensor (doERIs, cython/twoe.pyx:12-31) -- every
  unique quartet -- and two full formPT builds (cython/fock.pyx:13-87: the
  core-guess density and an incremental density difference) against the oracle,
  to 1e-12 per element.  These clusters hold far intermolecular quartets, so the
  large-T branch of the Boys function and the primitive-pair screening are covered.
* (H2O)16, the benchmark molecule itself: a stratified sample of at least 2000
  shell quartets of every angular class, spread evenly over the distance between
  the bra and ket pair centres and including the most distant ones, each in a
  random shell order; every component ERI (mmdg_eri_quartets) against the oracle's
  ERI (twoe.pyx:36-50), absolute 1e-12 and relative 1e-9 where |ERI| > 1e-6.

The oracle runs in a pool of processes (spawned) over the host's cores, one shell
quartet at a time with E and R memoised (the per-function form took 24x longer).
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def oracle_bfs(mol):
    """Oracle Basis objects of a Molecule (raw contraction coefficients from its basis file)."""
    import oracle as O
    out = []
    for atom in mol.atoms:
        for momentum, prims in mol.basis_data[atom.charge]:
            ex = [e for e, c in prims]
            co = [c for e, c in prims]
            for shell in mol.momentum2shell(momentum):
                out.append(O.Basis(atom.origin, shell, len(ex), ex, co))
    return out


def stratified_quartets(ss, per_class=2000, seed=0, bins=20):
    """(n, 4) shell quartets (a, b, c, d): for every angular class (la lb|lc ld),
    la >= lb, lc >= ld, (la, lb) >= (lc, ld), ``per_class`` quartets drawn evenly
    from ``bins`` bins of the distance between the bra and ket pair midpoints, plus
    the 5 % most distant of a large candidate draw; each quartet's shell order is
    randomised (pair-internal and bra/ket swaps)."""
    rng = np.random.default_rng(seed)
    L, cen = ss.L, ss.center
    S = ss.nshell
    a, b = np.tril_indices(S)
    swap = L[a] < L[b]
    pa, pb = np.where(swap, b, a), np.where(swap, a, b)
    pcls = L[pa] * (L[pa] + 1) // 2 + L[pb]
    mid = 0.5 * (cen[pa] + cen[pb])
    out = []
    for cb in range(6):
        for ck in range(cb + 1):
            bra = np.flatnonzero(pcls == cb)
            ket = np.flatnonzero(pcls == ck)
            if len(bra) == 0 or len(ket) == 0:
                continue
            nc = 40 * per_class
            ib = bra[rng.integers(0, len(bra), nc)]
            ik = ket[rng.integers(0, len(ket), nc)]
            r = np.linalg.norm(mid[ib] - mid[ik], axis=1)
            far = np.argsort(-r)[: per_class // 20]
            edges = np.linspace(0.0, r.max() + 1e-9, bins + 1)
            which = np.clip(np.digitize(r, edges) - 1, 0, bins - 1)
            sel = list(far)
            want = (per_class - len(sel)) // bins + 1
            for k in range(bins):
                idx = np.flatnonzero(which == k)
                sel.extend(rng.choice(idx, size=min(want, len(idx)), replace=False).tolist())
            extra = per_class - len(sel)
            if extra > 0:
                sel.extend(rng.integers(0, nc, extra).tolist())
            sel = np.array(sel[: max(per_class, len(sel))])
            q = np.stack([pa[ib[sel]], pb[ib[sel]], pa[ik[sel]], pb[ik[sel]]], axis=1)
            flip1 = rng.random(len(q)) < 0.5
            flip2 = rng.random(len(q)) < 0.5
            q[flip1, 0], q[flip1, 1] = q[flip1, 1].copy(), q[flip1, 0].copy()
            q[flip2, 2], q[flip2, 3] = q[flip2, 3].copy(), q[flip2, 2].copy()
            bk = rng.random(len(q)) < 0.5
            q[bk] = q[bk][:, [2, 3, 0, 1]]
            out.append(q)
    return np.concatenate(out).astype(np.int64)


def _cluster(n):
    from mmd.clusters import water_cluster
    from mmd.molecule import Molecule
    return Molecule(water_cluster(n, seed=16), "6-31gss")


def _densities(mol):
    """The core-guess density (first Fock build of a direct RHF) and the next
    incremental density difference, as host arrays."""
    st = mol.scf_begin(direct=True, build=True)
    st.iterate()
    P1 = st.P.cpu().numpy()
    st.iterate()
    P2 = st.P.cpu().numpy()
    return P1, P2


@pytest.mark.parametrize("n", [2, 4])
def test_full_eri_tensor_and_formPT_of_water_clusters_vs_oracle(n):
    import oracle as O
    from mmd.integrals.fock import formPT
    from mmd.integrals.shells import shells_from_bfs
    from mmd.integrals.twoe import doERIs
    mol = _cluster(n)
    N = mol.nbasis
    ob = oracle_bfs(mol)
    # ERI tensor: every unique quartet (the oracle evaluates each shell quartet once,
    # memoised; pinned to its per-function ERI in the CPU suite)
    T = doERIs(N, np.zeros((N, N, N, N)), mol.bfs)
    i, j, k, l = O.unique_index(N)
    shells = [[int(f) for f in row if f >= 0] for row in shells_from_bfs(mol.bfs).func]
    ref = O.parallel_eri_unique_shells(ob, shells)
    err = np.abs(T[i, j, k, l] - ref)
    assert err.max() < 1e-12, (n, err.max())
    del T
    # Schwarz table
    scr = O.screen_table(ob)
    assert np.abs(mol.context.screen() - scr).max() < 1e-12
    # formPT with the oracle's screen dict: core-guess density, then an increment
    screen = {x: float(v) for x, v in enumerate(scr)}
    P1, P2 = _densities(mol)
    for P, Po in ((P1, np.zeros_like(P1)), (P2, P1)):
        G = formPT(P, Po, mol.bfs, N, screen, 1e-12)
        Go = O.formPT_table(P, Po, ref, N, scr, 1e-12)  # the oracle's ERIs computed above
        assert np.abs(G.imag).max() == 0.0
        gerr = np.abs(G.real - Go).max()
        assert gerr < 1e-12, (n, gerr)


def test_formPT_of_h2o2_matches_the_reference_call():
    """The first formPT call of the reference's own direct RHF on the benchmark
    generator's (H2O)2 / 6-31G** (inputs, output and its Schwarz table recorded by
    tests/golden/make_golden_h2o2_formpt.py): the GPU formPT through the reference's
    signature gives the reference's G to 1e-12."""
    from mmd.integrals.fock import formPT
    from mmd.molecule import Molecule
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "h2o2_631gss_formpt.npz"))
    mol = Molecule(str(g["geometry"]), "6-31gss")
    N = mol.nbasis
    screen = {x: float(v) for x, v in enumerate(g["screen"])}
    G = formPT(g["P"].astype(complex), np.zeros((N, N), dtype=complex), mol.bfs, N, screen, float(g["tol"]))
    assert np.abs(G.real - g["G"]).max() < 1e-12
    assert np.abs(mol.context.screen() - g["screen"]).max() < 1e-12


def test_h2o16_stratified_shell_quartets_vs_oracle():
    import oracle as O
    from mmd.integrals.shells import shells_from_bfs
    mol = _cluster(16)
    assert mol.nbasis == 400
    ss = shells_from_bfs(mol.bfs)
    q = stratified_quartets(ss, per_class=2000, seed=7)
    assert len(q) >= 21 * 2000
    got = mol.context.eri_quartets(q).cpu().numpy()
    shells = [[int(f) for f in row if f >= 0] for row in ss.func]
    ref = O.parallel_eri_shells(oracle_bfs(mol), [tuple(shells[s] for s in x) for x in q])
    worst_abs, worst_rel = 0.0, 0.0
    far_seen = 0
    for x, (qq, r) in enumerate(zip(q, ref)):
        g = got[x, : r.shape[0], : r.shape[1], : r.shape[2], : r.shape[3]]
        d = np.abs(g - r)
        worst_abs = max(worst_abs, float(d.max()))
        big = np.abs(r) > 1e-6
        if big.any():
            worst_rel = max(worst_rel, float((d[big] / np.abs(r[big])).max()))
        # components beyond the shells are zero
        assert np.count_nonzero(got[x]) <= r.size
    # the largest bra-ket distances of the sample (large-T Boys branch)
    cen = ss.center
    rpq = np.linalg.norm(0.5 * (cen[q[:, 0]] + cen[q[:, 1]]) - 0.5 * (cen[q[:, 2]] + cen[q[:, 3]]), axis=1)
    far_seen = int((rpq > 15.0).sum())
    assert worst_abs < 1e-12, worst_abs
    assert worst_rel < 1e-9, worst_rel
    assert far_seen > 100, far_seen


def test_eri_quartets_in_every_shell_order_match_the_tensor():
    """mmdg_eri_quartets on every shell quartet of water/6-31G** (all orders, so every
    orientation flag) against the ERI tensor of the same context."""
    from mmd.integrals.shells import shells_from_bfs
    from mmd.molecule import Molecule
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "mol_water_631gss.npz"))
    mol = Molecule(str(d["geometry"]), "6-31gss")
    ctx = mol.context
    T = ctx.eri_tensor().cpu().numpy()
    ss = shells_from_bfs(mol.bfs)
    S = ss.nshell
    q = np.array(np.meshgrid(*[np.arange(S)] * 4, indexing="ij")).reshape(4, -1).T
    got = ctx.eri_quartets(q).cpu().numpy()
    for x, (a, b, c, e) in enumerate(q):
        fa, fb, fc, fd = (ss.func[s][ss.func[s] >= 0] for s in (a, b, c, e))
        ref = T[np.ix_(fa, fb, fc, fd)]
        assert np.abs(got[x, : len(fa), : len(fb), : len(fc), : len(fd)] - ref).max() < 1e-14
    idx = d["TwoE_idx"]  # the reference's own values of a sample of the tensor
    assert np.abs(T[idx[:, 0], idx[:, 1], idx[:, 2], idx[:, 3]] - d["TwoE_val"]).max() < 1e-12
