"""Host-side logic (CPU): basis parsing and normalisation, shell grouping, clusters,
flop model, the C-ABI symbol table of libmmdg.so, the Boys table, the autotuner
cache, the batched SCF's padding and host eigensolves, DIIS against the reference's
formula, and the Crawford-format integral files."""
import os
import re

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_basis_normalisation_matches_oracle(golden):
    import oracle as O
    from mmd.integrals.twoe import Basis
    g = golden("eri_functions.npz")
    for o, s, k, e, c in zip(g["origin"], g["shell"], g["nprim"], g["exps"], g["coefs"]):
        a = Basis(o, s, int(k), e[:k], c[:k])
        b = O.Basis(o, s, int(k), e[:k], c[:k])
        assert np.allclose(a.coefs, b.coefs, rtol=1e-14, atol=0)
        assert np.allclose(a.norm, b.norm, rtol=1e-14, atol=0)


def test_molecule_basis_layout(golden):
    from mmd.molecule import Molecule
    d = golden("mol_water_631gss.npz")
    m = Molecule(str(d["geometry"]), "6-31gss")
    assert m.nbasis == int(d["nbasis"]) == 25
    assert m.nocc == 5
    # Cartesian order of momentum2shell (mmd/molecule.py:108-114); H: s3, s1, p1
    shells = [tuple(int(x) for x in b.shell) for b in m.bfs]
    assert shells[-5:] == [(0, 0, 0), (0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1)]
    d_idx = [i for i, s in enumerate(shells) if sum(s) == 2]
    assert [shells[i] for i in d_idx] == [(2, 0, 0), (1, 1, 0), (1, 0, 1), (0, 2, 0), (0, 1, 1), (0, 0, 2)]


def test_shell_grouping():
    from mmd.molecule import Molecule
    from mmd.integrals.shells import shells_from_bfs
    water = Molecule("\n0 1\nO 0 -0.075791844 0\nH 0.866811829 0.601435779 0\nH -0.866811829 0.601435779 0\n",
                     "6-31gss")
    ss = shells_from_bfs(water.bfs)
    assert ss.nshell == 12
    assert list(ss.L) == [0, 0, 1, 0, 1, 2, 0, 0, 1, 0, 0, 1]
    # every function appears exactly once
    f = ss.func[ss.func >= 0]
    assert sorted(f.tolist()) == list(range(25))
    # a ragged list: a lone d_zz, a p shell missing its y component, an s
    bfs = [water.bfs[i] for i in (14, 2, 4, 0)]
    ss2 = shells_from_bfs(bfs)
    assert ss2.nshell == 3
    assert ss2.func[0].tolist() == [-1, -1, -1, -1, -1, 0]
    assert ss2.func[1].tolist() == [1, -1, 2, -1, -1, -1]


def test_shell_grouping_rejects_f():
    from mmd.integrals.twoe import Basis
    from mmd.integrals.shells import shells_from_bfs
    with pytest.raises(ValueError):
        shells_from_bfs([Basis([0, 0, 0], (3, 0, 0), 1, [1.0], [1.0])])


def test_cluster_generator():
    from mmd.clusters import water_cluster_coords, water_cluster
    s1, x1 = water_cluster_coords(16, seed=3)
    s2, x2 = water_cluster_coords(16, seed=3)
    assert np.array_equal(x1, x2) and len(s1) == 48
    oxy = x1[0::3]
    d = np.linalg.norm(oxy[:, None] - oxy[None], axis=-1) + np.eye(16) * 1e9
    assert d.min() >= 2.5
    # rigid monomers: O-H bond lengths preserved
    for k in range(16):
        for h in (1, 2):
            assert abs(np.linalg.norm(x1[3 * k] - x1[3 * k + h]) - 1.0997) < 1e-3
    assert water_cluster(2, seed=1).count("\n") == 8


def test_flop_model():
    from mmd.flop_model import class_flops, prim_quartet_flops
    # (ss|ss): Boys + R only
    assert prim_quartet_flops(0, 0, 0, 0) == 12 + 3 + 2 + 2 + 2
    assert class_flops((1, 1, 1, 1), 1, 1, 1) > class_flops((1, 0, 0, 0), 1, 1, 1)


def _header_symbols():
    txt = open(os.path.join(REPO, "include", "mmdg.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|long long|const char\*)\s+(mmdg_\w+)\s*\(", txt, flags=re.M)))


def test_capi_exports_every_declared_symbol(built_lib):
    import ctypes
    lib = ctypes.CDLL(built_lib)
    syms = _header_symbols()
    assert "mmdg_fock" in syms and "mmdg_eri_tensor" in syms and len(syms) >= 10
    for s in syms:
        assert hasattr(lib, s), s


def test_boys_table_vs_mpmath(built_lib):
    """The GPU Boys table (built on the host in double-double arithmetic) is
    correctly rounded: F_{L+n}(T_k)/n! and exp(-T_k)/n! against mpmath."""
    import ctypes
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    lib = ctypes.CDLL(built_lib)
    lib.mmdg_boys_table.restype = ctypes.c_longlong
    lib.mmdg_boys_table.argtypes = [ctypes.c_void_p, ctypes.c_longlong]
    n = lib.mmdg_boys_table(None, 0)
    tab = np.zeros(n)
    assert lib.mmdg_boys_table(tab.ctypes.data, n) == n
    ngrid, lmax, row = 768, 8, 8
    fact = [1, 1, 2, 6, 24, 120, 720, 5040]
    for k in (0, 1, 17, 100, 333, 500, 767):
        T = mp.mpf(k) / 16
        for L in (0, 1, 4, 8):
            for nn in range(7):
                m = L + nn
                ex = mp.hyp1f1(m + mp.mpf(1) / 2, m + mp.mpf(3) / 2, -T) / (2 * m + 1) / fact[nn]
                got = tab[(L * ngrid + k) * row + nn]
                assert abs(got - float(ex)) <= 1.2e-16 * abs(float(ex)), (k, L, nn)
        e = tab[ngrid * (lmax + 1) * row + k * row]
        assert abs(e - float(mp.exp(-T))) <= 1.2e-16 * float(mp.exp(-T))


def test_realtime_rejects_unknown_direction():
    from mmd.realtime import _axis
    assert [_axis(d) for d in "xYz"] == [0, 1, 2]
    import pytest as _pt
    with _pt.raises(ValueError):
        _axis("w")


def test_single_threaded_blas_scope_restores_the_thread_count():
    import numpy as np
    from mmd.batch import _openblas_controls, _single_threaded_blas
    ctl = _openblas_controls()
    if ctl is None:
        import pytest as _pt
        _pt.skip("numpy's OpenBLAS not found in this process")
    before = ctl[0]()
    with _single_threaded_blas():
        assert ctl[0]() == 1
        w = np.linalg.eigh(np.diag([3.0, 1.0, 2.0]))[0]
    assert ctl[0]() == before
    assert w.tolist() == [1.0, 2.0, 3.0]


def test_autotune_cache_round_trip(tmp_path, monkeypatch):
    """The tuning cache stores one entry per key and survives a corrupt file."""
    from mmd import autotune
    monkeypatch.setattr(autotune, "CACHE", str(tmp_path / "tuning.json"))
    assert autotune._load_cache() == {}
    autotune._store_cache("gpu|a", autotune.Tuning([0] * 21, 4, {"x": 1}))
    autotune._store_cache("gpu|b", autotune.Tuning([152] * 21, 1))
    c = autotune._load_cache()
    assert c["gpu|a"]["streams"] == 4 and c["gpu|a"]["measured"] == {"x": 1}
    assert c["gpu|b"]["grids"] == [152] * 21
    (tmp_path / "tuning.json").write_text("{not json")
    assert autotune._load_cache() == {}
    assert not list(tmp_path.glob("*.tmp"))


def test_batch_padding_and_host_eigensolves():
    """The batched SCF's packed <-> padded density maps and its per-molecule host
    eigensolves (thread pool, converged molecules skipped) on CPU tensors."""
    import types
    import torch
    from mmd import batch
    N = np.array([3, 5, 2])
    br = object.__new__(batch.BatchRHF)
    br.torch, br.dev, br.N, br.B, br.Nmax = torch, "cpu", N, len(N), int(N.max())
    base = np.concatenate([[0], np.cumsum(N ** 2)[:-1]])
    br.ctx = types.SimpleNamespace(nn=int(np.sum(N ** 2)))
    pk, pd = [], []
    for b, n in enumerate(N):
        i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
        pk.append(base[b] + (i * n + j).ravel())
        pd.append(b * br.Nmax ** 2 + (i * br.Nmax + j).ravel())
    br.pk, br.pd = torch.as_tensor(np.concatenate(pk)), torch.as_tensor(np.concatenate(pd))
    rng = np.random.default_rng(3)
    packed = torch.as_tensor(rng.standard_normal(br.ctx.nn))
    padded = br._pad(packed)
    assert padded.shape == (3, 5, 5)
    assert torch.equal(padded[1, :5, :5].reshape(-1), packed[9:34])
    assert float(padded[0, 3:, :].abs().sum()) == 0.0 and float(padded[2, :, 2:].abs().sum()) == 0.0
    assert torch.equal(br._pack(padded), packed)
    sym = padded + padded.transpose(1, 2)
    E, C = br._eigh(sym, active=np.array([True, False, True]))
    for b in (0, 2):
        n = N[b]
        w = np.linalg.eigvalsh(sym[b, :n, :n].numpy())
        assert np.abs(E[b, :n].numpy() - w).max() < 1e-12
        V = C[b, :n, :n].numpy()
        assert np.abs(sym[b, :n, :n].numpy() @ V - V * E[b, :n].numpy()).max() < 1e-12
    assert float(E[1].abs().sum()) == 0.0 and float(C[1].abs().sum()) == 0.0


def test_diis_extrapolation_matches_the_reference_formula():
    """SCF._diis (device tensors, host (n+1)^2 solve) against a numpy restatement of
    the reference's updateDIIS (mmd/scf.py:146-180): error X (FPS - SPF) X, B_ij =
    tr(e_i^T e_j), an 8-deep window, F = sum_i w_i F_i; run on CPU tensors."""
    import types
    import torch
    from mmd.scf import SCF
    rng = np.random.default_rng(11)
    n = 6
    A = rng.standard_normal((n, n))
    S = A @ A.T + n * np.eye(n)
    w, U = np.linalg.eigh(S)
    X = (U / np.sqrt(w)) @ U.T
    P = rng.standard_normal((n, n))
    P = P + P.T
    fake = types.SimpleNamespace(context=types.SimpleNamespace(torch=torch))
    t = lambda a: torch.as_tensor(a, dtype=torch.float64)
    fs, es, rf, re_ = [], [], [], []
    for k in range(11):
        F = rng.standard_normal((n, n))
        F = F + F.T
        Fd, err = SCF._diis(fake, t(F), t(P), t(S), t(X), fs, es)
        # the reference's algorithm
        e = X @ (F @ P @ S - S @ P @ F) @ X
        rf.append(F)
        re_.append(e)
        if len(rf) > 8:
            del rf[0], re_[0]
        m = len(rf)
        B = np.zeros((m + 1, m + 1))
        B[-1, :] = B[:, -1] = -1.0
        B[-1, -1] = 0.0
        for i in range(m):
            for j in range(i + 1):
                B[i, j] = B[j, i] = np.trace(re_[i].T @ re_[j])
        r = np.zeros(m + 1)
        r[-1] = -1.0
        wts = np.linalg.solve(B, r)
        Fref = sum(wts[i] * rf[i] for i in range(m))
        assert len(fs) == m
        assert np.abs(Fd.numpy() - Fref).max() < 1e-10 * max(1.0, np.abs(Fref).max())
        assert abs(err - np.linalg.norm(e)) < 1e-10 * max(1.0, np.linalg.norm(e))


def test_save_integrals_writes_the_crawford_files(golden, tmp_path):
    """Molecule.save_integrals (mmd/molecule.py:295-315): enuc/nbf/nelec/s/t/v.dat,
    eri.dat as 1-based "i j k l value" lines over all N^4 indices, geometry.txt; the
    arrays read back equal the golden water/STO-3G integrals."""
    from mmd.molecule import Molecule
    d = golden("mol_water_sto3g.npz")
    m = Molecule(str(d["geometry"]), "sto-3g")
    m.S, m.T, m.V, m.TwoE = d["S"], d["T"], d["V"], d["TwoE"]
    m.nuc_energy = float(d["nuc_energy"])
    m.is_built = True
    out = str(tmp_path / "ints")
    m.save_integrals(out)
    N = m.nbasis
    assert float(np.loadtxt(out + "/enuc.dat")) == float(d["nuc_energy"])
    assert int(np.loadtxt(out + "/nbf.dat")) == N == 7
    assert int(np.loadtxt(out + "/nelec.dat")) == 10
    for name, ref in (("s", d["S"]), ("t", d["T"]), ("v", d["V"])):
        assert np.abs(np.loadtxt(out + f"/{name}.dat") - ref).max() < 1e-15
    rows = np.loadtxt(out + "/eri.dat")
    assert rows.shape == (N ** 4, 5)
    idx = rows[:, :4].astype(int) - 1
    assert (idx[:3] == [[0, 0, 0, 0], [0, 0, 0, 1], [0, 0, 0, 2]]).all()
    assert np.abs(rows[:, 4] - d["TwoE"][idx[:, 0], idx[:, 1], idx[:, 2], idx[:, 3]]).max() < 1e-15
    assert open(out + "/geometry.txt").read().strip() == str(d["geometry"]).strip()


def test_issued_and_useful_flop_counts():
    """The issued-FLOP count mirrors the code: one chunk pass and no padding equals
    the useful count; chunked classes and the warp kernel's padded lanes issue more;
    the Boys branch matters; (ss|ss) is counted by hand."""
    from mmd import flop_model as F
    row = [100.0, 10.0, 50.0, 20.0, 10.0]  # fq, shell q., prim q., bra passes, asymptotic Boys
    for c in F.CLASSES:
        i, u = F.issued_flops(c, row), F.useful_flops(c, row)
        assert i >= u > 0
        if F.fock_kernel(c) == "thread" and F._thread_config(tuple(c))[0] == 1:
            assert i == u
    assert F.fock_kernel((2, 2, 2, 2)) == "warp" and F.fock_kernel((1, 0, 0, 0)) == "thread"
    # (ss|ss), near: P-Q 3, |PQ|^2 5, pq, p+q, pq|PQ|^2 3, rsqrt 7 (a product and three
    # FMAs), alpha 2, T 1, Boys on float pairs 4 (y, one conversion sum, the last FMA),
    # R0 1; far: the common part and R0; ket 2 per primitive quartet, bra 2 per bra
    # pass, 6 per digested function quartet
    assert F.r0_flops(0, False) == 3 + 5 + 3 + 7 + 2 + 1 + 4 + 1
    assert F.r0_flops(0, True) == 3 + 5 + 3 + 7 + 1
    # (ps|ss): near and far share R0, rr M, R1 (3) and pq rr^2 (2); near adds T and two
    # Boys rows; (dd|dd) keeps the Boys-function form
    assert F.r0_flops(1, True) == 18 + 2 + 3
    assert F.r0_flops(1, False) == 18 + 2 + 1 + F.boys_df_flops(1) + 3
    assert F.r0_flops(8, True) == 3 + 5 + 1 + 7 + 3 + 1 + F.boys_flops(8, True) + 18
    assert F.useful_flops((0, 0, 0, 0), [1, 1, 1, 1, 0]) == F.r0_flops(0, False) + 2 + 2 + 6
    assert F.boys_flops(3, True) < F.boys_flops(3, False)
    # the recursion counts 1 FLOP for a first step, 2 for fma(X, R1, R2) (m = 2) and 3
    # for fma(X, R1, (m-1) R2); level 3 has 10 entries with m = 1, 6 with m = 2, 3 with m = 3
    assert F.recursion_flops(1) == 3 and F.recursion_flops(2) == 3 + 6 * 1 + 3 * 2
    assert F.recursion_flops(3) == F.recursion_flops(2) + 10 * 1 + 6 * 2 + 3 * 3


def test_context_cache_eviction_keeps_held_contexts_open(monkeypatch):
    """Dropping a cache entry must not close a context a Molecule still uses."""
    from mmd.integrals import twoe

    class FakeCtx:
        closed = False

        def device_bytes(self):
            return 10

        def close(self):
            self.closed = True

    monkeypatch.setattr(twoe, "CONTEXT_CACHE_MAX", 2)
    twoe._ctx_cache.clear()
    held = []
    for k in range(4):
        c = FakeCtx()
        held.append(c)
        twoe._ctx_cache[("k", k)] = c
        twoe._trim_cache(keep=("k", k))
    assert len(twoe._ctx_cache) == 2 and not any(c.closed for c in held)
    twoe.clear_context_cache()
    assert not twoe._ctx_cache and not any(c.closed for c in held)


def test_occupied_subspace_iteration_matches_the_dense_solve():
    """Chebyshev-filtered subspace iteration (torch on the CPU here) against
    numpy.linalg.eigh on a Fock-like spectrum: 8 core orbitals near -20.55 Eh, 32
    valence in [-1.35, -0.45], virtuals in [0.1, 4]; warm-started through a sequence of
    perturbations of decreasing size, as between SCF iterations."""
    import torch
    from mmd.scf import OccupiedSubspace
    rng = np.random.default_rng(11)
    N, nocc = 200, 40
    w = np.concatenate([-20.55 + 0.02 * rng.standard_normal(8), np.sort(rng.uniform(-1.35, -0.45, 32)),
                        np.sort(rng.uniform(0.1, 4.0, N - 40))])
    Q, _ = np.linalg.qr(rng.standard_normal((N, N)))
    F = (Q * w) @ Q.T
    sub = OccupiedSubspace(nocc, tol=1e-9)
    assert OccupiedSubspace.applicable(N, nocc)
    w0, v0 = np.linalg.eigh(F)
    sub.start(torch.tensor(F), w0, v0)
    # the core orbitals are split off from the valence slice
    assert sub.core_count(sub.theta, sub.theta[-1], sub.lmax) == 8
    for eps in (1e-1, 1e-2, 1e-4, 1e-6):
        E = rng.standard_normal((N, N))
        F = F + eps * (E + E.T) / np.linalg.norm(E + E.T, 2)
        r = sub.solve(torch.tensor(F))
        assert r is not None
        theta, V = r[0], r[1].numpy()
        we, ve = np.linalg.eigh(F)
        assert np.abs(theta - we[:nocc]).max() < 1e-10
        Pe = ve[:, :nocc] @ ve[:, :nocc].T
        assert np.linalg.norm(V @ V.T - Pe) < 1e-7
    assert sub.fallbacks == 0 and sub.solves == 4
    # a warm start from an unrelated matrix does not pass the residual test silently
    G = rng.standard_normal((N, N))
    r = sub.solve(torch.tensor(G + G.T))
    if r is not None:
        wg = np.linalg.eigvalsh(G + G.T)
        assert np.abs(r[0] - wg[:nocc]).max() < 1e-8


def test_float_pair_boys_rows_match_fp64_horner():
    """The float-pair evaluation of the Boys Taylor rows (md_device.cuh, boys_eval_df),
    restated in numpy float32 with exact FMA products: the tail n >= 5 in FP32, the
    steps n = 4..1 as float pairs, the last step c_0 + y * tail in FP64.  Over T < 48,
    orders 0..4 and the exp rows it stays within 4e-16 of the FP64 Horner value of the
    same table row (the device table is the host table, split into (hi, lo) floats)."""
    import ctypes
    from mmd import _native
    n = _native.lib().mmdg_boys_table(None, 0)
    tab = np.zeros(n)
    _native.lib().mmdg_boys_table(tab.ctypes.data_as(ctypes.c_void_p), n)
    NG, ROW, LMAX = 768, 8, 8
    EXPOFF = NG * (LMAX + 1) * ROW
    f32 = np.float32

    def fmaf(a, b, c):  # float products are exact in float64
        return f32(np.float64(a) * np.float64(b) + np.float64(c))

    def two_sum(a, b):
        s = f32(a + b)
        bb = f32(s - a)
        return s, f32(f32(a - f32(s - bb)) + f32(b - bb))

    def df_fma(ah, al, yh, yl, ch, cl):
        p = f32(ah * yh)
        e = fmaf(al, yh, fmaf(ah, yl, fmaf(ah, yh, -p)))
        sh, sl = two_sum(p, ch)
        s = f32(sh + f32(sl + f32(e + cl)))
        return s, f32(f32(sl + f32(e + cl)) - f32(s - sh))

    def split(x):
        h = f32(x)
        return h, f32(x - np.float64(h))

    def row_df(row, y, deg):
        m, e = np.frexp(y)
        yh = f32(np.trunc(m * 2 ** 24) / 2 ** 24 * 2.0 ** e) if y != 0 else f32(0)
        yl = f32(y - np.float64(yh))
        hl = [split(c) for c in row]
        t = fmaf(hl[7][0], yh, hl[6][0]) if deg == 7 else hl[6][0]
        ph, pl = fmaf(t, yh, hl[5][0]), f32(0)
        for j in (4, 3, 2, 1):
            ph, pl = df_fma(ph, pl, yh, yl, hl[j][0], hl[j][1])
        return y * (np.float64(ph) + np.float64(pl)) + row[0]

    def row_64(row, y, deg):
        f = row[deg]
        for j in range(deg - 1, -1, -1):
            f = f * y + row[j]
        return f

    rng = np.random.default_rng(5)
    worst = 0.0
    for T in rng.uniform(0.0, 47.9, 120):
        k = min(int(np.rint(np.float32(T) * 16)), NG - 1)
        y = k / 16.0 - T
        rows = [(tab[(L * NG + k) * ROW:(L * NG + k + 1) * ROW], 6) for L in range(5)]
        rows.append((tab[EXPOFF + k * ROW:EXPOFF + (k + 1) * ROW], 7))
        for row, deg in rows:
            ref = row_64(row, y, deg)
            worst = max(worst, abs(row_df(row, y, deg) - ref) / abs(ref))
    assert worst < 4e-16, worst


def test_rsqrt_step_restated_equals_the_fp64_step():
    """rsqrt_dd (md_device.cuh) restated on the CPU with exact FMAs: from the FP32 seed
    y0 (correctly rounded, and 1 or 2 ulp off either way, as CUDA's rsqrtf may be) and
    e = 1 - x y0^2, the step y0 + (y0/2)(e + (3e/4) e) with 3e/4 taken in FP32 gives the
    same double as the all-FP64 step y0 + y0 e (1/2 + 3e/8), within 1 ulp of 1/sqrt(x),
    over p + q of primitive pairs, pq |PQ|^2 of far quartets and T >= 48."""
    from fractions import Fraction
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    f32 = np.float32

    def fma(a, b, c):  # one rounding, as the device FMA
        return float(Fraction(a) * Fraction(b) + Fraction(c))

    def f32_tz(x):  # md_device.cuh f32_of_nonneg / f32_of_double_tz: toward zero
        m, ex = np.frexp(abs(x))
        v = np.copysign(np.floor(m * 2.0 ** 24) / 2.0 ** 24 * 2.0 ** ex, x)
        return f32(v) if abs(v) >= 2.0 ** -126 else f32(0)

    def seed(x, k):
        y = f32(1.0 / np.sqrt(np.float64(f32_tz(x))))
        for _ in range(abs(k)):
            y = np.nextafter(y, f32(np.inf) if k > 0 else f32(0))
        return y

    rng = np.random.default_rng(5)
    xs = np.concatenate([10.0 ** rng.uniform(-2, 11, 400), rng.uniform(0.1, 100.0, 400),
                         [1.0, 2.0, 4.0, 0.25, 48.0, 47.96875, 123456.789]])
    for x in xs:
        exact = float(1 / mp.sqrt(mp.mpf(float(x))))
        for k in (-2, -1, 0, 1, 2):
            y0f = seed(x, k)
            y0 = float(y0f)
            e = fma(-x, y0 * y0, 1.0)
            assert abs(e) < 2.0 ** -20
            new = fma(float(f32(0.5) * y0f), fma(float(f32(f32(0.75) * f32_tz(e))), e, e), y0)
            old = fma(y0, e * fma(e, 0.375, 0.5), y0)
            assert new == old
            assert abs(new - exact) <= np.spacing(exact)


def test_device_constants_are_correctly_rounded():
    """The mathematical constants written as literals in the CUDA sources equal the
    correctly rounded doubles of their values (a digit off in sqrt(2 pi^{5/2}), which
    every E' coefficient carries, shifts every ERI by the same relative amount)."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    csrc = os.path.join(REPO, "mcmurchie-davidson_gb300", "csrc")

    def literal(fname, pattern):
        with open(os.path.join(csrc, fname)) as f:
            m = re.search(pattern, f.read())
        assert m, (fname, pattern)
        return float(m.group(1))

    num = r"([0-9]+\.[0-9]+(?:[eE][-+]?[0-9]+)?)"
    cases = [
        ("md_device.cuh", r"kTwoPi52 = " + num, 2 * mp.pi ** mp.mpf(2.5)),
        ("md_device.cuh", r"kSqrtTwoPi52 = " + num, mp.sqrt(2 * mp.pi ** mp.mpf(2.5))),
        ("md_device.cuh", r"kHalfSqrtPi = " + num, mp.sqrt(mp.pi) / 2),
        ("capi.cu", r"comp_norm\(int l\) \{ return l >= 2 \? " + num, 1 / mp.sqrt(3)),
        ("grad.cu", r"comp_norm\(int l\) \{ return l >= 2 \? " + num, 1 / mp.sqrt(3)),
        ("capi.cu", r"const double PI = " + num, mp.pi),
        ("grad.cu", r"kPi = " + num, mp.pi),
    ]
    for fname, pattern, exact in cases:
        assert literal(fname, pattern) == float(exact), (fname, pattern)


def test_update_diis_host_helper_matches_the_reference_steps():
    """SCF.updateDIIS (host arrays, the reference's public helper mmd/scf.py:146-180)
    against a loop restatement: the current self.F joins the history (not the F
    argument), the error is X (FPS - SPF) X, B_ij = Re tr(e_i^H e_j), 8-deep window,
    complex result."""
    import types
    from mmd.scf import SCF
    rng = np.random.default_rng(12)
    n = 5
    A = rng.standard_normal((n, n))
    S = A @ A.T + n * np.eye(n)
    w, U = np.linalg.eigh(S)
    X = (U / np.sqrt(w)) @ U.T
    mol = types.SimpleNamespace(S=S, X=X, nbasis=n, adj=lambda x: np.conjugate(x).T)
    rf, re_ = [], []
    for k in range(11):
        Fc = rng.standard_normal((n, n)); Fc = Fc + Fc.T        # self.F
        Fa = rng.standard_normal((n, n)); Fa = Fa + Fa.T        # the F argument
        P = rng.standard_normal((n, n)); P = P + P.T
        mol.F = Fc.astype(complex)
        got = SCF.updateDIIS(mol, Fa, P)
        FPS = Fa @ P @ S
        rf.append(Fc)
        re_.append(X @ (FPS - FPS.T) @ X)
        if len(rf) > 8:
            del rf[0], re_[0]
        m = len(rf)
        B = np.zeros((m + 1, m + 1))
        B[-1, :] = B[:, -1] = -1.0
        B[-1, -1] = 0.0
        for i in range(m):
            for j in range(i + 1):
                B[i, j] = B[j, i] = np.trace(re_[i].T @ re_[j])
        r = np.zeros(m + 1)
        r[-1] = -1.0
        wts = np.linalg.solve(B, r)
        ref = sum(wts[i] * rf[i] for i in range(m))
        assert got.dtype == complex and got.shape == (n, n)
        assert len(mol.fockSet) == m == len(mol.errorSet)
        assert np.abs(got - ref).max() < 1e-10 * max(1.0, np.abs(ref).max())


def test_rhf_results_keep_the_reference_attributes():
    """_RHFState.finish hands back the reference's attributes as complex host arrays,
    including F_old (the Fock matrix before the last build, mmd/scf.py:32) and, after
    a conventional run, the last build's J and K (mmd/scf.py:97-98); run on CPU tensors."""
    import types
    import torch
    from mmd.scf import _RHFState
    n = 4
    gen = torch.Generator().manual_seed(3)
    t = lambda: torch.randn(n, n, dtype=torch.float64, generator=gen)
    for direct in (False, True):
        mol = types.SimpleNamespace(nuc_energy=1.0, direct=direct, _last_jk=(t(), t()))
        st = _RHFState.__new__(_RHFState)
        st.mol, st.E, st.energy = mol, torch.arange(n, dtype=torch.float64), -5.0
        st.P, st.P_old, st.F, st.FO, st.C, st.CO, st.F_old = (t() for _ in range(7))
        _RHFState.finish(st)
        for name in ("P", "P_old", "F", "FO", "C", "CO", "F_old"):
            assert getattr(mol, name).dtype == np.complex128, name
        assert np.array_equal(mol.F_old.real, st.F_old.numpy())
        assert mol.el_energy == -6.0 and mol.MO.dtype == np.float64
        if direct:
            assert not hasattr(mol, "J")
        else:
            assert np.array_equal(mol.J.real, mol._last_jk[0].numpy())
            assert np.array_equal(mol.K.real, mol._last_jk[1].numpy())


def test_memoised_basis_normalisation_is_bit_identical():
    """Basis functions with the same shell, exponents and coefficients reuse one
    normalisation: bit-identical to normalising afresh, and each function owns copies."""
    from mmd.integrals import twoe
    ex, co = [5.0331513, 1.1695961, 0.3803890], [-0.09996723, 0.39951283, 0.70011547]
    twoe._NORMALISED.clear()
    a = twoe.Basis([0.0, 0.0, 0.0], (1, 1, 0), 3, ex, co)   # computed
    b = twoe.Basis([1.0, 2.0, 3.0], (1, 1, 0), 3, ex, co)   # from the memo
    twoe._NORMALISED.clear()
    c = twoe.Basis([1.0, 2.0, 3.0], (1, 1, 0), 3, ex, co)   # computed again
    for x in (a, b):
        assert np.array_equal(x.norm, c.norm) and np.array_equal(x.coefs, c.coefs)
    b.coefs[0] = 0.0
    d = twoe.Basis([0.0, 0.0, 0.0], (1, 1, 0), 3, ex, co)
    assert np.array_equal(d.coefs, c.coefs) and not np.shares_memory(d.coefs, c.coefs)
    e = twoe.Basis([0.0, 0.0, 0.0], (2, 0, 0), 3, ex, co)   # another shell: its own entry
    assert not np.array_equal(e.norm, c.norm)
