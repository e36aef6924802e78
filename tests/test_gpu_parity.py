"""GPU parity: the CUDA path (through the C ABI) against the reference's golden
outputs and the oracle.  Tolerances: 1e-12 absolute per ERI / Fock element /
one-electron integral, 1e-10 Eh per SCF energy, 1e-14 relative for the Boys
function (orders 0..8)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
MOLS = ["h2_sto3g", "water_sto3g", "methane_sto3g", "helium_ccpvtz", "formaldehyde_sto3g", "water_dz",
        "water_321g", "water_631g", "water_631gss", "water_631ppgss", "w2_631g", "w3_631g"]


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return built_lib


def _load(name):
    return dict(np.load(os.path.join(GOLDEN, name), allow_pickle=False))


def _mol(d):
    from mmd.molecule import Molecule
    return Molecule(str(d["geometry"]), str(d["basis"]))


def test_boys_gpu_vs_mpmath():
    import torch
    from mmd import _native
    g = _load("boys_grid.npz")
    ctx = _native.scratch_context()
    T = torch.tensor(g["T"], dtype=torch.float64, device="cuda")
    for m in range(9):
        got = ctx.boys(m, T).cpu().numpy()
        ex = g["mpmath"][m]
        rel = np.abs(got - ex) / np.abs(ex)
        assert rel.max() < 1e-14, (m, rel.max(), g["T"][rel.argmax()])


def test_rsqrt_of_the_eri_kernels_within_one_ulp():
    """rsqrt_dd (FP32 estimate + one third-order Newton/Householder step in FP64) is
    within 1 ulp of the exact 1/sqrt(x) over the range the kernels use it on (p + q of
    primitive pairs, and T >= 48 in the Boys function), like CUDA's own rsqrt."""
    import ctypes
    import torch
    from mmd import _native
    mp = pytest.importorskip("mpmath")
    rng = np.random.default_rng(11)
    x = np.concatenate([10.0 ** rng.uniform(-2, 9, 20000), rng.uniform(0.1, 100.0, 20000),
                        np.array([1.0, 2.0, 3.0, 48.0, 47.96875, 1e-3, 123456.789])])
    xd = torch.tensor(x, device="cuda")
    ours, cuda = torch.empty_like(xd), torch.empty_like(xd)
    ctx = _native.scratch_context()
    _native.check(_native.lib().mmdg_rsqrt(ctx._h, xd.numel(), ctypes.c_void_p(xd.data_ptr()),
                                           ctypes.c_void_p(ours.data_ptr()), ctypes.c_void_p(cuda.data_ptr()),
                                           _native.stream_ptr()), "mmdg_rsqrt")
    o, c = ours.cpu().numpy(), cuda.cpu().numpy()
    mp.mp.dps = 40
    sel = np.arange(0, len(x), 7)
    exact = np.array([float(1 / mp.sqrt(mp.mpf(float(v)))) for v in x[sel]])
    ulp = np.spacing(exact)
    assert np.abs(o[sel] - exact).max() <= 1.0 * ulp.max() and np.all(np.abs(o[sel] - exact) <= ulp)
    assert np.all(np.abs(c[sel] - exact) <= ulp)
    assert np.all(np.abs(o - c) <= 2 * np.spacing(c))


def test_boys_gpu_rejects_orders_outside_the_path():
    from mmd.integrals.onee import _boys
    with pytest.raises(ValueError):
        _boys(9, 1.0)
    assert abs(_boys(0, 0.0) - 1.0) < 1e-15


def test_eri_every_class_vs_reference():
    """Contracted ERIs of all 81 (la lb|lc ld) orderings, carbon 6-31G** s/p/d on three centres."""
    from mmd.integrals.twoe import Basis, doERIs
    g = _load("eri_functions.npz")
    bfs = [Basis(o, s, int(k), e[:k], c[:k]) for o, s, k, e, c in
           zip(g["origin"], g["shell"], g["nprim"], g["exps"], g["coefs"])]
    N = len(bfs)
    T = doERIs(N, np.zeros((N, N, N, N)), bfs)
    q = g["quartets"]
    got = T[q[:, 0], q[:, 1], q[:, 2], q[:, 3]]
    err = np.abs(got - g["eri"])
    assert err.max() < 1e-12, err.max()
    # the 8-fold permutational symmetry of the tensor
    assert np.abs(T - T.transpose(1, 0, 2, 3)).max() == 0.0
    assert np.abs(T - T.transpose(2, 3, 0, 1)).max() == 0.0


def test_eri_single_call_api():
    """ERI(a, b, c, d) on individual functions (the reference's tests/test013.py usage)."""
    from mmd.integrals.twoe import Basis, ERI
    g = _load("eri_functions.npz")
    bfs = [Basis(o, s, int(k), e[:k], c[:k]) for o, s, k, e, c in
           zip(g["origin"], g["shell"], g["nprim"], g["exps"], g["coefs"])]
    for n in range(0, len(g["quartets"]), 97):
        i, j, k, l = g["quartets"][n]
        assert abs(ERI(bfs[i], bfs[j], bfs[k], bfs[l]) - g["eri"][n]) < 1e-12


@pytest.mark.parametrize("name", MOLS)
def test_molecule_integrals_vs_reference(name):
    d = _load(f"mol_{name}.npz")
    mol = _mol(d)
    mol.build(direct=False)
    for key in ("S", "T", "V"):
        assert np.abs(getattr(mol, key) - d[key]).max() < 1e-12, key
    assert abs(mol.nuc_energy - float(d["nuc_energy"])) < 1e-12
    if "TwoE" in d:
        assert np.abs(mol.TwoE - d["TwoE"]).max() < 1e-12
    else:
        idx = d["TwoE_idx"]
        got = mol.TwoE[idx[:, 0], idx[:, 1], idx[:, 2], idx[:, 3]]
        assert np.abs(got - d["TwoE_val"]).max() < 1e-12


@pytest.mark.parametrize("name", [m for m in MOLS if "screen" in _load(f"mol_{m}.npz")])
def test_schwarz_table_vs_reference(name):
    d = _load(f"mol_{name}.npz")
    mol = _mol(d)
    scr = mol.context.screen()
    assert np.abs(scr - d["screen"]).max() < 1e-12


@pytest.mark.parametrize("name", [m for m in MOLS if "formPT0_G" in _load(f"mol_{m}.npz")])
def test_formPT_vs_reference_records(name):
    """The reference's own recorded formPT calls (inputs and unsymmetrised output)."""
    from mmd.integrals.fock import formPT
    d = _load(f"mol_{name}.npz")
    mol = _mol(d)
    N = mol.nbasis
    screen = {i: float(v) for i, v in enumerate(d["screen"])}
    k = 0
    while f"formPT{k}_G" in d:
        G = formPT(d[f"formPT{k}_P"], d[f"formPT{k}_Pold"], mol.bfs, N, screen, 1e-12)
        err = np.abs(G.real - d[f"formPT{k}_G"]).max()
        assert err < 1e-12, (k, err)
        assert np.abs(G.imag).max() == 0.0
        k += 1


def test_formPT_vs_oracle_random_density():
    """Random symmetric density on water/6-31G** (every class up to (dd|dd)) vs the oracle."""
    import oracle as O
    from mmd.integrals.fock import formPT
    d = _load("mol_water_631gss.npz")
    mol = _mol(d)
    N = mol.nbasis
    obfs = []
    for atom in mol.atoms:
        for momentum, prims in mol.basis_data[atom.charge]:
            ex = [e for e, c in prims]
            co = [c for e, c in prims]
            for sh in mol.momentum2shell(momentum):
                obfs.append(O.Basis(atom.origin, sh, len(ex), ex, co))
    rng = np.random.default_rng(5)
    A = rng.standard_normal((N, N)) * 0.1
    P = A + A.T
    Po = P * 0.9
    G = formPT(P, Po, mol.bfs, N, d["screen"], 1e-12)
    Go = O.formPT(P, Po, obfs, N, d["screen"], 1e-12)
    assert np.abs(G - Go).max() < 1e-12


@pytest.mark.parametrize("name", MOLS)
def test_rhf_energy_conventional(name):
    """Tightly converged (conver 1e-12, dE < 1e-10) energies agree to 1e-10 Eh.  At the
    default conver = 1e-8 the stopping iterate is path dependent (rounding in eigh and
    DIIS moves it), and the reference's energy pairs the last density with the Fock
    matrix of the one before, an error first order in ||P - P_old|| < 1e-8: that
    energy is held to 5e-8 (1.3e-8 seen on methane with a different LAPACK driver)."""
    d = _load(f"mol_{name}.npz")
    E12 = _mol(d).RHF(doPrint=False, conver=1e-12)
    assert abs(E12 - float(d["energy_conv_1e12"])) < 1e-10, (E12, float(d["energy_conv_1e12"]))
    E = _mol(d).RHF(doPrint=False)
    assert abs(E - float(d["energy_conv"])) < 5e-8, (E, float(d["energy_conv"]))


@pytest.mark.parametrize("name", [m for m in MOLS if "energy_direct" in _load(f"mol_{m}.npz")])
def test_rhf_energy_direct(name):
    d = _load(f"mol_{name}.npz")
    mol = _mol(d)
    E = mol.RHF(doPrint=False, direct=True)
    assert abs(E - float(d["energy_direct"])) < 5e-8, (E, float(d["energy_direct"]))  # see above
    assert mol.is_converged
    # converged as far as the incremental build allows (the acc2e = 1e-12 screening of
    # every build leaves a ||dP|| floor near 1e-11, for the reference as for this
    # path): the energy equals the tightly converged conventional reference to the
    # size of that screening error
    m10 = _mol(d)
    E10 = m10.RHF(doPrint=False, direct=True, conver=1e-10)
    assert m10.is_converged
    assert abs(E10 - float(d["energy_conv_1e12"])) < 5e-10, (E10, float(d["energy_conv_1e12"]))


def test_dipole_water():
    d = _load("mol_water_sto3g.npz")
    mol = _mol(d)
    mol.RHF(doPrint=False, conver=1e-14)
    # reference tests/test002.py:17-18
    assert np.allclose(mol.mu, np.array([0.0, 1.5340, 0.0]), atol=1e-4)


def test_unsupported_angular_momentum_is_an_error():
    from mmd import _native
    from mmd.integrals.shells import ShellSet
    ss = ShellSet(nfunc=10, L=np.array([3], dtype=np.int32), nprim=np.array([1], dtype=np.int32),
                  center=np.zeros((1, 3)), exps=np.array([1.0]), coefs=np.array([1.0]),
                  func=np.array([[0, 1, 2, 3, 4, 5]], dtype=np.int32))
    with pytest.raises(_native.MMDGError):
        _native.Context(ss)


def test_bad_inputs_are_errors():
    from mmd import _native
    from mmd.integrals.shells import ShellSet
    bad = ShellSet(nfunc=1, L=np.array([0], dtype=np.int32), nprim=np.array([1], dtype=np.int32),
                   center=np.zeros((1, 3)), exps=np.array([-1.0]), coefs=np.array([1.0]),
                   func=np.array([[0, -1, -1, -1, -1, -1]], dtype=np.int32))
    with pytest.raises(_native.MMDGError):
        _native.Context(bad)
    oob = ShellSet(nfunc=1, L=np.array([1], dtype=np.int32), nprim=np.array([1], dtype=np.int32),
                   center=np.zeros((1, 3)), exps=np.array([1.0]), coefs=np.array([1.0]),
                   func=np.array([[0, 1, 2, -1, -1, -1]], dtype=np.int32))
    with pytest.raises(_native.MMDGError):
        _native.Context(oob)


def test_single_function_basis():
    """Ragged edge: one s function (a 1^4 tensor, one Fock element)."""
    from mmd.integrals.twoe import Basis, doERIs
    import oracle as O
    b = Basis([0.1, 0.2, 0.3], (0, 0, 0), 2, [1.3, 0.4], [0.5, 0.6])
    ob = O.Basis([0.1, 0.2, 0.3], (0, 0, 0), 2, [1.3, 0.4], [0.5, 0.6])
    T = doERIs(1, np.zeros((1, 1, 1, 1)), [b])
    assert abs(T[0, 0, 0, 0] - O.ERI(ob, ob, ob, ob)) < 1e-12


def test_fock_counts_and_linearity():
    """G is linear in dP (a size-independent property) and the counters are consistent."""
    import torch
    d = _load("mol_w3_631g.npz")
    mol = _mol(d)
    ctx = mol.context
    N = mol.nbasis
    rng = np.random.default_rng(1)
    A = rng.standard_normal((N, N))
    P1 = torch.tensor(A + A.T, device="cuda").reshape(-1)
    B = rng.standard_normal((N, N))
    P2 = torch.tensor(B + B.T, device="cuda").reshape(-1)
    G1 = ctx.fock(P1, tol=0.0, counts=True).clone()
    c1 = ctx.last_counts.copy()
    G2 = ctx.fock(P2, tol=0.0).clone()
    G12 = ctx.fock(P1 + 2 * P2, tol=0.0)
    assert torch.max(torch.abs(G12 - (G1 + 2 * G2))).item() < 1e-11
    # with tol = 0 every unique function quartet is digested: N(N+1)/2 pairs, triangle
    npair = N * (N + 1) // 2
    assert int(c1[:, 0].sum()) == npair * (npair + 1) // 2


def test_mixed_precision_fock_and_energy():
    """FP32 for shell quartets with Schwarz bound below 1e-5 (FP64 for the rest, for
    the Boys branches' inputs of large-bound quartets, Fock accumulation, DIIS,
    eigensolve and energy): per-build max |dF| and the final energy against the
    all-FP64 path on a seeded (H2O)4 / 6-31G** cluster."""
    import torch
    from mmd.clusters import water_cluster
    from mmd.molecule import Molecule
    geom = water_cluster(4, seed=3)
    m64 = Molecule(geom, "6-31gss")
    E64 = m64.RHF(doPrint=False, direct=True)
    m32 = Molecule(geom, "6-31gss")
    E32 = m32.RHF(doPrint=False, direct=True, fp32_below=1e-5)
    assert abs(E32 - E64) < 1e-8, (E32, E64)
    # one full build on the converged density: max element error of G
    ctx = m64.context
    P = torch.tensor(np.real(m64.P), device="cuda").reshape(-1).contiguous()
    G64 = ctx.fock(P, tol=1e-12).clone()
    G32 = ctx.fock(P, tol=1e-12, fp32_below=1e-5)
    assert torch.max(torch.abs(G64 - G32)).item() < 1e-9


def test_primitive_pair_screening_is_below_the_parity_tolerance():
    """Contexts built with the default primitive-pair screening (1e-18) and with none
    (prim_tol = 0) give the same Fock builds and ERI tensors to far below 1e-12, with
    the same screened function quartets and fewer primitive quartets."""
    import torch
    from mmd import _native
    from mmd.clusters import water_cluster
    from mmd.integrals.shells import shells_from_bfs
    from mmd.molecule import Molecule
    m = Molecule(water_cluster(4, seed=3), "6-31gss")
    ss = shells_from_bfs(m.bfs)
    full, pruned = _native.Context(ss, prim_tol=0.0), _native.Context(ss)
    rng = np.random.default_rng(5)
    A = rng.standard_normal((m.nbasis, m.nbasis)) * 0.1
    dP = torch.as_tensor(A + A.T, device="cuda").reshape(-1).contiguous()
    G0 = full.fock(dP, counts=True).cpu().numpy()
    c0 = full.last_counts.astype(np.int64)
    G1 = pruned.fock(dP, counts=True).cpu().numpy()
    c1 = pruned.last_counts.astype(np.int64)
    assert np.abs(G1 - G0).max() < 1e-13
    assert (c1[:, 0] == c0[:, 0]).all() and (c1[:, 1] == c0[:, 1]).all()
    assert c1[:, 2].sum() < 0.95 * c0[:, 2].sum()
    w = _mol(_load("mol_water_631gss.npz"))
    ws = shells_from_bfs(w.bfs)
    T0 = _native.Context(ws, prim_tol=0.0).eri_tensor().cpu().numpy()
    T1 = _native.Context(ws).eri_tensor().cpu().numpy()
    assert np.abs(T1 - T0).max() < 1e-14


def test_fp64_pipe_probe_reports_both_pipes():
    """mmdg_measure_fp64_pipes: DFMA and FP64 tensor-core rates are positive and the
    combined kernel takes at least as long as either stream alone."""
    from mmd import _native
    r = _native.measure_fp64_pipes(_native.scratch_context(), 8)
    assert r["dfma_tflops"] > 0.1 and r["dmma_tflops"] > 0.1
    assert r["both_ms"] >= 0.9 * max(r["dfma_ms"], r["dmma_ms"])
