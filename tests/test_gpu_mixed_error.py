"""Per-ERI error of the FP32 class code that mixed-precision Fock builds use for
quartets whose Schwarz bound is below their threshold (FP32 Boys interpolation,
Hermite recursion and transforms; the Fock accumulation stays FP64).

Measured on a stratified sample of (H2O)4 / 6-31G** shell quartets of every angular
class (mmdg_eri_quartets in both precisions): the error of every ERI relative to its
Cauchy-Schwarz bound sqrt((ij|ij)(kl|kl)), the quantity the threshold is applied to,
stays below KAPPA.  An FP32 quartet therefore carries an absolute error below
KAPPA x threshold (1e-5 -> 2e-11 Eh, 1e-3 -> 2e-9 Eh per ERI), and its weight in G
is that times a density element."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KAPPA = 2e-6  # bound of |ERI_fp32 - ERI_fp64| / sqrt((ij|ij)(kl|kl)); FP32 unit roundoff is 6e-8


def test_fp32_quartet_error_relative_to_the_schwarz_bound():
    from mmd.clusters import water_cluster
    from mmd.integrals.shells import shells_from_bfs
    from mmd.molecule import Molecule
    from test_gpu_benchsize import stratified_quartets
    mol = Molecule(water_cluster(4, seed=16), "6-31gss")
    ctx = mol.context
    ss = shells_from_bfs(mol.bfs)
    q = stratified_quartets(ss, per_class=400, seed=5)
    e64 = ctx.eri_quartets(q).cpu().numpy()
    e32 = ctx.eri_quartets(q, fp32=True).cpu().numpy()
    scr = ctx.screen()
    N = mol.nbasis
    diag = np.zeros((N, N))
    ii, jj = np.tril_indices(N)
    diag[ii, jj] = scr[ii * (ii + 1) // 2 + jj]
    diag = diag + diag.T - np.diag(np.diag(diag))
    worst = 0.0
    for x, (a, b, c, d) in enumerate(q):
        fa, fb, fc, fd = (ss.func[s][ss.func[s] >= 0] for s in (a, b, c, d))
        bound = np.sqrt(np.einsum("ij,kl->ijkl", diag[np.ix_(fa, fb)], diag[np.ix_(fc, fd)]))
        err = np.abs(e32[x, : len(fa), : len(fb), : len(fc), : len(fd)] - e64[x, : len(fa), : len(fb), : len(fc), : len(fd)])
        ok = bound > 1e-30
        if ok.any():
            worst = max(worst, float((err[ok] / bound[ok]).max()))
        assert np.all(err[~ok] < 1e-30)
    print(f"max |ERI_fp32 - ERI_fp64| / Schwarz bound = {worst:.3e}")
    assert worst < KAPPA, worst
