"""CPU oracle of the post-SCF consumers: MP2, CIS, TDHF (TEST INFRASTRUCTURE ONLY).

A float64 numpy restatement of what the reference computes after a conventional
RHF: the RHF itself (mmd/scf.py:10-80: P = C_occ C_occ^T without the factor 2,
F = H + 2J - K, DIIS on the orthogonalised commutator, stop on ||P - P_old||_F),
the spin-orbital integrals <pq||rs> of ``ao2mo`` (mmd/postscf.py:21-41; spin orbital
2p + sigma), the MP2 correlation energies (mmd/postscf.py:44-73, spatial and
spin-orbital), the CIS matrix A (mmd/postscf.py:249-267) and the three TDHF
eigenproblems (mmd/postscf.py:325-381).  It starts from the one- and two-electron
integrals of the golden fixtures, so it runs without a GPU; the GPU PostSCF is
checked against the reference's own MP2 and excitation energies directly.
"""
import numpy as np
import scipy.linalg

HARTREE_EV = 27.211399  # the reference's conversion factor (mmd/postscf.py:313, 383)


def rhf(S, T, V, TwoE, nocc, conver=1e-12, maxiter=200, ndiis=8):
    """Conventional RHF; returns (C, orbital energies)."""
    H = T + V
    w, U = np.linalg.eigh(S)
    X = (U / np.sqrt(w)) @ U.T
    P = np.zeros_like(S)
    F = H.copy()
    focks, errs = [], []
    for _ in range(maxiter):
        FO = X.T @ F @ X
        e, CO = scipy.linalg.eigh(FO)
        C = X @ CO
        P_new = C[:, :nocc] @ C[:, :nocc].T
        if np.linalg.norm(P_new - P) < conver:
            return C, e
        P = P_new
        J = np.einsum("pqrs,sr->pq", TwoE, P)
        K = np.einsum("psqr,sr->pq", TwoE, P)
        F = H + 2.0 * J - K
        err = X.T @ (F @ P @ S - S @ P @ F) @ X
        focks.append(F)
        errs.append(err)
        focks, errs = focks[-ndiis:], errs[-ndiis:]
        n = len(focks)
        if n > 1:
            B = -np.ones((n + 1, n + 1))
            B[n, n] = 0.0
            for i in range(n):
                for j in range(n):
                    B[i, j] = np.sum(errs[i] * errs[j])
            rhs = np.zeros(n + 1)
            rhs[n] = -1.0
            c = np.linalg.solve(B, rhs)
            F = sum(c[i] * focks[i] for i in range(n))
    raise RuntimeError("RHF not converged")


def spin_integrals(C, TwoE):
    """<pq||rs> over spin orbitals 2p + sigma, from the MO integrals (pq|rs)."""
    mo = np.einsum("pqrs,pP,qQ,rR,sS->PQRS", TwoE, C, C, C, C, optimize=True)
    n = 2 * mo.shape[0]
    sp, sg = np.arange(n) // 2, np.arange(n) % 2
    same = (sg[:, None] == sg[None, :]).astype(float)
    phys = mo[np.ix_(sp, sp, sp, sp)].transpose(0, 2, 1, 3)          # <pq|rs> = (pr|qs) spatially
    coul = phys * same[:, None, :, None] * same[None, :, None, :]
    return coul - coul.transpose(0, 1, 3, 2)


def mp2_spatial(C, e_mo, TwoE, nocc):
    """Sum_ijab (ia|jb) [2 (ia|jb) - (ib|ja)] / (e_i + e_j - e_a - e_b)."""
    mo = np.einsum("pqrs,pP,qQ,rR,sS->PQRS", TwoE, C, C, C, C, optimize=True)
    o, v = slice(0, nocc), slice(nocc, len(e_mo))
    iajb = mo[o, v, o, v]
    d = e_mo[o][:, None, None, None] - e_mo[v][None, :, None, None] + e_mo[o][None, None, :, None] - \
        e_mo[v][None, None, None, :]
    return float(np.sum(iajb * (2.0 * iajb - iajb.transpose(0, 3, 2, 1)) / d))


def mp2_spin(e_mo, dbl, nelec):
    """(1/4) Sum_ijab |<ij||ab>|^2 / (e_i + e_j - e_a - e_b) over spin orbitals."""
    e = np.repeat(e_mo, 2)
    o, v = slice(0, nelec), slice(nelec, len(e))
    d = e[o][:, None, None, None] + e[o][None, :, None, None] - e[v][None, None, :, None] - e[v][None, None, None, :]
    return float(0.25 * np.sum(dbl[o, o, v, v] ** 2 / d))


def singles(e_mo, dbl, nelec):
    """A[ia,jb] = (e_a - e_i) d_ij d_ab + <aj||ib>,  B[ia,jb] = <ab||ij>."""
    e = np.repeat(e_mo, 2)
    n = len(e)
    o, v = slice(0, nelec), slice(nelec, n)
    no, nv = nelec, n - nelec
    A = np.einsum("ajib->iajb", dbl[v, o, o, v]).reshape(no * nv, no * nv)
    A = A + np.diag((e[v][None, :] - e[o][:, None]).reshape(-1))
    B = np.einsum("abij->iajb", dbl[v, v, o, o]).reshape(no * nv, no * nv)
    return A, B


def cis(A):
    """CIS excitation energies (eV)."""
    return scipy.linalg.eigh(A, eigvals_only=True) * HARTREE_EV


def tdhf(A, B, alg="hermitian"):
    """TDHF excitation energies (eV) by the reference's three algorithms."""
    if alg == "hermitian":
        lam, U = np.linalg.eigh(A - B)
        root = (U * np.sqrt(lam)) @ U.T
        w = np.sqrt(scipy.linalg.eigh(root @ (A + B) @ root, eigvals_only=True))
    elif alg == "reduced":
        w = np.sort(np.sqrt(np.linalg.eigvals((A - B) @ (A + B))).real)
    elif alg == "full":
        n = A.shape[0]
        lam = np.linalg.eigvals(np.block([[A, B], [-B.T, -A.T]]))
        w = np.sort(lam.real)[n:]
    else:
        raise ValueError(alg)
    return w * HARTREE_EV
