"""Learned initial density guess for RHF on water clusters in 6-31G.

The reference starts every SCF from P = 0, i.e. F = Core (mmd/scf.py:15,23-24).
Here a small network predicts the converged density matrix block by block from
atom-pair features, and ``Molecule.RHF(guess=P)`` starts from it (one full Fock
build of the guess), falling back to the core guess if the DIIS error grows for
three consecutive iterations.

Features of an ordered atom pair (A, B), A <= B, within 8 Angstrom (53 numbers):

* pair type one-hot (6): O-O, O-H, H-O, H-H, O self block, H self block;
* the distance expanded on 32 Gaussians centred 0.5 .. 8 Angstrom (width 0.24 A);
* the direction of B in A's local frame and of A in B's (3 + 3);
* the rotation between the two local frames, R_A R_B^T (9).

An atom's local frame is built from its two nearest atoms (first axis to the
nearest, second from the next one, third their cross product), so features and
predictions rotate with the molecule.  The target is the density block in the two
local frames, T_A P[A,B] T_B^T, where T rotates the p triplets and leaves s
functions alone; it is padded to 9 x 9 (O has 9 functions in 6-31G, H has 2) with
a mask.

The network: 53 -> 256 -> 256 -> 81, SiLU, BF16 weights with FP32 accumulation,
trained with Adam on the GPU by the kernels of csrc/mlp.cu (``mmdg_mlp_*``).

The same construction covers 6-31G** (``B631GSS``: O has 15 functions with the d
sextet, H has 5 with a p triplet; blocks padded to 15 x 15, 225 outputs).  Cartesian
d functions rotate as quadratic monomials (``d_transform``), a non-orthogonal
transform, so a block goes to the local frames as T_A^-T P[A,B] T_B^-1 and back as
T_A^T P' T_B.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _native

ANG = 0.52917721092
NIN, NHID, NOUT = 53, 256, 81
NFUNC = {8: 9, 1: 2}           # 6-31G Cartesian functions per element
PTRIPLETS = {8: (2, 6), 1: ()}  # first index of each p triplet in the atom's functions
TYPES = {(8, 8): 0, (8, 1): 1, (1, 8): 2, (1, 1): 3}
RBF_CENTERS = np.linspace(0.5, 8.0, 32) / ANG
RBF_WIDTH = 0.24 / ANG
CUTOFF = 8.0 / ANG
DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")
WEIGHTS = os.path.join(DATA, "guess_mlp_631g.npz")


class GuessBasis:
    """Function layout a network predicts: the shells of each element in basis order
    ('S', 'P', 'D'), the block padding and the weights file."""

    def __init__(self, name, shells, weights):
        self.name = name
        self.shells = shells
        self.nfunc = {z: sum({"S": 1, "P": 3, "D": 6}[c] for c in sh) for z, sh in shells.items()}
        self.nmax = max(self.nfunc.values())
        self.nout = self.nmax * self.nmax
        self.weights = weights
        self.has_d = any("D" in sh for sh in shells.values())


B631G = GuessBasis("6-31g", {8: "SSPSP", 1: "SS"}, WEIGHTS)
B631GSS = GuessBasis("6-31gss", {8: "SSPSPD", 1: "SSP"}, os.path.join(DATA, "guess_mlp_631gss.npz"))
BASES = {"6-31g": B631G, "6-31gss": B631GSS}


# ---------------------------------------------------------------- geometry
def atom_frames(coords: np.ndarray) -> np.ndarray:
    n = len(coords)
    R = np.tile(np.eye(3), (n, 1, 1))
    if n < 2:
        return R
    d = np.linalg.norm(coords[:, None] - coords[None], axis=-1)
    d[np.diag_indices(n)] = np.inf
    order = np.argsort(d, axis=1)
    for a in range(n):
        e1 = coords[order[a, 0]] - coords[a]
        e1 /= np.linalg.norm(e1)
        if n > 2:
            v = coords[order[a, 1]] - coords[a]
        else:
            v = np.array([0.0, 0.0, 1.0]) if abs(e1[2]) < 0.9 else np.array([1.0, 0.0, 0.0])
        e2 = v - np.dot(v, e1) * e1
        nr = np.linalg.norm(e2)
        if nr < 1e-8:
            v = np.array([0.0, 0.0, 1.0]) if abs(e1[2]) < 0.9 else np.array([1.0, 0.0, 0.0])
            e2 = v - np.dot(v, e1) * e1
            nr = np.linalg.norm(e2)
        e2 /= nr
        R[a] = np.stack([e1, e2, np.cross(e1, e2)])
    return R


_DPAIRS = ((0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2))  # xx xy xz yy yz zz
_DNORM = np.array([1.0 / np.sqrt(3.0), 1.0, 1.0, 1.0 / np.sqrt(3.0), 1.0, 1.0 / np.sqrt(3.0)])


def d_transform(R: np.ndarray) -> np.ndarray:
    """Cartesian d functions n_ab x_a x_b in the frame x' = R x: phi' = T phi with
    T[ab, kl] = n_ab / n_kl (R_ak R_bl + R_al R_bk) (k < l) or n_ab / n_kk R_ak R_bk."""
    T = np.zeros((6, 6))
    for i, (a, b) in enumerate(_DPAIRS):
        for j, (k, l) in enumerate(_DPAIRS):
            c = R[a, k] * R[b, l] + (R[a, l] * R[b, k] if k != l else 0.0)
            T[i, j] = _DNORM[i] / _DNORM[j] * c
    return T


def block_transform(Z: int, R: np.ndarray, gb: GuessBasis = B631G) -> np.ndarray:
    """Functions of an atom in its local frame, phi' = T phi (s unchanged, p triplets
    rotated by R, d sextets by d_transform)."""
    T = np.eye(gb.nfunc[Z])
    o = 0
    for c in gb.shells[Z]:
        if c == "P":
            T[o:o + 3, o:o + 3] = R
        elif c == "D":
            T[o:o + 6, o:o + 6] = d_transform(R)
        o += {"S": 1, "P": 3, "D": 6}[c]
    return T


def _to_local(T):
    """Density-block transform to the local functions: P' = T^-T P T^-1 (= T P T^T for
    the orthogonal s/p transform)."""
    return np.linalg.inv(T).T


def molecule_layout(mol, gb: GuessBasis = B631G):
    """Atomic numbers, coordinates (bohr) and first-function offsets of a Molecule."""
    Z = np.array([a.charge for a in mol.atoms])
    X = np.array([a.origin for a in mol.atoms])
    if any(int(z) not in gb.nfunc for z in Z):
        raise ValueError(f"the learned guess covers H and O in {gb.name} only")
    off = np.concatenate([[0], np.cumsum([gb.nfunc[int(z)] for z in Z])[:-1]])
    if off[-1] + gb.nfunc[int(Z[-1])] != mol.nbasis:
        raise ValueError(f"the learned guess covers H and O in {gb.name} only")
    return Z, X, off


def pair_features(Z, X, R):
    """Ordered pairs (A <= B) within the cutoff and their feature rows: element-pair
    one-hot (or the element of a diagonal block), the distance on 32 Gaussians, the
    bond direction in each atom's local frame, and the relative frame orientation."""
    n = len(Z)
    Z = np.asarray(Z).astype(int)
    ia, ib = np.triu_indices(n)                       # a <= b, row-major: (0,0), (0,1), ...
    v = X[ib] - X[ia]
    d = np.linalg.norm(v, axis=1)
    keep = d <= CUTOFF
    ia, ib, v, d = ia[keep], ib[keep], v[keep], d[keep]
    diag = ia == ib
    F = np.zeros((len(ia), NIN))
    rows = np.arange(len(ia))
    tcol = np.array([TYPES[(int(za), int(zb))] for za, zb in zip(Z[ia], Z[ib])], dtype=int) if len(ia) else \
        np.zeros(0, dtype=int)
    dcol = np.where(Z[ia] == 8, 4, 5)
    F[rows, np.where(diag, dcol, tcol)] = 1.0
    off = ~diag
    u = np.zeros_like(v)
    u[off] = v[off] / d[off, None]
    F[off, 38:41] = np.einsum("pij,pj->pi", R[ia[off]], u[off])
    F[off, 41:44] = np.einsum("pij,pj->pi", R[ib[off]], -u[off])
    F[:, 6:38] = np.exp(-((d[:, None] - RBF_CENTERS[None, :]) / RBF_WIDTH) ** 2)
    F[:, 44:53] = np.einsum("pik,pjk->pij", R[ia], R[ib]).reshape(-1, 9)
    pairs = list(zip(ia.tolist(), ib.tolist()))
    return pairs, F.astype(np.float32)


def _atom_transforms(Z, R, gb: GuessBasis, local: bool = False):
    """block_transform of every atom (its inverse transpose with ``local`` for a basis
    with d functions), computed once per atom rather than once per pair."""
    T = [block_transform(int(z), r, gb) for z, r in zip(Z, R)]
    if local and gb.has_d:
        T = [_to_local(t) for t in T]
    return T


def pair_targets(P, Z, R, off, pairs, gb: GuessBasis = B631G):
    nm = gb.nmax
    Y = np.zeros((len(pairs), gb.nout), dtype=np.float32)
    M = np.zeros((len(pairs), gb.nout), dtype=np.float32)
    T = _atom_transforms(Z, R, gb, local=True)
    for k, (a, b) in enumerate(pairs):
        na, nb = gb.nfunc[int(Z[a])], gb.nfunc[int(Z[b])]
        blk = P[off[a]:off[a] + na, off[b]:off[b] + nb]
        loc = T[a] @ blk @ T[b].T
        t = np.zeros((nm, nm))
        m = np.zeros((nm, nm))
        t[:na, :nb] = loc
        m[:na, :nb] = 1.0
        Y[k] = t.ravel()
        M[k] = m.ravel()
    return Y, M


def assemble(pred, Z, R, off, pairs, N, gb: GuessBasis = B631G):
    """Lab-frame density from the predicted local-frame blocks: P[A,B] = T_A^T P' T_B
    (diagonal blocks symmetrised, P[B,A] = P[A,B]^T)."""
    nm = gb.nmax
    P = np.zeros((N, N))
    T = _atom_transforms(Z, R, gb)
    for k, (a, b) in enumerate(pairs):
        na, nb = gb.nfunc[int(Z[a])], gb.nfunc[int(Z[b])]
        loc = pred[k].reshape(nm, nm)[:na, :nb]
        blk = T[a].T @ loc @ T[b]
        if a == b:
            blk = 0.5 * (blk + blk.T)
        P[off[a]:off[a] + na, off[b]:off[b] + nb] = blk
        if a != b:
            P[off[b]:off[b] + nb, off[a]:off[a] + na] = blk.T
    return P


def molecule_samples(mol, P=None, gb: GuessBasis = B631G):
    Z, X, off = molecule_layout(mol, gb)
    R = atom_frames(X)
    pairs, F = pair_features(Z, X, R)
    if P is None:
        return pairs, F, None, None, (Z, R, off)
    Y, M = pair_targets(np.asarray(P), Z, R, off, pairs, gb)
    return pairs, F, Y, M, (Z, R, off)


# ---------------------------------------------------------------- the network
class DensityMLP:
    """53 -> 256 -> 256 -> 81 MLP; FP32 master weights, BF16 copies used by the kernels."""

    def __init__(self, seed=0, weights=None, gb: GuessBasis = B631G):
        torch = _native._torch()
        self.torch = torch
        self.dev = "cuda"
        self.gb = gb
        L = _native.lib()
        self._sig(L)
        rng = np.random.default_rng(seed)
        shapes = [(NHID, NIN), (NHID, NHID), (gb.nout, NHID)]
        if weights is None:
            W = [rng.standard_normal(s) * np.sqrt(1.0 / s[1]) for s in shapes]
            b = [np.zeros(s[0]) for s in shapes]
        else:
            W = [weights[f"W{i}"] for i in range(3)]
            b = [weights[f"b{i}"] for i in range(3)]
        f32 = lambda a: torch.tensor(np.asarray(a, dtype=np.float32), device=self.dev)
        self.W = [f32(w).contiguous() for w in W]
        self.b = [f32(x).contiguous() for x in b]
        self.Wb = [torch.empty(w.shape, dtype=torch.bfloat16, device=self.dev) for w in self.W]
        for w, wb in zip(self.W, self.Wb):
            _native.check(L.mmdg_mlp_to_bf16(self._p(w), self._p(wb), w.numel(), _native.stream_ptr()), "to_bf16")
        self.mW = [torch.zeros_like(w) for w in self.W]
        self.vW = [torch.zeros_like(w) for w in self.W]
        self.mb = [torch.zeros_like(x) for x in self.b]
        self.vb = [torch.zeros_like(x) for x in self.b]
        self.step = 0

    @staticmethod
    def _sig(L):
        p, c_int, c_ll, c_f = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_float
        for name, args in {
            "mmdg_mlp_gemm": [c_int, c_int, c_int, p, c_int, c_int, c_int, p, c_int, c_int, c_int, p, c_int, c_f, p],
            "mmdg_mlp_bias_act": [p, p, p, c_ll, c_int, c_int, p],
            "mmdg_mlp_act_grad": [p, p, p, c_ll, c_int, p],
            "mmdg_mlp_colsum": [p, p, c_ll, c_int, p],
            "mmdg_mlp_mse": [p, p, p, p, p, c_ll, c_f, p],
            "mmdg_mlp_adam": [p, p, p, p, p, c_ll, c_f, c_f, c_f, c_f, c_int, p],
            "mmdg_mlp_to_bf16": [p, p, c_ll, p],
        }.items():
            fn = getattr(L, name)
            fn.restype = ctypes.c_int
            fn.argtypes = args

    @staticmethod
    def _p(t):
        return ctypes.c_void_p(t.data_ptr())

    def forward(self, X):
        """X: (B, 53) float32 CUDA tensor -> list of (Z, Y) per layer (Y of the last = output)."""
        torch, L, st = self.torch, _native.lib(), _native.stream_ptr()
        acts = []
        h = X
        for i in range(3):
            out = self.W[i].shape[0]
            Zt = torch.empty((h.shape[0], out), dtype=torch.float32, device=self.dev)
            _native.check(L.mmdg_mlp_gemm(h.shape[0], out, h.shape[1], self._p(h), h.shape[1], 0, 0,
                                          self._p(self.Wb[i]), h.shape[1], 1, 1, self._p(Zt), out, 0.0, st), "gemm")
            Yt = torch.empty_like(Zt)
            _native.check(L.mmdg_mlp_bias_act(self._p(Zt), self._p(Yt), self._p(self.b[i]), h.shape[0], out,
                                              1 if i < 2 else 0, st), "bias_act")
            acts.append((h, Zt, Yt))
            h = Yt
        return acts

    def predict(self, X):
        return self.forward(X)[-1][2]

    def backward(self, acts, dY):
        """Gradients (dW, db) of every layer from the output gradient dY."""
        torch, L, st = self.torch, _native.lib(), _native.stream_ptr()
        grads = [None] * 3
        d = dY
        for i in (2, 1, 0):
            h, Zt, _ = acts[i]
            out, inp = self.W[i].shape
            dZ = torch.empty_like(Zt)
            _native.check(L.mmdg_mlp_act_grad(self._p(Zt), self._p(d), self._p(dZ), dZ.numel(), 1 if i < 2 else 0, st),
                          "act_grad")
            dW = torch.empty((out, inp), dtype=torch.float32, device=self.dev)
            _native.check(L.mmdg_mlp_gemm(out, inp, h.shape[0], self._p(dZ), out, 1, 0, self._p(h), inp, 0, 0,
                                          self._p(dW), inp, 0.0, st), "gemm dW")
            db = torch.empty(out, dtype=torch.float32, device=self.dev)
            _native.check(L.mmdg_mlp_colsum(self._p(dZ), self._p(db), h.shape[0], out, st), "colsum")
            grads[i] = (dW, db)
            if i > 0:
                dh = torch.empty((h.shape[0], inp), dtype=torch.float32, device=self.dev)
                _native.check(L.mmdg_mlp_gemm(h.shape[0], inp, out, self._p(dZ), out, 0, 0, self._p(self.Wb[i]), inp,
                                              0, 1, self._p(dh), inp, 0.0, st), "gemm dX")
                d = dh
        return grads

    def loss_grad(self, Y, T, M):
        torch, L, st = self.torch, _native.lib(), _native.stream_ptr()
        dY = torch.empty_like(Y)
        loss = torch.zeros(1, dtype=torch.float64, device=self.dev)
        cnt = float(max(M.sum().item(), 1.0))
        _native.check(L.mmdg_mlp_mse(self._p(Y), self._p(T), self._p(M), self._p(dY), self._p(loss), Y.numel(),
                                     1.0 / cnt, st), "mse")
        return loss, dY

    def adam(self, grads, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        L, st = _native.lib(), _native.stream_ptr()
        self.step += 1
        for i, (dW, db) in enumerate(grads):
            _native.check(L.mmdg_mlp_adam(self._p(self.W[i]), self._p(self.Wb[i]), self._p(dW), self._p(self.mW[i]),
                                          self._p(self.vW[i]), dW.numel(), lr, b1, b2, eps, self.step, st), "adam W")
            _native.check(L.mmdg_mlp_adam(self._p(self.b[i]), None, self._p(db), self._p(self.mb[i]),
                                          self._p(self.vb[i]), db.numel(), lr, b1, b2, eps, self.step, st), "adam b")

    def state(self):
        out = {}
        for i in range(3):
            out[f"W{i}"] = self.W[i].cpu().numpy()
            out[f"b{i}"] = self.b[i].cpu().numpy()
        return out

    def save(self, path=None):
        path = path or self.gb.weights
        os.makedirs(os.path.dirname(path), exist_ok=True)
        np.savez_compressed(path, **self.state())

    @classmethod
    def load(cls, path=WEIGHTS):
        w = dict(np.load(path))
        nout = w["W2"].shape[0]
        gb = next(b for b in BASES.values() if b.nout == nout)
        return cls(weights=w, gb=gb)


def train(features, targets, masks, epochs=30, batch=8192, lr=2e-3, seed=0, log=None, gb: GuessBasis = B631G):
    """Adam on masked MSE; features/targets/masks are float32 arrays (rows = pairs)."""
    net = DensityMLP(seed=seed, gb=gb)
    torch = net.torch
    Xd = torch.tensor(features, device="cuda")
    Yd = torch.tensor(targets, device="cuda")
    Md = torch.tensor(masks, device="cuda")
    n = Xd.shape[0]
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    history = []
    for ep in range(epochs):
        perm = torch.randperm(n, device="cuda", generator=g)
        lr_ep = lr * 0.5 * (1 + np.cos(np.pi * ep / epochs))
        tot = 0.0
        for s in range(0, n, batch):
            idx = perm[s:s + batch]
            X, T, M = Xd[idx].contiguous(), Yd[idx].contiguous(), Md[idx].contiguous()
            acts = net.forward(X)
            loss, dY = net.loss_grad(acts[-1][2], T, M)
            net.adam(net.backward(acts, dY), lr=lr_ep)
            tot += float(loss.item()) * X.shape[0]
        history.append(tot / n)
        if log:
            log(f"epoch {ep}: loss {tot / n:.3e}")
    net.history = history
    return net


def predict_density(net, mol):
    """Initial density of ``mol``.  A 6-31G molecule is predicted directly; a basis
    that contains 6-31G (6-31G*, 6-31G**: the same s and p functions first on every
    atom, polarisation functions after them) gets the 6-31G prediction embedded, zero
    on the polarisation functions.  The embedded matrix is a valid density of the
    larger basis (P S P = P and tr(P S) = N/2 hold on the shared functions)."""
    gb = getattr(net, "gb", B631G)
    try:
        molecule_layout(mol, gb)
    except ValueError:
        if gb is not B631G:
            raise
        return _embedded_prediction(net, mol)
    pairs, F, _, _, (Z, R, off) = molecule_samples(mol, None, gb)
    pred = net.predict(net.torch.tensor(F, device="cuda")).cpu().numpy()
    return assemble(pred, Z, R, off, pairs, mol.nbasis, gb)


def network_for(mol):
    """The committed network that covers ``mol``'s basis: its own if trained (6-31G,
    6-31G**), else the 6-31G one (embedded in a 6-31G superset)."""
    for gb in (B631GSS, B631G):
        if os.path.exists(gb.weights):
            try:
                molecule_layout(mol, gb)
            except ValueError:
                continue
            return DensityMLP.load(gb.weights)
    return DensityMLP.load(WEIGHTS)


def _embedded_prediction(net, mol):
    from .molecule import Molecule
    small = Molecule(mol.geometry_input, "6-31g")
    return embed_density(small, mol, predict_density(net, small))


def embed_density(small, mol, Ps):
    """Ps of the 6-31G molecule ``small`` placed on the matching functions of ``mol``
    (same geometry, a basis whose first functions on every atom are 6-31G's)."""
    big_of_atom, small_of_atom = {}, {}
    for k, a in enumerate(mol.bf_atom):
        big_of_atom.setdefault(a, []).append(k)
    for k, a in enumerate(small.bf_atom):
        small_of_atom.setdefault(a, []).append(k)
    idx = np.empty(small.nbasis, dtype=np.int64)
    for a, ks in small_of_atom.items():
        kb = big_of_atom.get(a, [])[:len(ks)]
        if len(kb) != len(ks):
            raise ValueError("the basis does not contain 6-31G")
        for i, j in zip(ks, kb):
            bs, bb = small.bfs[i], mol.bfs[j]
            if (tuple(np.asarray(bs.shell)) != tuple(np.asarray(bb.shell))
                    or not np.allclose(np.asarray(bs.exps)[:bs.num_exps], np.asarray(bb.exps)[:bb.num_exps])):
                raise ValueError("the basis does not contain 6-31G")
            idx[i] = j
    P = np.zeros((mol.nbasis, mol.nbasis))
    P[np.ix_(idx, idx)] = Ps
    return P
