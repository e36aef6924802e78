"""ctypes binding of ``libmmdg.so`` (include/mmdg.h) and the per-basis device context.

The GPU path has no CPU fallback: if the library is missing or no CUDA device is
visible, every call raises ``MMDGError``.  Device buffers are torch tensors (torch
is used for device memory and streams only); their ``data_ptr()`` crosses the C ABI.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libmmdg.so")
NCLASS = 21
NCOUNT = 5  # per-class counters of a Fock build (mmdg_fock)
DEFAULT_STREAMS_SINGLE = 4
MAX_COMP = 6
LMAX = 2

_lib = None
_lock = threading.Lock()


class MMDGError(RuntimeError):
    pass


def _bind(L):
    c_int, c_ll, c_d, p = ctypes.c_int, ctypes.c_longlong, ctypes.c_double, ctypes.c_void_p
    sig = {
        "mmdg_last_error": (ctypes.c_char_p, []),
        "mmdg_create": (c_int, [ctypes.POINTER(p), c_int]),
        "mmdg_destroy": (c_int, [p]),
        "mmdg_set_basis": (c_int, [p, c_int, p, c_int, p, p, p, p, p, p, p]),
        "mmdg_get_screen": (c_int, [p, p, c_ll]),
        "mmdg_set_screen": (c_int, [p, p, c_ll]),
        "mmdg_eri_tensor": (c_int, [p, p, p]),
        "mmdg_fock": (c_int, [p, p, p, c_d, c_d, p, p]),
        "mmdg_fock_timed": (c_int, [p, p, p, c_d, c_d, p, p, p]),
        "mmdg_measure_peaks": (c_int, [p, p, p]),
        "mmdg_boys": (c_int, [p, c_int, c_ll, p, p, p]),
        "mmdg_fock_update": (c_int, [p, p, p, p, p]),
        "mmdg_jk_dense": (c_int, [p, c_ll, p, p, p, p, p]),
        "mmdg_one_electron": (c_int, [p, c_int, p, p, p, p, p, p, p, p, p]),
        "mmdg_set_tuning": (c_int, [p, c_int, c_int]),
        "mmdg_set_streams": (c_int, [p, c_int]),
        "mmdg_set_tile": (c_int, [p, c_int, c_int, c_int]),
        "mmdg_set_prim_tol": (c_int, [p, ctypes.c_double]),
        "mmdg_rhf_gradient": (c_int, [p, p, p, c_int, p, p, p, c_d, p, p]),
        "mmdg_fock_graph": (c_int, [p, p, p, c_d, c_d, p]),
        "mmdg_eri_quartets": (c_int, [p, c_ll, p, p, c_int, p]),
        "mmdg_set_partition": (c_int, [p, c_int, c_int, p, c_ll]),
        "mmdg_device_bytes": (c_int, [p, ctypes.POINTER(c_ll)]),
        "mmdg_ao2mo": (c_int, [c_ll, p, p, p, p, p]),
        "mmdg_rsqrt": (c_int, [p, c_ll, p, p, p, p]),
        "mmdg_measure_fp64_pipes": (c_int, [p, c_int, p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


def lib():
    """Load libmmdg.so (build it with ``mcmurchie-davidson_gb300/build.py`` first)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise MMDGError(f"{LIB_PATH} not built: run mcmurchie-davidson_gb300/build.py "
                                "(the GPU path has no CPU fallback)")
            _lib = _bind(ctypes.CDLL(LIB_PATH))
    return _lib


def check(rc: int, what: str = "") -> None:
    if rc != 0:
        msg = lib().mmdg_last_error().decode(errors="replace")
        raise MMDGError(f"{what} failed ({rc}): {msg}")


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise MMDGError("no CUDA device visible: the two-electron path runs only on the GPU")
    return torch


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


def stream_ptr(stream=None):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


class Context:
    """One device context holding the primitive-pair data of a basis (one or many molecules).

    ``shells`` is a ``ShellSet`` (``mmd.integrals.shells``) or a list of them (a
    batch of molecules)."""

    def __init__(self, shells, device: int | None = None, prim_tol: float | None = None):
        torch = _torch()
        self.torch = torch
        self.device = torch.cuda.current_device() if device is None else int(device)
        h = ctypes.c_void_p()
        check(lib().mmdg_create(ctypes.byref(h), self.device), "mmdg_create")
        self._h = h
        sets = shells if isinstance(shells, (list, tuple)) else [shells]
        self.sets = list(sets)
        self.nmol = len(sets)
        self.nfunc = np.array([s.nfunc for s in sets], dtype=np.int32)
        mol = np.concatenate([np.full(s.nshell, m, dtype=np.int32) for m, s in enumerate(sets)])
        L = np.concatenate([s.L for s in sets]).astype(np.int32)
        K = np.concatenate([s.nprim for s in sets]).astype(np.int32)
        cen = np.ascontiguousarray(np.concatenate([s.center for s in sets]), dtype=np.float64)
        ex = np.ascontiguousarray(np.concatenate([s.exps for s in sets]), dtype=np.float64)
        co = np.ascontiguousarray(np.concatenate([s.coefs for s in sets]), dtype=np.float64)
        fn = np.ascontiguousarray(np.concatenate([s.func for s in sets]), dtype=np.int32)
        self.nshell = len(L)
        self._keep = (mol, L, K, cen, ex, co, fn)
        if prim_tol is not None:  # primitive-pair screening (default 1e-18; 0 keeps every pair)
            check(lib().mmdg_set_prim_tol(h, float(prim_tol)), "mmdg_set_prim_tol")
        with torch.cuda.device(self.device):
            check(lib().mmdg_set_basis(h, self.nmol, _ptr(self.nfunc), self.nshell, _ptr(mol), _ptr(L), _ptr(K),
                                       _ptr(cen), _ptr(ex), _ptr(co), _ptr(fn)), "mmdg_set_basis")
        if self.nmol == 1:
            # one molecule: the class kernels of a Fock build run on four concurrent
            # streams (the autotuner's choice on (H2O)16 / 6-31G**: 52.7 against 62.1 ms
            # per build in FP64, 31.4 against 43.5 ms mixed); batched contexts keep one
            check(lib().mmdg_set_streams(h, DEFAULT_STREAMS_SINGLE), "mmdg_set_streams")
        self.nn = int(np.sum(self.nfunc.astype(np.int64) ** 2))
        self.ntri = int(np.sum(self.nfunc.astype(np.int64) * (self.nfunc + 1) // 2))
        self.base = np.concatenate([[0], np.cumsum(self.nfunc.astype(np.int64) ** 2)[:-1]])
        self.tbase = np.concatenate([[0], np.cumsum(self.nfunc.astype(np.int64) * (self.nfunc + 1) // 2)[:-1]])
        self.last_counts = None
        self.nparts = 1  # sharded Fock builds (set_partition)

    def close(self):
        if getattr(self, "_h", None):
            lib().mmdg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -------------------------------------------------------------- Schwarz table
    def screen(self) -> np.ndarray:
        out = np.zeros(self.ntri)
        check(lib().mmdg_get_screen(self._h, _ptr(out), self.ntri), "mmdg_get_screen")
        return out

    def set_screen(self, screen: np.ndarray) -> None:
        s = np.ascontiguousarray(screen, dtype=np.float64)
        if s.size != self.ntri:
            raise ValueError("screen table has the wrong length")
        check(lib().mmdg_set_screen(self._h, _ptr(s), self.ntri), "mmdg_set_screen")

    # -------------------------------------------------------------- integrals
    def eri_tensor(self, out=None):
        torch = self.torch
        if self.nmol != 1:
            raise MMDGError("eri_tensor is defined for a single molecule")
        N = int(self.nfunc[0])
        if out is None:
            out = torch.empty((N, N, N, N), dtype=torch.float64, device=f"cuda:{self.device}")
        check(lib().mmdg_eri_tensor(self._h, ctypes.c_void_p(out.data_ptr()), stream_ptr()), "mmdg_eri_tensor")
        return out

    def eri_quartets(self, shells, out=None, fp32: bool = False):
        """All component ERIs of listed shell quartets: ``shells`` is an (n, 4) array of
        global shell indices (a, b, c, d); returns a device tensor (n, 6, 6, 6, 6) with
        (ab|cd) for components [ca, cb, cc, cd] in the caller's shell order (entries
        beyond a shell's components are zero).  ``fp32``: the FP32 class code of the
        mixed-precision path instead of the FP64 one."""
        torch = self.torch
        q = np.ascontiguousarray(shells, dtype=np.int32).reshape(-1, 4)
        n = q.shape[0]
        if out is None:
            out = torch.empty((n, MAX_COMP, MAX_COMP, MAX_COMP, MAX_COMP), dtype=torch.float64,
                              device=f"cuda:{self.device}")
        check(lib().mmdg_eri_quartets(self._h, n, _ptr(q), ctypes.c_void_p(out.data_ptr()), 1 if fp32 else 0,
                                      stream_ptr()), "mmdg_eri_quartets")
        return out

    def function_quartets(self, idx, mol: int = 0):
        """ERIs (ij|kl) of listed function quartets of molecule ``mol`` (an (n, 4) array
        of molecule-local function indices), as a host array of n values."""
        idx = np.asarray(idx, dtype=np.int64).reshape(-1, 4)
        ss = self.sets[mol]
        base = sum(s.nshell for s in self.sets[:mol])
        fshell = np.full(ss.nfunc, -1, dtype=np.int64)
        fcomp = np.zeros(ss.nfunc, dtype=np.int64)
        for s, row in enumerate(ss.func):
            for c, f in enumerate(row):
                if f >= 0:
                    fshell[f], fcomp[f] = s, c
        sh = fshell[idx]
        uq, inv = np.unique(sh, axis=0, return_inverse=True)
        blocks = self.eri_quartets(uq + base).cpu().numpy()
        inv = inv.reshape(-1)
        c = fcomp[idx]
        return blocks[inv, c[:, 0], c[:, 1], c[:, 2], c[:, 3]]

    def set_partition(self, part: int, nparts: int, owner=None):
        """Shard later Fock builds: only the shell quartets of ``part`` (owner per
        canonical shell pair, ``mmd.distributed.canonical_pairs`` order); nparts = 1
        switches sharding off."""
        if int(nparts) == 1:
            check(lib().mmdg_set_partition(self._h, 0, 1, None, 0), "mmdg_set_partition")
            self.nparts = 1
            return
        o = np.ascontiguousarray(owner, dtype=np.int32)
        check(lib().mmdg_set_partition(self._h, int(part), int(nparts), _ptr(o), o.size), "mmdg_set_partition")
        self.nparts = int(nparts)

    def device_bytes(self) -> int:
        """Device memory held by this context (quartet lists included once allocated)."""
        if not getattr(self, "_h", None):
            return 0
        b = ctypes.c_longlong()
        check(lib().mmdg_device_bytes(self._h, ctypes.byref(b)), "mmdg_device_bytes")
        return int(b.value)

    def fock(self, dP, G=None, tol: float = 1e-12, fp32_below: float = 0.0, counts: bool = False):
        """Unsymmetrised G(dP) (formPT semantics); dP/G are packed device float64 tensors."""
        torch = self.torch
        if dP.dtype != torch.float64 or not dP.is_cuda or not dP.is_contiguous() or dP.numel() != self.nn:
            raise ValueError("dP must be a contiguous CUDA float64 tensor of sum N_m^2 elements")
        if G is None:
            G = torch.empty_like(dP)
        cnt = np.zeros(NCOUNT * NCLASS, dtype=np.uint64) if counts else None
        check(lib().mmdg_fock(self._h, ctypes.c_void_p(dP.data_ptr()), ctypes.c_void_p(G.data_ptr()), float(tol),
                              float(fp32_below), _ptr(cnt) if counts else None, stream_ptr()), "mmdg_fock")
        if counts:
            self.last_counts = cnt.reshape(NCLASS, NCOUNT)
        return G

    def fock_timed(self, dP, G=None, tol: float = 1e-12, fp32_below: float = 0.0):
        """As ``fock`` with per-class device times (ms) and counts: returns (G, class_ms, counts)."""
        if G is None:
            G = self.torch.empty_like(dP)
        cnt = np.zeros(NCOUNT * NCLASS, dtype=np.uint64)
        ms = np.zeros(NCLASS, dtype=np.float32)
        check(lib().mmdg_fock_timed(self._h, ctypes.c_void_p(dP.data_ptr()), ctypes.c_void_p(G.data_ptr()),
                                    float(tol), float(fp32_below), _ptr(cnt), _ptr(ms), stream_ptr()),
              "mmdg_fock_timed")
        self.last_counts = cnt.reshape(NCLASS, NCOUNT)
        return G, ms, self.last_counts

    def fock_update(self, G, F_in, F_out):
        check(lib().mmdg_fock_update(self._h, ctypes.c_void_p(G.data_ptr()), ctypes.c_void_p(F_in.data_ptr()),
                                     ctypes.c_void_p(F_out.data_ptr()), stream_ptr()), "mmdg_fock_update")
        return F_out

    def jk_dense(self, T, P, J, K):
        N = P.shape[-1]
        check(lib().mmdg_jk_dense(self._h, N, ctypes.c_void_p(T.data_ptr()), ctypes.c_void_p(P.data_ptr()),
                                  ctypes.c_void_p(J.data_ptr()), ctypes.c_void_p(K.data_ptr()), stream_ptr()),
              "mmdg_jk_dense")
        return J, K

    def boys(self, m: int, T):
        out = self.torch.empty_like(T)
        check(lib().mmdg_boys(self._h, int(m), T.numel(), ctypes.c_void_p(T.data_ptr()),
                              ctypes.c_void_p(out.data_ptr()), stream_ptr()), "mmdg_boys")
        return out


def measure_peaks(ctx) -> tuple[float, float]:
    """(FP64, FP32) TFLOP/s of the current GPU (independent FMA chains)."""
    a = ctypes.c_double()
    b = ctypes.c_double()
    check(lib().mmdg_measure_peaks(ctx._h, ctypes.byref(a), ctypes.byref(b)), "mmdg_measure_peaks")
    return a.value, b.value


def measure_fp64_pipes(ctx, warps_per_sm: int = 16) -> dict:
    """DFMA and FP64 tensor-core (DMMA) throughput and whether they overlap
    (mmdg_measure_fp64_pipes)."""
    r = np.zeros(5)
    check(lib().mmdg_measure_fp64_pipes(ctx._h, int(warps_per_sm), _ptr(r)), "mmdg_measure_fp64_pipes")
    return {"warps_per_sm": int(warps_per_sm), "dfma_tflops": float(r[0]), "dmma_tflops": float(r[1]),
            "dfma_ms": float(r[2]), "dmma_ms": float(r[3]), "both_ms": float(r[4]),
            "both_over_sum": float(r[4] / (r[2] + r[3])), "both_over_max": float(r[4] / max(r[2], r[3]))}


_default_ctx = None


def scratch_context():
    """A context without basis (for mmdg_boys / mmdg_jk_dense)."""
    global _default_ctx
    torch = _torch()
    if _default_ctx is None:
        class _Bare:
            pass
        b = _Bare()
        h = ctypes.c_void_p()
        check(lib().mmdg_create(ctypes.byref(h), torch.cuda.current_device()), "mmdg_create")
        b._h = h
        b.torch = torch
        b.boys = lambda m, T: Context.boys(b, m, T)
        b.jk_dense = lambda T, P, J, K: Context.jk_dense(b, T, P, J, K)
        _default_ctx = b
    return _default_ctx


def ao2mo(C, eri, out=None, work=None):
    """(PQ|RS) = sum C[p,P] C[q,Q] C[r,R] C[s,S] (pq|rs) on the device (mmdg_ao2mo):
    ``C`` (N x N) and ``eri`` (N^4) are CUDA float64 tensors; returns ``out``."""
    torch = _torch()
    N = int(C.shape[0])
    if C.dtype != torch.float64 or eri.dtype != torch.float64 or eri.numel() != N ** 4:
        raise ValueError("ao2mo: float64 C (N x N) and ERI tensor (N^4) expected")
    C = C.contiguous()
    eri = eri.contiguous()
    out = torch.empty_like(eri) if out is None else out
    work = torch.empty_like(eri) if work is None else work
    check(lib().mmdg_ao2mo(N, ctypes.c_void_p(C.data_ptr()), ctypes.c_void_p(eri.data_ptr()),
                           ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(work.data_ptr()), stream_ptr()),
          "mmdg_ao2mo")
    return out
