"""FP64 matrix products from BF16 tensor-core GEMMs by exact operand splitting.

A measurement of the alternative to the FP64 pipe for the d-class Hermite transforms
(the E' x R contraction of cython/twoe.pyx:77-91): every row of A and every column of
B is scaled by a power of two to magnitudes below 1, its 56 leading bits are cut into
seven 8-bit digits (the error-free splitting of T. Ozaki, T. Ogita, S. M. Rump and
S. Oishi, "Error-free transformations of matrix multiplication by using fast routines
of matrix multiplication and its applications", Numer. Algorithms 59, 2012, here with
integer digits), and each digit matrix is an exact BF16 operand (integers 0..255 carry
8 significant bits).  A product of two digit matrices over K <= 256 terms is an integer
below 2^24, so the BF16 tensor-core GEMM with FP32 accumulation and FP32 output returns
it exactly; the FP64 result is the sum of those exact partial products, each scaled by
its power of two.  Of the 49 digit pairs (s, t) the 28 with s + t <= 6 (0-based) are
formed; the dropped ones and the 56-bit truncation of both operands together stay
below K 2^-52 max|A_i.| max|B_.j| per element.

``split_operand_mm`` is the algorithm; ``measure`` times it on the d-class transform
shape against cuBLAS DGEMM and prints one JSON line (``python -m mmd.split_operand``).
It is not on the product path: the ERI kernels keep the FP64 pipe.
"""
from __future__ import annotations

import json

import torch

DIGITS = 7  # 56 bits: the 53-bit significand of the row (column) maximum and 3 guard bits
BASE = 256.0


def pow2(k: torch.Tensor) -> torch.Tensor:
    """2**k as float64, exactly, for integer k in [-1022, 1023] (exponent-field bits)."""
    return ((k.to(torch.int64) + 1023) << 52).view(torch.float64)


def split(X: torch.Tensor, dim: int, digits: int = DIGITS):
    """Digits and scale exponents of a float64 matrix, per row (``dim=1``: the maximum
    over each row) or per column (``dim=0``): X = 2^e * sum_s d_s 256^-(s+1) up to
    2^(e-56), each d_s a BF16 matrix of signed integers with |d_s| <= 255."""
    amax = X.abs().amax(dim=dim, keepdim=True)
    _, e = torch.frexp(amax)  # amax = m 2^e, m in [0.5, 1); 0 -> e = 0
    x = X.abs() * pow2(-e)   # [0, 1), exact
    sign = torch.sign(X)
    out = []
    for _ in range(digits):
        x = x * BASE          # exact
        d = torch.floor(x)
        x = x - d             # exact: the fraction of a double below 2^53
        out.append((sign * d).to(torch.bfloat16))
    return torch.stack(out), e


def tensor_core_mm(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """BF16 x BF16 -> FP32 product on the tensor cores (cuBLAS, FP32 accumulation)."""
    return torch.mm(a, b, out_dtype=torch.float32)


def split_operand_mm(A: torch.Tensor, B: torch.Tensor, mm=tensor_core_mm, digits: int = DIGITS,
                     parts: dict | None = None) -> torch.Tensor:
    """A @ B (float64, K <= 256) from digit products.  The digits of A are stacked into
    one (digits*m, K) operand, so B's digit t costs one GEMM with the ``digits - t``
    leading A digits.  ``mm`` multiplies two BF16 matrices into an exact FP32 result.
    ``parts`` (optional) receives the split, product and sum sub-results for timing."""
    m, K = A.shape
    n = B.shape[1]
    if K > 256:
        raise ValueError("split_operand_mm: K above 256 can round the FP32 digit products")
    Ad, ea = split(A, 1, digits)          # (digits, m, K), (m, 1)
    Bd, eb = split(B, 0, digits)          # (digits, K, n), (1, n)
    # zero digits pad K and n to multiples of 8 (16-byte rows for the tensor-core GEMM)
    Kp, npad = -(-K // 8) * 8, -(-n // 8) * 8
    Ad = torch.nn.functional.pad(Ad, (0, Kp - K))
    Bd = torch.nn.functional.pad(Bd, (0, npad - n, 0, Kp - K))
    A2 = Ad.reshape(digits * m, Kp)
    C = torch.zeros(m, n, dtype=torch.float64, device=A.device)
    # smallest terms first: t descending, then s descending inside each product
    for t in range(digits - 1, -1, -1):
        ns = digits - t
        P = mm(A2[: ns * m], Bd[t]).view(ns, m, npad)[:, :, :n]
        for s in range(ns - 1, -1, -1):
            C += P[s].to(torch.float64) * BASE ** (-(s + t + 2))
    C *= pow2(ea)
    C *= pow2(eb)
    if parts is not None:
        parts.update(Ad=Ad, Bd=Bd, ea=ea, eb=eb)
    return C


def _rows_like_r(M: int, K: int, gen, device):
    """M stacked K x K matrices with the spread of Hermite Coulomb tables: each entry a
    unit normal times 10^u, u uniform in [-6, 0], signs mixed."""
    x = torch.randn(M * K, K, generator=gen, dtype=torch.float64, device=device)
    u = torch.rand(M * K, K, generator=gen, dtype=torch.float64, device=device)
    return x * torch.pow(10.0, -6.0 * u)


def measure(M: int = 32768, K: int = 35, n: int = 36, reps: int = 5, seed: int = 0) -> dict:
    """Times the (dd|dd) ket transform shape -- M primitive quartets, each a K x K
    Hermite table (K = 35 Hermite functions up to order 4) times the ket pair's K x n
    E' table (n = 36 Cartesian function pairs) -- as one (M K) x K @ K x n product:
    by split operands on the BF16 tensor cores, and by cuBLAS DGEMM.  Rates are
    FP64-equivalent (2 M K K n FLOPs per product); the A operand is 320 MB at the
    default M, above the 129 MB L2."""
    dev = torch.device("cuda")
    try:
        probe = torch.ones(16, 16, dtype=torch.bfloat16, device=dev)
        tensor_core_mm(probe, probe)
    except (RuntimeError, TypeError) as e:  # torch without the FP32-output BF16 mm
        return {"probe": "split-operand FP64 GEMM", "unavailable": f"{type(e).__name__}: {e}"[:200],
                "torch": torch.__version__}
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    A = _rows_like_r(M, K, gen, dev)
    B = torch.randn(K, n, generator=gen, dtype=torch.float64, device=dev)
    flops = 2.0 * M * K * K * n
    ref = torch.mm(A, B)

    def timed(fn):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ev[0].record()
        for _ in range(reps):
            fn()
        ev[1].record()
        torch.cuda.synchronize()
        return ev[0].elapsed_time(ev[1]) / reps

    ms_dgemm = timed(lambda: torch.mm(A, B))
    ms_split_a = timed(lambda: split(A, 1))
    parts: dict = {}
    C = split_operand_mm(A, B, parts=parts)
    Ad, Bd = parts["Ad"], parts["Bd"]
    Kp, npad = Ad.shape[-1], Bd.shape[-1]
    A2 = Ad.reshape(DIGITS * M * K, Kp)

    def gemms_only():
        for t in range(DIGITS):
            tensor_core_mm(A2[: (DIGITS - t) * M * K], Bd[t])

    ms_gemm = timed(gemms_only)
    ms_total = timed(lambda: split_operand_mm(A, B))
    bound = torch.mm(A.abs(), B.abs())
    err = ((C - ref).abs() / bound).max().item()
    err_dgemm_scale = ((C - ref).abs() / (bound * 2.0 ** -53)).max().item()
    rowcol = K * A.abs().amax(dim=1, keepdim=True) * B.abs().amax(dim=0, keepdim=True) * 2.0 ** -52
    err_rowcol = ((C - ref).abs() / rowcol).max().item()
    gemm_bytes = sum((DIGITS - t) * M * K * (Kp * 2 + npad * 4) + Kp * npad * 2 for t in range(DIGITS))
    return {
        "probe": "split-operand FP64 GEMM on the BF16 tensor cores vs cuBLAS DGEMM",
        "shape": {"M_prim_quartets": M, "K_hermite": K, "n_ket_pairs": n, "padded": [Kp, npad], "digits": DIGITS,
                  "digit_products": DIGITS * (DIGITS + 1) // 2},
        "fp64_equiv_flops": flops,
        "dgemm": {"ms": ms_dgemm, "tflops": flops / ms_dgemm * 1e-9},
        "split_operand": {"ms_total": ms_total, "tflops_equiv": flops / ms_total * 1e-9,
                          "ms_split_A": ms_split_a, "ms_gemms": ms_gemm,
                          "gemm_tflops_equiv": flops / ms_gemm * 1e-9,
                          "gemm_bytes": gemm_bytes, "gemm_gbs": gemm_bytes / ms_gemm * 1e-6,
                          "ms_sum_and_rest": ms_total - ms_gemm - ms_split_a},
        "max_err_over_abs_product": err,
        "max_err_in_units_of_2^-53_abs_product": err_dgemm_scale,
        "max_err_over_stated_bound": err_rowcol,
        "torch": torch.__version__,
        "gpu": torch.cuda.get_device_name(0),
    }


if __name__ == "__main__":
    print(json.dumps(measure()))
