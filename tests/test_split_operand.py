"""Split-operand FP64 products (mmd.split_operand) restated on the CPU: the digits
rebuild each operand to 56 bits, every digit product is an integer below 2^24 (what
the BF16 tensor-core GEMM with FP32 accumulation returns exactly), and the assembled
product stays within the stated bound of the exact product."""
from fractions import Fraction

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from mmd import split_operand as so  # noqa: E402


def _exact_mm(a, b):
    """Digit product as the tensor cores form it: exact integer sums, returned in FP32
    (the test checks that FP32 holds them exactly)."""
    p = a.double() @ b.double()
    assert float((p - p.round()).abs().max()) == 0.0
    assert float(p.abs().max()) < 2.0 ** 24
    return p.float()


def _r_like(m, k, seed):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((m, k)) * 10.0 ** (-6.0 * rng.random((m, k)))
    return torch.from_numpy(x)


def test_digits_rebuild_each_row_to_56_bits():
    A = _r_like(64, 35, 1)
    A[3] = 0.0                                   # a zero row
    A[5, 7] = 2.0 ** -1000                       # tiny entries keep their row's scale
    d, e = so.split(A, 1)
    assert d.dtype == torch.bfloat16 and d.shape == (so.DIGITS, 64, 35)
    dd = d.double()
    assert float((dd - dd.round()).abs().max()) == 0.0 and float(dd.abs().max()) <= 255.0
    back = sum(dd[s] * so.BASE ** (-(s + 1)) for s in range(so.DIGITS)) * so.pow2(e)
    scale = so.pow2(e)
    assert float(((A - back).abs() / scale).max()) < 2.0 ** -56
    assert float(back[3].abs().max()) == 0.0


def test_pow2_is_exact():
    k = torch.arange(-1022, 1024)
    assert torch.equal(so.pow2(k), torch.tensor([2.0 ** int(i) for i in k], dtype=torch.float64))


@pytest.mark.parametrize("shape", [(40, 35, 36), (17, 10, 6), (8, 256, 8)])
def test_split_product_within_the_stated_bound(shape):
    m, K, n = shape
    A = _r_like(m, K, 2)
    B = torch.from_numpy(np.random.default_rng(3).standard_normal((K, n)))
    C = so.split_operand_mm(A, B, mm=_exact_mm)
    an, bn = A.numpy(), B.numpy()
    exact = np.array([[float(sum(Fraction(an[i, k]) * Fraction(bn[k, j]) for k in range(K)))
                       for j in range(n)] for i in range(m)])
    rowcol = K * np.abs(an).max(1, keepdims=True) * np.abs(bn).max(0, keepdims=True) * 2.0 ** -52
    assert np.max(np.abs(C.numpy() - exact) / rowcol) < 1.0
    # and in practice as close as FP64 itself on these matrices
    ref = an @ bn
    bound = np.abs(an) @ np.abs(bn)
    assert np.max(np.abs(C.numpy() - exact) / bound) < 64 * 2.0 ** -53
    assert np.max(np.abs(ref - exact) / bound) < 64 * 2.0 ** -53


def test_k_above_256_is_refused():
    with pytest.raises(ValueError):
        so.split_operand_mm(torch.ones(2, 257, dtype=torch.float64), torch.ones(257, 2, dtype=torch.float64),
                            mm=_exact_mm)
