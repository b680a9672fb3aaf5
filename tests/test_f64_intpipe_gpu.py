"""float64 operations computed on the integer pipes must be bit-identical to
IEEE float64 arithmetic:

* sqrt (correctly rounded) against numpy's sqrt on random bit patterns of
  every magnitude, subnormals, values next to exact squares and next to
  half-way cases, and the special values (NaN compared as NaN);
* multiplication by a tape constant (powers of two scale the exponent on the
  integer pipe) against numpy's product, including subnormal, overflowing and
  signed-zero results and non-power-of-two constants;
* max / min / argmax / argmin of float64 with +-0 ties, NaN and infinities
  against the oracle (strict comparisons, first index, NaN never wins)."""
import numpy as np
import pytest

import ncarray_gb300 as nca
from ncarray_gb300.dtype import DType, RedOp
from tests.helpers import SEED

pytestmark = pytest.mark.gpu


def _doubles(rng, n):
    u = rng.integers(0, 2**63 - 1, n, dtype=np.int64).astype(np.uint64)
    parts = [u.view(np.float64)]                                        # every exponent
    parts.append(rng.random(n))                                         # [0, 1)
    parts.append((rng.integers(1, 2**52, n // 4, dtype=np.int64)).astype(np.uint64).view(np.float64))  # subnormals
    q = (rng.integers(2**52, 2**53, n // 4, dtype=np.int64)).astype(np.float64)
    sq = (q * q) * np.ldexp(1.0, rng.integers(-400, -100, n // 4))      # exact squares (scaled)
    parts.append(sq)
    parts.append(np.nextafter(sq, np.inf))
    parts.append(np.nextafter(sq, 0.0))
    h = (2 * q + 1)
    hw = (h * h) * np.ldexp(1.0, rng.integers(-600, -300, n // 4))    # half-way neighbourhoods
    parts.append(hw)
    parts.append(np.nextafter(hw, np.inf))
    parts.append(np.nextafter(hw, 0.0))
    parts.append(np.array([0.0, -0.0, np.inf, -np.inf, np.nan, -1.0, -1e-300, 5e-324, 2.2250738585072014e-308,
                           1.7976931348623157e308, 1.0, 4.0, 0.25, 2.0, 3.0]))
    x = np.concatenate(parts)
    return x[np.isfinite(x) | np.isnan(x) | np.isinf(x)]


def _same_bits(got, want):
    both_nan = np.isnan(got) & np.isnan(want)
    return bool(np.all(both_nan | (got.view(np.uint64) == want.view(np.uint64))))


def test_sqrt_bit_exact(cuda):
    rng = np.random.default_rng(SEED + 700)
    for _ in range(2):
        x = np.abs(_doubles(rng, 1 << 20))
        x[:3] = [-0.0, -1.0, np.nan]
        d = nca.NCDevArray.from_host(x)
        with nca.lazy_mode():
            e = nca.sqrt(d)
        got = e.materialize().to_host()
        with np.errstate(invalid="ignore"):
            want = np.sqrt(x)
        assert _same_bits(got, want)


@pytest.mark.parametrize("c", [0.5, 2.0, -0.25, 2.0**-1000, 2.0**1000, -1.0, 3.0, 2.0**-1074, 0.0, -0.0,
                               2.0**1023, 1.5])
def test_multiply_by_constant_bit_exact(cuda, c):
    rng = np.random.default_rng(SEED + 701)
    x = _doubles(rng, 1 << 18)
    x = np.concatenate([x, -x])
    d = nca.NCDevArray.from_host(x)
    with nca.lazy_mode():
        e1 = d * np.float64(c)
        e2 = nca.DevExpr.const(np.float64(c)) * d   # the constant first on the tape
    want = x * np.float64(c)
    assert _same_bits(e1.materialize().to_host(), want)
    assert _same_bits(e2.materialize().to_host(), want)


def test_extremes_with_signed_zeros_and_nan(cuda, orc):
    rng = np.random.default_rng(SEED + 702)
    n = 70_007   # 7 x 10001
    cases = []
    x = np.zeros(n); x[::3] = -0.0; cases.append(x)                     # +-0 ties only
    x = -np.abs(rng.normal(size=n)); x[[10, 500, 60_000]] = -0.0; x[[11, 501]] = 0.0; cases.append(x)
    x = rng.normal(size=n); x[[0, 5, 69_999]] = np.nan; cases.append(x)
    x = np.full(n, -np.inf); cases.append(x)
    x = rng.normal(size=n); x[[100, 200]] = np.inf; x[[300, 400]] = -np.inf; cases.append(x)
    for h in cases:
        hv = h.reshape(7, -1)
        d = nca.NCDevArray.from_host(hv)
        for op in (RedOp.MAX, RedOp.MIN, RedOp.ARGMAX, RedOp.ARGMIN):
            (res,) = d._expr().evaluate(reductions=[(op, None)])
            got = res.to_host().reshape(-1)
            want = np.asarray(orc.reduce(hv, int(DType.float64), int(op))).reshape(-1)
            assert got.tobytes() == want.tobytes(), (op, h[:4])
        for op in (RedOp.MAX, RedOp.ARGMIN, RedOp.MIN, RedOp.ARGMAX):
            (res,) = d._expr().evaluate(reductions=[(op, 1)])
            want = orc.reduce(hv, int(DType.float64), int(op), [1])
            assert res.to_host().tobytes() == want.tobytes(), op
