"""Reductions on the GPU vs the oracle.

Integer sums, max/min, argmax/argmin are bit-exact; float sums and means are
within a stated tolerance of the float64 oracle:
  float32/bf16/f16 inputs: |got - ref| <= 2**-23 |ref| + 1e-12 sum|x|
  float64 inputs:          |got - ref| <= 1e-15 |ref| + 1e-13 sum|x|
Known answers follow tests/cxx/test_gpu_reductions.cu:191-294,
tests/cxx/test_reductions.cc:26-102 and tests/python/test_gpu_operations.py."""
import numpy as np
import pytest

import ncarray_gb300 as nca
from ncarray_gb300.dtype import DType, FLOATS, RedOp
from tests.helpers import SEED, assert_bits_equal, rand

pytestmark = pytest.mark.gpu

F_TOL = {DType.float32: (2.0**-23, 1e-12), DType.bfloat16: (2.0**-23, 1e-12), DType.float16: (2.0**-23, 1e-12),
         DType.float64: (1e-15, 1e-13)}


def dev(h, dt=None):
    return nca.NCDevArray.from_host(h, dt)


def as_float(h, dt):
    if dt == DType.bfloat16:
        return (h.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    return h.astype(np.float64)


def check_reduction(orc, h, dt, op, axes, got):
    want = orc.reduce(h, int(dt), int(op), axes)
    got = np.asarray(got)
    if op in (RedOp.SUM, RedOp.MEAN) and dt in FLOATS:
        rt, at = F_TOL[dt]
        absx = np.abs(as_float(h, dt))
        scale = absx.sum() if axes is None else absx.sum(axis=tuple([axes] if isinstance(axes, int) else axes))
        if op == RedOp.MEAN:
            n = h.size if axes is None else h.size // max(np.asarray(scale).size, 1)
            scale = scale / max(n, 1)
        err = np.abs(got.astype(np.float64) - want.astype(np.float64))
        lim = rt * np.abs(want.astype(np.float64)) + at * scale + 1e-300
        assert np.all(err <= lim), f"{dt.name} {op.name} axes={axes}: max err {err.max()} lim {np.min(lim)}"
    else:
        assert_bits_equal(got.reshape(want.shape), want, f"{dt.name} {op.name} axes={axes}")


DTS = [DType.bool, DType.int8, DType.uint8, DType.int16, DType.int32, DType.uint32, DType.int64,
       DType.uint64, DType.float32, DType.float64, DType.bfloat16, DType.float16]
OPS = [RedOp.SUM, RedOp.MEAN, RedOp.MAX, RedOp.MIN, RedOp.ARGMAX, RedOp.ARGMIN]


@pytest.mark.parametrize("dt", DTS)
def test_full_reductions(cuda, orc, dt):
    rng = np.random.default_rng(SEED + 100 + int(dt))
    for shape in [(1,), (7,), (1000,), (3, 5, 7), (257, 1031)]:
        h = rand(rng, shape, dt)
        d = dev(h, dt)
        for op in OPS:
            (res,) = d._expr().evaluate(reductions=[(op, None)])
            check_reduction(orc, h, dt, op, None, res.to_host())


@pytest.mark.parametrize("dt", [DType.int32, DType.float32, DType.float64, DType.uint8, DType.bfloat16])
def test_axis_reductions(cuda, orc, dt):
    rng = np.random.default_rng(SEED + 200 + int(dt))
    h = rand(rng, (6, 10, 12, 16), dt)
    d = dev(h, dt)
    for axes in [0, 1, 2, 3, (0, 1), (1, 3), (0, 2, 3), (2, 3), (0, 1, 2, 3)]:
        for op in OPS:
            (res,) = d._expr().evaluate(reductions=[(op, axes)])
            check_reduction(orc, h, dt, op, axes, res.to_host())


def test_reductions_of_views(cuda, orc):
    rng = np.random.default_rng(SEED + 300)
    h = rng.normal(size=(16, 12, 10)).astype(np.float32)
    d = dev(h)
    for dv, hv in [(d.transpose(2, 0, 1), h.transpose(2, 0, 1)), (d[::2, ::-1, 3:], h[::2, ::-1, 3:])]:
        for axes in [None, 0, 1, 2, (0, 2)]:
            for op in (RedOp.SUM, RedOp.MAX, RedOp.ARGMIN):
                (res,) = dv._expr().evaluate(reductions=[(op, axes)])
                check_reduction(orc, np.ascontiguousarray(hv), DType.float32, op, axes, res.to_host())


def test_large_float_sum_accuracy(cuda, orc):
    """2^22 lognormal(0,2) values with random signs: the float32 path keeps a
    float-float per thread, so the result is within a few ulp of float64."""
    rng = np.random.default_rng(SEED + 400)
    x = (np.exp(rng.normal(0, 2, 1 << 22)) * rng.choice([-1, 1], 1 << 22)).astype(np.float32)
    d = dev(x)
    s = d.sum()
    ref = float(orc.reduce(x, 10, 0))
    ref64 = float(np.sum(x.astype(np.float64)))
    assert abs(s - ref) <= 2.0**-23 * abs(ref) + 1e-12 * float(np.abs(x).sum())
    assert abs(ref - ref64) <= 1e-9 * float(np.abs(x).sum())


def test_edge_values(cuda, orc):
    """NaN never wins, ties keep the first index, -inf-only input reports
    lowest() and index 0 (host scan of src/lib/ncarray/host/reductions.hh:118-169)."""
    cases = [
        np.array([np.nan, 1.0, 3.0, 3.0, np.nan, -2.0], dtype=np.float32),
        np.array([-np.inf, -np.inf], dtype=np.float32),
        np.array([0.0, -0.0, 0.0], dtype=np.float32),
        np.array([np.nan, np.nan], dtype=np.float64),
        np.array([2**31 - 1, -2**31, 5, 2**31 - 1], dtype=np.int32),
    ]
    for h in cases:
        dt = {np.float32: DType.float32, np.float64: DType.float64, np.int32: DType.int32}[h.dtype.type]
        d = dev(h)
        for op in OPS[2:]:
            (res,) = d._expr().evaluate(reductions=[(op, None)])
            check_reduction(orc, h, dt, op, None, res.to_host())


def test_reference_known_answers(cuda):
    f = nca.NCDevArray.from_host(np.arange(256, dtype=np.float32))
    assert f.sum() == 32640.0 and f.max() == 255.0 and f.min() == 0.0
    i = nca.NCDevArray.from_host(np.arange(1, 7, dtype=np.int32).reshape(2, 3))
    assert np.array_equal(i.sum(0).to_host(), [5, 7, 9])
    assert np.array_equal(i.sum(1).to_host(), [6, 15])
    assert np.array_equal(i.max(0).to_host(), [4, 5, 6]) and np.array_equal(i.min(1).to_host(), [1, 4])
    s = nca.NCDevArray([4, 4], DType.int32).fill(1)
    s[1:3, 1:3].fill(10)
    assert s.sum() == 52
    t = nca.NCDevArray([10, 2], DType.int32).fill(1)
    r = t._expr().evaluate(reductions=[(RedOp.SUM, None)])[0]
    assert r.dtype == DType.int32 and int(r.to_host()) == 20
    u = nca.NCDevArray.from_host(np.arange(256, dtype=np.uint32))
    assert u.sum() == 32640 and u.max() == 255 and u.min() == 0
    m = nca.NCDevArray.from_host(np.array([1.0, 2.0, 3.0], dtype=np.float32))
    assert m.mean() == 2.0


def test_fused_c1(cuda, orc):
    """C1 in one pass: out = expr, axis-0 sum and max, then full sum/max from them."""
    rng = np.random.default_rng(SEED + 0)
    a, b, c = (rng.uniform(-1, 1, (128, 128, 128)) for _ in range(3))
    da, db, dc = dev(a), dev(b), dev(c)
    with nca.lazy_mode():
        e = da * db + nca.sqrt(abs(dc)) - 0.5 * da
    out = nca.NCDevArray(e.shape, e.dtype)
    s0, m0 = e.evaluate(out=out, reductions=[(RedOp.SUM, 0), (RedOp.MAX, 0)])
    ref = a * b + np.sqrt(np.abs(c)) - np.float32(0.5) * a
    np.testing.assert_array_equal(out.to_host(), ref)
    check_reduction(orc, ref, DType.float64, RedOp.SUM, 0, s0.to_host())
    check_reduction(orc, ref, DType.float64, RedOp.MAX, 0, m0.to_host())
    check_reduction(orc, ref, DType.float64, RedOp.SUM, None, s0.sum())
    assert m0.max() == float(orc.reduce(ref, 11, 2))


def test_fused_c2_axis2(cuda, orc):
    """C2 shape family: y stored + max/argmax over axis 2 in one pass."""
    rng = np.random.default_rng(SEED + 1)
    x = rng.normal(size=(16, 64, 32, 8)).astype(np.float32)
    xp = x.transpose(3, 1, 2, 0)
    v = rng.normal(size=(64,)).astype(np.float32)
    k = rng.integers(-1000, 1001, xp.shape).astype(np.int32)
    dx, dv, dk = dev(x).permute(3, 1, 2, 0), dev(v).reshape(1, 64, 1, 1), dev(k)
    with nca.lazy_mode():
        y = dx * dv + dk
    out = nca.NCDevArray(y.shape, y.dtype)
    mx, am = y.evaluate(out=out, reductions=[(RedOp.MAX, 2), (RedOp.ARGMAX, 2)])
    yr = xp * v.reshape(1, -1, 1, 1) + k.astype(np.float32)
    np.testing.assert_array_equal(out.to_host(), yr)
    check_reduction(orc, yr, DType.float32, RedOp.MAX, 2, mx.to_host())
    check_reduction(orc, yr, DType.float32, RedOp.ARGMAX, 2, am.to_host())
    assert np.array_equal(am.to_host(), np.argmax(yr, axis=2))
