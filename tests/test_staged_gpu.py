"""Fused expressions + reductions whose operands are transposed relative to the
output, staged through shared memory by the JIT kernel classes 6 (register
staging, any layout) and 7 (TMA tiles on a warp-specialised pipeline, units
split between CTAs merged in CTA order), vs the oracle.

Covers partial p tiles, q extents from 2 to 32, two staged operands, float64
and int32 staged operands, several reduced axes, every reduction op, units
split between CTAs, and each class-7 case again on class 6.
Expression values bit-exact; reductions per tests/test_reduce_gpu.py."""
import numpy as np
import pytest

import ncarray_gb300 as nca
from ncarray_gb300.dtype import DType, RedOp
from tests.helpers import SEED, assert_bits_equal, oracle_eval
from tests.test_reduce_gpu import check_reduction

pytestmark = pytest.mark.gpu


def dev(h, dt=None):
    return nca.NCDevArray.from_host(h, dt)


@pytest.mark.parametrize("shape,axes", [
    ((8, 16, 32, 64), 2),        # the C2 layout family
    ((5, 7, 9, 70), 2),          # partial p tile, odd extents
    ((32, 3, 100, 33), (1, 2)),  # q = 32, two reduced axes
    ((2, 40, 6, 128), 1),        # q = 2
])
@pytest.mark.parametrize("op", [RedOp.MAX, RedOp.ARGMAX, RedOp.SUM, RedOp.MIN, RedOp.ARGMIN, RedOp.MEAN])
def test_staged_reduce(cuda, orc, shape, axes, op):
    rng = np.random.default_rng(SEED + 70)
    q, b, r, p = shape
    # x stored (p, b, r, q) -> viewed (q, b, r, p): unit stride along q
    x = rng.normal(size=(p, b, r, q)).astype(np.float32)
    xp = x.transpose(3, 1, 2, 0)
    k = rng.integers(-1000, 1001, xp.shape).astype(np.int32)
    dx, dk = dev(x).permute(3, 1, 2, 0), dev(k)
    with nca.lazy_mode():
        y = dx * 2.0 + dk
    out = nca.NCDevArray(y.shape, y.dtype)
    (res,) = y.evaluate(out=out, reductions=[(op, axes)])
    yr = oracle_eval(orc, y, [xp, k])
    assert_bits_equal(out.to_host(), yr, "stored value")
    check_reduction(orc, yr, DType.float32, op, axes, res.to_host())


def test_two_staged_operands_and_f64(cuda, orc):
    rng = np.random.default_rng(SEED + 71)
    a = rng.normal(size=(96, 4, 48, 6))            # (p, b, r, q) float64
    c = rng.integers(-50, 50, (96, 4, 48, 6)).astype(np.int32)
    ap, cp = a.transpose(3, 1, 2, 0), c.transpose(3, 1, 2, 0)
    da, dc = dev(a).permute(3, 1, 2, 0), dev(c).permute(3, 1, 2, 0)
    with nca.lazy_mode():
        y = da * dc - da
    out = nca.NCDevArray(y.shape, y.dtype)
    mx, am, sm = y.evaluate(out=out, reductions=[(RedOp.MAX, 2), (RedOp.ARGMAX, 2), (RedOp.SUM, 2)])
    yr = oracle_eval(orc, y, [ap, cp])
    assert_bits_equal(out.to_host(), yr, "stored value")
    check_reduction(orc, yr, DType.float64, RedOp.MAX, 2, mx.to_host())
    check_reduction(orc, yr, DType.float64, RedOp.ARGMAX, 2, am.to_host())
    check_reduction(orc, yr, DType.float64, RedOp.SUM, 2, sm.to_host())


def test_staged_without_store(cuda, orc):
    rng = np.random.default_rng(SEED + 72)
    x = rng.normal(size=(64, 8, 200, 8)).astype(np.float32)
    xp = x.transpose(3, 1, 2, 0)
    with nca.lazy_mode():
        y = dev(x).permute(3, 1, 2, 0) + 1.0
    mx, am = y.evaluate(reductions=[(RedOp.MAX, 2), (RedOp.ARGMAX, 2)])
    yr = oracle_eval(orc, y, [xp])
    check_reduction(orc, yr, DType.float32, RedOp.MAX, 2, mx.to_host())
    check_reduction(orc, yr, DType.float32, RedOp.ARGMAX, 2, am.to_host())


# views that class 7 takes: 4-byte elements, p extent a multiple of 32,
# q extent 4..32, rows 16-byte aligned
ASYNC_CASES = [
    ((8, 16, 32, 64), 2),        # the C2 layout family
    ((8, 4, 2048, 64), 2),       # few units, each split between many CTAs
    ((16, 6, 40, 96), (1, 2)),   # q = 16, p tiles of 32, two loop dims
    ((32, 3, 16, 64), 2),        # q = 32: eight items per thread
    ((4, 10, 64, 64), 2),        # q = 4
]


@pytest.mark.parametrize("async_on", ["1", "0"])
@pytest.mark.parametrize("shape,axes", ASYNC_CASES)
@pytest.mark.parametrize("op", [RedOp.MAX, RedOp.ARGMAX, RedOp.SUM, RedOp.MEAN, RedOp.MIN])
def test_async_staged_reduce(cuda, orc, monkeypatch, async_on, shape, axes, op):
    """C2's expression (staged x times a broadcast vector plus an int32 array
    in p rows) on class 7, and the same views on class 6."""
    monkeypatch.setenv("NCA_STAGED_ASYNC", async_on)
    rng = np.random.default_rng(SEED + 73)
    q, b, r, p = shape
    x = rng.normal(size=(p, b, r, q)).astype(np.float32)
    xp = x.transpose(3, 1, 2, 0)
    vv = rng.normal(size=b).astype(np.float32)
    k = rng.integers(-1000, 1001, xp.shape).astype(np.int32)
    dx, dv, dk = dev(x).permute(3, 1, 2, 0), dev(vv).reshape(1, b, 1, 1), dev(k)
    with nca.lazy_mode():
        y = dx * dv + dk
    out = nca.NCDevArray(y.shape, y.dtype)
    (res,) = y.evaluate(out=out, reductions=[(op, axes)])
    yr = oracle_eval(orc, y, [xp, vv.reshape(1, b, 1, 1), k])
    assert_bits_equal(out.to_host(), yr, "stored value")
    check_reduction(orc, yr, DType.float32, op, axes, res.to_host())


@pytest.mark.parametrize("async_on", ["1", "0"])
def test_async_staged_plain_and_argmax_ties(cuda, orc, monkeypatch, async_on):
    """A transposed expression without reductions (one unit over all CTAs),
    then max/argmax over values with many ties (first index must win)."""
    monkeypatch.setenv("NCA_STAGED_ASYNC", async_on)
    rng = np.random.default_rng(SEED + 74)
    x = rng.integers(-3, 4, size=(64, 8, 512, 8)).astype(np.float32)
    xp = x.transpose(3, 1, 2, 0)
    with nca.lazy_mode():
        y = dev(x).permute(3, 1, 2, 0) * 3.0 - 1.0
    out = nca.NCDevArray(y.shape, y.dtype)
    y.evaluate(out=out)
    yr = oracle_eval(orc, y, [xp])
    assert_bits_equal(out.to_host(), yr, "stored value")
    mx, am = y.evaluate(reductions=[(RedOp.MAX, 2), (RedOp.ARGMAX, 2)])
    check_reduction(orc, yr, DType.float32, RedOp.MAX, 2, mx.to_host())
    check_reduction(orc, yr, DType.float32, RedOp.ARGMAX, 2, am.to_host())


@pytest.mark.parametrize("rb,stages,outbufs", [("4", "3", "2"), ("8", "3", "1"), ("16", "2", "1"), ("8", "6", "2")])
@pytest.mark.parametrize("shape", [(8, 16, 32, 64), (16, 6, 48, 96)])
def test_async_staged_tuning_knobs(cuda, orc, monkeypatch, rb, stages, outbufs, shape):
    """Class 7 under other blocks of loop indices, pipeline depths and one or
    two output tiles: the same bits as the oracle for the stored value and
    max/argmax."""
    monkeypatch.setenv("NCA_STAGED_ASYNC", "1")
    monkeypatch.setenv("NCA_STAGED_RB", rb)
    monkeypatch.setenv("NCA_STAGED_STAGES", stages)
    monkeypatch.setenv("NCA_STAGED_OUTBUFS", outbufs)
    rng = np.random.default_rng(SEED + 75)
    q, b, r, p = shape
    x = rng.normal(size=(p, b, r, q)).astype(np.float32)
    xp = x.transpose(3, 1, 2, 0)
    vv = rng.normal(size=b).astype(np.float32)
    k = rng.integers(-1000, 1001, xp.shape).astype(np.int32)
    dx, dv, dk = dev(x).permute(3, 1, 2, 0), dev(vv).reshape(1, b, 1, 1), dev(k)
    with nca.lazy_mode():
        y = dx * dv + dk
    out = nca.NCDevArray(y.shape, y.dtype)
    mx, am = y.evaluate(out=out, reductions=[(RedOp.MAX, 2), (RedOp.ARGMAX, 2)])
    yr = oracle_eval(orc, y, [xp, vv.reshape(1, b, 1, 1), k])
    assert_bits_equal(out.to_host(), yr, "stored value")
    check_reduction(orc, yr, DType.float32, RedOp.MAX, 2, mx.to_host())
    check_reduction(orc, yr, DType.float32, RedOp.ARGMAX, 2, am.to_host())
