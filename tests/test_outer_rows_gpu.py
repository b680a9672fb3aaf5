"""Outer reductions (innermost axis kept) in their four schedules against the
oracle: the row-lane form on splits with the last CTA merging them (default),
with a finalize launch (NCA_K4_ROWS=2) or on a persistent grid of equal unit
ranges (NCA_K4_ROWS=3), and the thread-per-column-group form (NCA_K4_ROWS=0). Max/min/argmax/argmin and
integer sums bit-exact, float sums within the tolerances of
test_reduce_gpu; the stored expression value bit-exact.

Shapes: one split (many kept columns), many splits (few kept columns, many
rows), ragged row counts, kept groups that do not fill a CTA, a middle
reduced axis, strided and broadcast operands, NaN / ties / -0.0 at the
extremes."""
import os

import numpy as np
import pytest

import ncarray_gb300 as nca
from ncarray_gb300.dtype import DType, RedOp
from tests.helpers import SEED, assert_bits_equal, rand
from tests.test_reduce_gpu import check_reduction

pytestmark = pytest.mark.gpu

MODES = ["default", "3", "2", "0"]


def _with_mode(mode, fn):
    old = os.environ.get("NCA_K4_ROWS")
    if mode == "default":
        os.environ.pop("NCA_K4_ROWS", None)
    else:
        os.environ["NCA_K4_ROWS"] = mode
    try:
        return fn()
    finally:
        if old is None:
            os.environ.pop("NCA_K4_ROWS", None)
        else:
            os.environ["NCA_K4_ROWS"] = old


CASES = [((4096, 1024), 0), ((5000, 64), 0), ((37, 4100), 0), ((3, 2, 260), 1), ((64, 300, 96), 1),
         ((9, 40000), 0), ((2049, 8), 0)]


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("dt", [DType.float32, DType.float64, DType.int32, DType.bfloat16])
def test_outer_axis_reductions(cuda, orc, mode, dt):
    rng = np.random.default_rng(SEED + 1200 + int(dt))
    for shape, ax in CASES:
        h = rand(rng, shape, dt)
        d = nca.NCDevArray.from_host(h, dt)
        for op in (RedOp.SUM, RedOp.MEAN, RedOp.MAX, RedOp.MIN, RedOp.ARGMAX, RedOp.ARGMIN):
            (res,) = _with_mode(mode, lambda: d._expr().evaluate(reductions=[(op, ax)]))
            check_reduction(orc, h, dt, op, ax, res.to_host())


@pytest.mark.parametrize("mode", MODES)
def test_outer_fused_expression_stored(cuda, orc, mode):
    """a*b + |c| over (300, 2048) float64 with c broadcast along axis 0 and a
    strided: the value stored and its axis-0 sum, max, argmin in one pass."""
    from tests.helpers import oracle_eval
    rng = np.random.default_rng(SEED + 1210)
    a = rng.normal(size=(300, 4096))
    b = rng.normal(size=(300, 2048))
    c = rng.normal(size=(1, 2048))
    da = nca.NCDevArray.from_host(a)[:, ::2]
    db, dc = nca.NCDevArray.from_host(b), nca.NCDevArray.from_host(c)
    with nca.lazy_mode():
        e = da * db + abs(dc)
    out = nca.NCDevArray(e.shape, e.dtype)
    s, mx, am = _with_mode(mode, lambda: e.evaluate(out=out, reductions=[(RedOp.SUM, 0), (RedOp.MAX, 0),
                                                                      (RedOp.ARGMIN, 0)]))
    ref = oracle_eval(orc, e, [np.ascontiguousarray(a[:, ::2]), b, np.broadcast_to(c, (300, 2048))])
    assert_bits_equal(out.to_host(), ref, "stored value")
    check_reduction(orc, ref, DType.float64, RedOp.SUM, 0, s.to_host())
    check_reduction(orc, ref, DType.float64, RedOp.MAX, 0, mx.to_host())
    check_reduction(orc, ref, DType.float64, RedOp.ARGMIN, 0, am.to_host())


@pytest.mark.parametrize("mode", MODES)
def test_outer_special_values(cuda, orc, mode):
    rng = np.random.default_rng(SEED + 1220)
    h = rng.normal(size=(3000, 256)).astype(np.float32)
    h[:, 0] = np.nan
    h[::7, 1] = np.nan
    h[:, 2] = 5.0                       # ties everywhere: first index wins
    h[100, 3], h[2000, 3] = 9.0, 9.0
    h[:, 4] = -0.0
    h[50, 4] = 0.0
    h[:, 5] = -np.inf
    h[:, 6] = np.inf
    d = nca.NCDevArray.from_host(h)
    for op in (RedOp.MAX, RedOp.MIN, RedOp.ARGMAX, RedOp.ARGMIN, RedOp.SUM):
        (res,) = _with_mode(mode, lambda: d._expr().evaluate(reductions=[(op, 0)]))
        want = orc.reduce(h, int(DType.float32), int(op), 0)
        if op == RedOp.SUM:
            got = res.to_host()
            fin = np.isfinite(want)
            assert np.array_equal(np.isnan(got), np.isnan(want))
            assert np.all(np.abs(got[fin] - want[fin]) <= 2.0**-23 * np.abs(want[fin]) +
                          1e-12 * np.abs(h[:, fin].astype(np.float64)).sum(axis=0))
        else:
            assert res.to_host().tobytes() == np.asarray(want).tobytes(), op
