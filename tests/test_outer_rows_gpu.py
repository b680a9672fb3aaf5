"""Outer reductions (innermost axis kept) in their five schedules against the
oracle: the row-lane form on splits with the last CTA merging them (default),
the same with its rows bulk-copied into shared memory (NCA_K4_BULK=1, where
the rows are contiguous and 16-byte aligned), with a finalize launch
(NCA_K4_ROWS=2) or on a persistent grid of equal unit ranges
(NCA_K4_ROWS=3), and the thread-per-column-group form (NCA_K4_ROWS=0). The
bulk-staged and the plain row-lane forms accumulate in the same order and are
compared bit for bit. Max/min/argmax/argmin and
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

MODES = ["default", "bulk", "3", "2", "0"]


def _with_mode(mode, fn):
    old = {k: os.environ.get(k) for k in ("NCA_K4_ROWS", "NCA_K4_BULK")}
    os.environ.pop("NCA_K4_ROWS", None)
    os.environ.pop("NCA_K4_BULK", None)
    if mode == "bulk":
        os.environ["NCA_K4_BULK"] = "1"
    elif mode != "default":
        os.environ["NCA_K4_ROWS"] = mode
    try:
        return fn()
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


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


@pytest.mark.parametrize("dt", [DType.float32, DType.int32, DType.uint8, DType.bfloat16])
def test_bulk_staged_matches_row_lane_bits(cuda, dt):
    """The bulk-staged form against the plain row-lane form: the same bits for
    sums, extremes and their indices (splits, a partial last column set, the
    middle axis of three, a stage count and rows per stage set by hand)."""
    rng = np.random.default_rng(SEED + 1230 + int(dt))
    for shape, ax in [((4096, 1024), 0), ((37, 4104), 0), ((64, 300, 96), 1), ((3, 2, 264), 1), ((2049, 8), 0),
                      ((1000, 2056), 0)]:
        h = rand(rng, shape, dt)
        d = nca.NCDevArray.from_host(h, dt)
        for op in (RedOp.SUM, RedOp.MAX, RedOp.ARGMIN):
            got = {}
            for mode in ("bulk", "default"):
                (res,) = _with_mode(mode, lambda: d._expr().evaluate(reductions=[(op, ax)]))
                got[mode] = res.to_host()
            assert got["bulk"].tobytes() == got["default"].tobytes(), (shape, op)
    h = rand(rng, (777, 1024), dt)
    d = nca.NCDevArray.from_host(h, dt)
    os.environ["NCA_K4B_RB"], os.environ["NCA_K4B_NS"] = "8", "2"
    try:
        (a,) = _with_mode("bulk", lambda: d._expr().evaluate(reductions=[(RedOp.SUM, 0)]))
    finally:
        del os.environ["NCA_K4B_RB"], os.environ["NCA_K4B_NS"]
    (b,) = _with_mode("default", lambda: d._expr().evaluate(reductions=[(RedOp.SUM, 0)]))
    assert a.to_host().tobytes() == b.to_host().tobytes()
    for cb in ("1", "2", "4"):          # 1 to 4 column blocks of 256 elements per CTA
        os.environ["NCA_K4B_CB"] = cb
        try:
            (c,) = _with_mode("bulk", lambda: d._expr().evaluate(reductions=[(RedOp.SUM, 0)]))
        finally:
            del os.environ["NCA_K4B_CB"]
        assert c.to_host().tobytes() == b.to_host().tobytes(), cb


def test_bulk_staged_stored_expression(cuda):
    """a * b + c over float32 rows of 2 operands plus a broadcast-free third:
    the stored value and its axis-0 sum and argmax, bulk-staged against the
    plain row-lane form."""
    rng = np.random.default_rng(SEED + 1240)
    a, b, c = (rng.normal(size=(1500, 3072)).astype(np.float32) for _ in range(3))
    da, db, dc = (nca.NCDevArray.from_host(x) for x in (a, b, c))
    outs = {}
    for mode in ("bulk", "default"):
        with nca.lazy_mode():
            e = da * db + dc
        out = nca.NCDevArray(e.shape, e.dtype)
        s, am = _with_mode(mode, lambda: e.evaluate(out=out, reductions=[(RedOp.SUM, 0), (RedOp.ARGMAX, 0)]))
        outs[mode] = (out.to_host(), s.to_host(), am.to_host())
    for x, y in zip(outs["bulk"], outs["default"]):
        assert x.tobytes() == y.tobytes()
    assert np.array_equal(outs["bulk"][0], a * b + c)
