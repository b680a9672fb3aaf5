"""General batched reductions (nca_batch_expr_*): thousands of uneven 1-D
arrays of mixed dtypes, each with up to four (expression, reduction) outputs,
in one persistent launch, against the oracle.

Per output, the oracle evaluates the same tape in the same compute dtype over
the array and reduces the result: max, min, argmax and argmin must match
exactly; sums and means within 2^-23 |ref| + 1e-12 sum|v| (v = the tape's
values). Graph replays must repeat the first launch's results exactly."""
import numpy as np
import pytest

import ncarray_gb300 as nca
from ncarray_gb300.batch import BatchExpr
from ncarray_gb300.dtype import DType, RedOp
from tests.helpers import SEED

pytestmark = pytest.mark.gpu

NPDT = {DType.float32: np.float32, DType.float64: np.float64, DType.int32: np.int32, DType.int64: np.int64,
        DType.float16: np.float16, DType.bfloat16: np.uint16}

FNS = {
    "id": None,
    "sq_m": lambda x: x * x - x,
    "abs2p1": lambda x: abs(x) * 2.0 + 1.0,
    "sqrtabs": lambda x: nca.sqrt(abs(x)),
    "half": lambda x: x * 0.5,
    "half_sq": lambda x: (x * 0.5) * (x * 0.5),
}


# output lists drawn by the mixed test: every tape and every reduction occurs
FLOAT_PATTERNS = [
    [("id", RedOp.SUM), ("id", RedOp.MEAN), ("id", RedOp.MAX), ("sq_m", RedOp.SUM)],
    [("id", RedOp.ARGMAX), ("id", RedOp.ARGMIN)],
    [("abs2p1", RedOp.MIN), ("sqrtabs", RedOp.ARGMAX), ("half", RedOp.MEAN)],
    [("sq_m", RedOp.ARGMIN)],
    [("sqrtabs", RedOp.SUM), ("id", RedOp.MIN), ("abs2p1", RedOp.ARGMIN), ("half_sq", RedOp.MAX)],
]
INT_PATTERNS = [
    [("half", RedOp.SUM), ("half", RedOp.ARGMAX), ("half_sq", RedOp.MEAN)],
    [("half", RedOp.MIN), ("half", RedOp.ARGMIN)],
    [("half_sq", RedOp.MAX), ("half", RedOp.MEAN), ("half_sq", RedOp.ARGMAX), ("half", RedOp.SUM)],
]


def _host(rng, dt, n):
    if dt in (DType.int32, DType.int64):
        return rng.integers(-10**6, 10**6, n).astype(NPDT[dt])
    x = (np.exp(rng.normal(size=n) * 2.0) * rng.choice([-1.0, 1.0], n)).astype(np.float32)
    if dt == DType.bfloat16:
        return (x.view(np.uint32) >> 16).astype(np.uint16)
    return x.astype(NPDT[dt])


def _check(orc, b, items_h, outs_spec, vals, idxs):
    for i, (h, dt) in enumerate(items_h):
        for o, (fname, op) in enumerate(outs_spec[i]):
            ins, sc, cdt, rdt = b._tapes[_tape_index(b, i, o)]
            y = orc.expr_eval(ins, [(int(d), v) for d, v in sc], int(cdt), [(h, int(dt))], h.shape, int(rdt))
            got_v, got_i = vals[i, o], idxs[i, o]
            if op in (RedOp.SUM, RedOp.MEAN):
                ref = float(orc.reduce(y, int(rdt), int(op)))
                scale = float(np.abs(y.astype(np.float64)).sum()) / (y.size if op == RedOp.MEAN else 1)
                assert abs(got_v - ref) <= 2.0**-23 * abs(ref) + 1e-12 * scale, (i, o, fname, op, got_v, ref)
            elif op in (RedOp.MAX, RedOp.MIN):
                ref = float(orc.reduce(y, int(rdt), int(op)))
                assert got_v == ref or (np.isnan(got_v) and np.isnan(ref)), (i, o, fname, op, got_v, ref)
            else:
                ref_i = int(orc.reduce(y, int(rdt), int(op)))
                assert got_i == ref_i, (i, o, fname, op, got_i, ref_i)
                ext = float(orc.reduce(y, int(rdt), 2 if op == RedOp.ARGMAX else 3))
                assert got_v == ext, (i, o, fname, op, got_v, ext)


def _tape_index(b, i, o):
    return b._item_tapes[i][o]


def _build(items):
    b = BatchExpr(items)
    # remember which tape each output uses (same order as the constructor's)
    b._item_tapes = []
    seen = {}
    for a, outs in items:
        row = []
        for fn, _ in outs:
            key = (fn, int(a.dtype))
            if key not in seen:
                seen[key] = len(seen)
            row.append(seen[key])
        b._item_tapes.append(row)
    return b


def test_mixed_batch_matches_oracle(cuda, orc):
    rng = np.random.default_rng(SEED + 600)
    dts = [DType.float32, DType.bfloat16, DType.float16, DType.float64, DType.int32, DType.int64]
    n_items = 1500
    lens = np.round(np.exp(rng.uniform(0, np.log(300_000), n_items))).astype(np.int64)
    lens[:6] = [1, 2, 63, 64, 65, 32768 * 4 + 3]
    items, items_h, spec = [], [], []
    for i in range(n_items):
        dt = dts[i % len(dts)]
        h = _host(rng, dt, int(lens[i]))
        d = nca.NCDevArray.from_host(h, dt)
        # an unaligned start for some float32 arrays: a view one element in
        if dt == DType.float32 and i % 12 == 0 and h.size > 1:
            d, h = d[1:], h[1:]
        # one of a few output lists per dtype class (a batch may hold at most 64
        # distinct (dtype, outputs) programs); integer inputs need a tape with a
        # floating result
        pool = INT_PATTERNS if dt in (DType.int32, DType.int64) else FLOAT_PATTERNS
        outs = pool[int(rng.integers(0, len(pool)))]
        items.append((d, [(FNS[f], op) for f, op in outs]))
        items_h.append((h, dt))
        spec.append(outs)
    b = _build(items)
    assert b.info()["programs"] >= 6
    vals, idxs = b.run(graph=True)
    _check(orc, b, items_h, spec, vals, idxs)
    v2, i2 = b.run(graph=True)     # a replay: the arrival counters were reset
    assert np.array_equal(v2, vals, equal_nan=True) and np.array_equal(i2, idxs)
    v3, i3 = b.run(graph=False)
    assert np.array_equal(v3, vals, equal_nan=True) and np.array_equal(i3, idxs)


def test_c5_outputs_and_plain_form(cuda, orc):
    """The C5 outputs (sum, mean, max, sum(x*x - x)) of float32 and bfloat16
    arrays through the general form, and the plain per-launch float64 form."""
    rng = np.random.default_rng(SEED + 601)
    n_items = 400
    lens = np.round(np.exp(rng.uniform(np.log(64), np.log(1 << 20), n_items))).astype(np.int64)
    items, items_h, spec = [], [], []
    outs = [("id", RedOp.SUM), ("id", RedOp.MEAN), ("id", RedOp.MAX), ("sq_m", RedOp.SUM)]
    for i in range(n_items):
        dt = DType.float32 if i % 2 == 0 else DType.bfloat16
        h = _host(rng, dt, int(lens[i]))
        items.append((nca.NCDevArray.from_host(h, dt), [(FNS[f], op) for f, op in outs]))
        items_h.append((h, dt))
        spec.append(outs)
    b = _build(items)
    assert b.info()["programs"] == 2
    vals, idxs = b.run()
    _check(orc, b, items_h, spec, vals, idxs)
    pv, _ = b.run(plain=True)
    # the plain form computes the tapes in float64: sums agree to float32
    # accuracy of the elementwise values, max exactly
    scale = np.array([float(np.abs(((h.astype(np.uint32) << 16).view(np.float32) if dt == DType.bfloat16 else h)
                                  .astype(np.float64)).sum()) for h, dt in items_h])
    assert np.all(np.abs(pv[:, 0] - vals[:, 0]) <= 1e-6 * scale)
    assert np.array_equal(pv[:, 2], vals[:, 2])


def test_special_values(cuda, orc):
    """NaN and +-inf inside arrays, all -inf / all +inf arrays, ties at the
    extremes, and empty arrays."""
    rng = np.random.default_rng(SEED + 602)
    cases = []
    x = rng.normal(size=5000).astype(np.float32); x[17] = np.nan; cases.append(x)
    x = rng.normal(size=70000).astype(np.float32); x[[5, 60000]] = np.inf; x[[7, 50001]] = -np.inf; cases.append(x)
    cases.append(np.full(40000, -np.inf, np.float32))
    cases.append(np.full(300, np.inf, np.float32))
    x = rng.normal(size=90000).astype(np.float32); x[[3, 40000, 89999]] = 9.0; x[[4, 40001]] = -9.0; cases.append(x)
    cases.append(np.zeros(0, np.float32))
    outs = [(None, RedOp.SUM), (None, RedOp.ARGMAX), (None, RedOp.ARGMIN), (None, RedOp.MAX)]
    items = [(nca.NCDevArray.from_host(h), outs) for h in cases]
    b = _build(items)
    vals, idxs = b.run()
    for i, h in enumerate(cases):
        for o, (_, op) in enumerate(outs):
            if h.size == 0:
                if op == RedOp.SUM:
                    assert vals[i, o] == 0.0
                continue
            if op == RedOp.SUM:
                ref = float(orc.reduce(h, 10, 0))
                assert (np.isnan(ref) and np.isnan(vals[i, o])) or vals[i, o] == ref or \
                    abs(vals[i, o] - ref) <= 2.0**-23 * abs(ref) + 1e-12 * float(np.abs(h.astype(np.float64)).sum())
            elif op == RedOp.MAX:
                assert vals[i, o] == float(orc.reduce(h, 10, 2))
            else:
                assert idxs[i, o] == int(orc.reduce(h, 10, int(op))), (i, op)


def test_pipelined_and_direct_forms_agree(cuda, orc):
    """The pipelined form (producer warp, shared-memory slabs: the default) and
    the direct-load form (NCA_BATCH_EXPR_PIPE=0) on arrays whose starts are not
    16-byte aligned, shorter than one vector, and spanning many slabs and
    chunks: extremes and indices equal, sums within the stated bound of the
    oracle."""
    import os
    rng = np.random.default_rng(SEED + 603)
    lens = [1, 3, 5, 17, 4095, 4097, 65539, 1 << 20, (1 << 21) + 7]
    items_h, items, spec = [], [], []
    for i, n in enumerate(lens):
        for dt in (DType.float32, DType.bfloat16, DType.float64, DType.int32):
            h = _host(rng, dt, n + 3)
            d = nca.NCDevArray.from_host(h, dt)
            off = i % 4          # 0..3 elements in: every start alignment
            d, h = d[off:off + n], h[off:off + n]
            pool = INT_PATTERNS if dt == DType.int32 else FLOAT_PATTERNS
            outs = pool[i % len(pool)]
            items.append((d, [(FNS[f], op) for f, op in outs]))
            items_h.append((h, dt))
            spec.append(outs)
    res = {}
    for mode in ("1", "0"):
        old = os.environ.get("NCA_BATCH_EXPR_PIPE")
        os.environ["NCA_BATCH_EXPR_PIPE"] = mode
        try:
            b = _build(items)
            res[mode] = b.run(graph=(mode == "1")) + (b,)
        finally:
            if old is None:
                del os.environ["NCA_BATCH_EXPR_PIPE"]
            else:
                os.environ["NCA_BATCH_EXPR_PIPE"] = old
    v1, i1, b1 = res["1"]
    v0, i0, b0 = res["0"]
    bad = [(k, o, int(i1[k, o]), int(i0[k, o]), items[k][0].size, int(items_h[k][1]), spec[k][o])
           for k in range(len(items)) for o in range(len(spec[k])) if i1[k, o] != i0[k, o]]
    assert not bad, bad[:8]
    _check(orc, b1, items_h, spec, v1, i1)
    _check(orc, b0, items_h, spec, v0, i0)
