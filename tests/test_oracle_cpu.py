"""Pins the oracle restatement (oracle/oracle.c) to the reference implementation.

1. Against the committed golden vectors of tests/golden/ref_golden.npz, which
   tests/golden/make_golden.py produced by running ncarray's own host code
   (its stack VM and ArrayImpl reductions) -- runs everywhere.
2. Directly against oracle/_ref (the reference compiled from its sources)
   where that library exists.
3. Against the known answers of the reference's own tests.

Expression outputs, integer sums, max/min and arg-reductions must be
bit-exact. Float sums and means are compared with the reference's own error
bound (it accumulates float32 in float32: |err| <= n * 2^-24 * sum|x|)."""
import json
from pathlib import Path

import numpy as np
import pytest

from tests.helpers import SEED

GOLDEN = Path(__file__).resolve().parent / "golden" / "ref_golden.npz"


def golden():
    z = np.load(GOLDEN)
    meta = json.loads(bytes(z["meta"]).decode())
    return z, meta


def test_golden_expressions(orc):
    z, meta = golden()
    n = 0
    for i, m in enumerate(meta):
        if m["kind"] != "expr":
            continue
        ops = [(z[f"e{i}_op{k}"], d) for k, d in enumerate(m["op_dtypes"])]
        want = z[f"e{i}_out"]
        compute = m["work"] if m["expr"] == 0 else m["expr"]
        got = orc.expr_eval(m["instrs"], [tuple(s) for s in m["scalars"]], compute, ops, want.shape, m["expr"])
        assert got.tobytes() == want.tobytes(), m["name"]
        n += 1
    assert n >= 30


def _float_sum_bound(h, axis=None):
    a = np.abs(h.astype(np.float64))
    cnt = h.size if axis is None else np.prod([h.shape[d] for d in axis])
    s = a.sum() if axis is None else a.sum(axis=tuple(axis))
    return cnt * 2.0**-24 * s + 1e-30


def test_golden_reductions(orc):
    z, meta = golden()
    for i, m in enumerate(meta):
        if m["kind"] != "reduce":
            continue
        h, dt = z[f"r{i}_in"], m["dtype"]
        isf = dt in (10, 11)
        for op_s, (val, odt) in m["full"].items():
            op = int(op_s)
            got = orc.reduce(h, dt, op)
            if op in (0, 1) and isf:
                assert abs(float(got) - float(val)) <= _float_sum_bound(h) / (h.size if op == 1 else 1)
            elif op == 1:
                assert float(got) == pytest.approx(float(val), rel=1e-12)
            else:
                assert odt == orc.red_out_dtype(op, dt), (dt, op)
                assert got.item() == val, (dt, op, got, val)
        for key, odt in m["axes"].items():
            op, axes = int(key.split("_")[0]), [int(x) for x in key.split("_")[1:]]
            want = z[f"r{i}_ax_{key}"]
            got = orc.reduce(h, dt, op, axes)
            assert odt == orc.red_out_dtype(op, dt)
            if op == 0 and isf:
                assert np.all(np.abs(got - want) <= _float_sum_bound(h, axes))
            else:
                assert got.tobytes() == want.tobytes(), (dt, key)


def test_direct_against_reference_vm(orc):
    """Random tapes through the reference VM (when oracle/_ref exists)."""
    if orc.ref() is None:
        pytest.skip("reference host code not built on this machine")
    rng = np.random.default_rng(SEED + 7)
    I = lambda op, i=0: (op << 24) | i  # noqa: E731
    for trial in range(60):
        dt = int(rng.choice([2, 4, 6, 7, 8, 9, 10, 11]))
        shape = (2, 3, 11)
        np_dt = orc.np_dtype(dt)
        if dt in (10, 11):
            a, b = rng.normal(size=shape).astype(np_dt), rng.normal(size=shape).astype(np_dt)
        else:
            a, b = rng.integers(1, 100, shape).astype(np_dt), rng.integers(1, 100, shape).astype(np_dt)
        ops = [14, 15, 16, 18, 20, 22, 24, 26, 27]
        instrs = [I(2, 0), I(2, 1), I(int(rng.choice(ops))), I(2, 0), I(int(rng.choice([14, 16])))]
        op_last = instrs[-1] >> 24
        expr = {14: {2: 5, 6: 9, 7: 9}.get(dt, dt), 16: dt}[op_last]
        want = orc.ref_expr_eval(instrs, [], dt, expr, [(a, dt), (b, dt)], shape)
        got = orc.expr_eval(instrs, [], expr, [(a, dt), (b, dt)], shape, expr)
        assert got.tobytes() == want.tobytes(), (trial, dt, instrs)


def test_reference_known_answers(orc):
    """tests/cxx/test_gpu_reductions.cu:191-294, test_reductions.cc:26-38,
    test_binary_operations.cc:216-230."""
    f = np.arange(256, dtype=np.float32)
    assert orc.reduce(f, 10, 0) == 32640.0 and orc.reduce(f, 10, 2) == 255.0 and orc.reduce(f, 10, 3) == 0.0
    i = np.arange(1, 7, dtype=np.int32).reshape(2, 3)
    assert np.array_equal(orc.reduce(i, 8, 0, [0]), [5, 7, 9])
    assert np.array_equal(orc.reduce(i, 8, 0, [1]), [6, 15])
    assert np.array_equal(orc.reduce(i, 8, 2, [0]), [4, 5, 6])
    assert np.array_equal(orc.reduce(i, 8, 3, [1]), [1, 4])
    s = np.ones((4, 4), dtype=np.int32)
    s[1:3, 1:3] = 10
    assert orc.reduce(s, 8, 0) == 52
    t = orc.reduce(np.ones((10, 2), dtype=np.int32), 8, 0)
    assert t.dtype == np.int32 and t == 20
    u = np.array([7, 8, 9], dtype=np.uint32)
    I = lambda op, i=0: (op << 24) | i  # noqa: E731
    got = orc.expr_eval([I(2, 0), I(4, 0), I(18)], [(2, 4)], 4, [(u, 4)], (3,), 4)
    assert np.array_equal(got, [3, 0, 1])


def test_stencil_oracle_properties(orc):
    """Zero weights keep the grid; a constant interior is a fixed point of the
    zero-sum 7-point Laplacian away from the zero halo."""
    rng = np.random.default_rng(SEED + 2)
    u = rng.normal(size=(6, 7, 8))
    w = np.zeros(27)
    assert np.array_equal(orc.stencil3d_f64(u, w, 0.1, 3), u)
    w7 = np.zeros(27)
    w7[13] = -6.0
    for idx in (4, 10, 12, 14, 16, 22):
        w7[idx] = 1.0
    c = np.full((5, 5, 5), 2.0)
    r = orc.stencil3d_f64(c, w7, 0.1, 1)
    assert r[2, 2, 2] == 2.0 and r[0, 0, 0] == 2.0 + 0.1 * (-3 * 2.0)


def test_hist_oracle_small(orc):
    x = np.array([0.0, 0.5, 0.999, 1.0, -0.1, np.nan, 0.25], dtype=np.float32)
    y = np.array([0.0, 0.5, 0.999, 0.5, 0.5, 0.5, 0.75], dtype=np.float32)
    w = np.arange(7, dtype=np.float32)
    counts, ws = orc.hist2d(x, y, w, 4, 4, 0.0, 1.0, 0.0, 1.0)
    c = counts.reshape(4, 4)
    assert c[0, 0] == 1 and c[2, 2] == 1 and c[3, 3] == 1 and c[3, 1] == 1 and c.sum() == 4
    assert ws.reshape(4, 4)[3, 1] == 6.0


def test_oracle_bitwise_ops_match_numpy(orc):
    """BAND/BOR/XOR/BNOT (which the reference VM skips) are defined as two's
    complement operations in the compute type; the oracle agrees with numpy."""
    rng = np.random.default_rng(7)
    a = rng.integers(-2**31, 2**31, size=257, dtype=np.int64).astype(np.int32)
    b = rng.integers(-2**31, 2**31, size=257, dtype=np.int64).astype(np.int32)
    L = lambda i: (2 << 24) | i  # noqa: E731  LOAD_NCARR i
    for op, want in ((28, a & b), (29, a | b), (30, a ^ b)):
        got = orc.expr_eval([L(0), L(1), op << 24], [], 8, [(a, 8), (b, 8)], a.shape, 8)
        assert np.array_equal(got, want), op
    got = orc.expr_eval([L(0), 13 << 24], [], 8, [(a, 8)], a.shape, 8)
    assert np.array_equal(got, ~a)


def test_golden_stencil(orc):
    """orc_stencil3d_f64 against the reference's VM over 27 shifted views of a
    zero-padded grid (7-point, 27-point and an asymmetric weight set, 1-3
    Jacobi steps): bit-exact."""
    z, meta = golden()
    n = 0
    for i, m in enumerate(meta):
        if m["kind"] != "stencil":
            continue
        got = orc.stencil3d_f64(z[f"s{i}_in"], z[f"s{i}_w"], m["dt"], m["iters"])
        assert got.tobytes() == z[f"s{i}_out"].tobytes(), m["name"]
        n += 1
    assert n == 3


def test_golden_hist(orc):
    """orc_hist2d against host::scatter_add_recursive of the reference fed the
    float32 bin indices (counts uint64, weights summed in float64 in point
    order): bit-exact, including NaN, inf, -0.0 and out-of-range points."""
    z, meta = golden()
    n = 0
    for i, m in enumerate(meta):
        if m["kind"] != "hist":
            continue
        counts, wsum = orc.hist2d(z[f"h{i}_x"], z[f"h{i}_y"], z[f"h{i}_w"], m["nbx"], m["nby"], *m["xr"], *m["yr"])
        assert np.array_equal(counts, z[f"h{i}_counts"])
        assert wsum.tobytes() == z[f"h{i}_wsum"].tobytes()
        n += 1
    assert n == 2


def test_golden_batch(orc):
    """orc_batch_reduce (float64, compensated) against the reference's
    ArrayImpl::sum/mean/max and the sum of its VM's x*x - x, per array: max
    bit-exact; sums and means within the reference's own float32 error
    (it accumulates float32 in float32, and rounds x*x - x to float32)."""
    z, meta = golden()
    cases = [(i, m) for i, m in enumerate(meta) if m["kind"] == "batch"]
    assert len(cases) == 12
    got = orc.batch_reduce([z[f"b{i}_x"] for i, _ in cases], [m["dtype"] for _, m in cases])
    for (i, m), g in zip(cases, got):
        raw = z[f"b{i}_x"]
        x = ((raw.astype(np.uint32) << 16).view(np.float32) if m["dtype"] == 22 else raw).astype(np.float64)
        n = x.size
        ref = {k: v[0] for k, v in m["ref"].items()}
        assert g[2] == ref["max"]
        b1 = (n + 1) * 2.0**-24 * np.abs(x).sum()
        assert abs(g[0] - ref["sum"]) <= b1
        assert abs(g[1] - ref["mean"]) <= b1 / n
        b2 = (n + 3) * 2.0**-24 * (x * x + np.abs(x)).sum()
        assert abs(g[3] - ref["sum_sq_m"]) <= b2


def test_golden_scatter(orc):
    """orc_scatter_add against host::scatter_add_recursive (dest dtype x index
    dtype x source dtype, negative and too-large indices dropped): bit-exact."""
    z, meta = golden()
    n = 0
    for i, m in enumerate(meta):
        if m["kind"] != "scatter":
            continue
        want = z[f"x{i}_dest"]
        dest = np.zeros_like(want)
        orc.scatter_add(dest, m["dest"], z[f"x{i}_idx"], m["idx"], z[f"x{i}_src"], m["src"])
        assert dest.tobytes() == want.tobytes(), m
        n += 1
    assert n == 6
