"""Operands strided by two elements along the innermost axis (the pixel-binning
views a[..., 0::2], a[..., 1::2] of examples/benchmark_binning.cu:34-452):
the ND kernel reads whole aligned windows of two vectors and keeps every other
lane, the even and odd phases of one array sharing the loads. Every case is
compared bit for bit with the oracle on the same tape, including the layouts
that must fall back to scalar loads (a window start off the 16-byte grid, row
strides that are not 16-byte multiples)."""
import numpy as np
import pytest

import ncarray_gb300 as nca
from ncarray_gb300.dtype import DType
from tests.helpers import SEED, assert_bits_equal, oracle_eval, rand

pytestmark = pytest.mark.gpu


def run(expr, pairs, orc, what):
    """Evaluates expr on the device and the oracle; pairs maps device views to host views."""
    out = nca.NCDevArray(expr.shape, expr.dtype)
    expr.evaluate(out=out)
    host = {id(d): h for d, h in pairs}
    want = oracle_eval(orc, expr, [host[id(a)] for a in expr.arrays])
    assert_bits_equal(out.to_host(), want, what)


@pytest.mark.parametrize("dt", [DType.float32, DType.float64, DType.float16, DType.bfloat16, DType.int32,
                                DType.int16, DType.uint8])
def test_even_plus_odd(cuda, orc, dt):
    """d[:, 0::2] + d[:, 1::2]: two phases of one window (shared loads)."""
    rng = np.random.default_rng(SEED + 140)
    h = rand(rng, (16, 512), dt)
    d = nca.NCDevArray.from_host(h, dt)
    a, b = d[:, 0::2], d[:, 1::2]
    with nca.lazy_mode():
        e = a + b
    run(e, [(a, h[:, 0::2]), (b, h[:, 1::2])], orc, f"even+odd {dt.name}")


@pytest.mark.parametrize("start", [0, 1, 2, 3, 4, 5])
def test_phases_alone(cuda, orc, start):
    """One strided operand from each start element: starts 0, 1, 4, 5 read
    windows (float32: 16-byte grid, lane 0 or 1), 2 and 3 fall back."""
    rng = np.random.default_rng(SEED + 141 + start)
    h = rand(rng, (8, 40 + 2 * 64), DType.float32)
    d = nca.NCDevArray.from_host(h)
    a = d[:, start:start + 128:2]
    with nca.lazy_mode():
        e = a * 3.0 - 1.0
    run(e, [(a, h[:, start:start + 128:2])], orc, f"start {start}")


def test_row_strides_off_grid(cuda, orc):
    """Rows of 34 float32 (136 bytes): the windows would leave the 16-byte
    grid on odd rows, so the planner keeps scalar loads."""
    rng = np.random.default_rng(SEED + 150)
    h = rand(rng, (9, 34), DType.float32)
    d = nca.NCDevArray.from_host(h)
    a, b = d[:, 0:32:2], d[:, 1:33:2]
    with nca.lazy_mode():
        e = a - b
    run(e, [(a, h[:, 0:32:2]), (b, h[:, 1:33:2])], orc, "off-grid rows")


def test_last_window_of_a_row(cuda, orc):
    """d[:, 0:16:2] + d[:, 1:17:2] on rows of 24: the last window of every row
    ends at element 15; the elements after it are never needed."""
    rng = np.random.default_rng(SEED + 151)
    h = rand(rng, (5, 24), DType.float32)
    d = nca.NCDevArray.from_host(h)
    a, b = d[:, 0:16:2], d[:, 1:17:2]
    with nca.lazy_mode():
        e = a + b
    run(e, [(a, h[:, 0:16:2]), (b, h[:, 1:17:2])], orc, "last window")


def test_mixed_with_contiguous_broadcast_scalar(cuda, orc):
    """Pairs next to a contiguous operand, a broadcast row and a scalar."""
    rng = np.random.default_rng(SEED + 152)
    h = rand(rng, (32, 256), DType.float32)
    c = rand(rng, (32, 128), DType.float32)
    r = rand(rng, (128,), DType.float32)
    d = nca.NCDevArray.from_host(h)
    dc, dr = nca.NCDevArray.from_host(c), nca.NCDevArray.from_host(r)
    a, b = d[:, 0::2], d[:, 1::2]
    rb = dr.reshape(1, 128)
    with nca.lazy_mode():
        e = (a * b + dc) * rb - a * 0.5
    run(e, [(a, h[:, 0::2]), (b, h[:, 1::2]), (dc, c), (rb, r.reshape(1, 128))], orc, "mixed")


@pytest.mark.parametrize("bins", [(2, 2, 2), (4, 2, 2), (1, 1, 2)])
def test_binning_pairs(cuda, orc, bins):
    """Sum of strided views with a pair of phases along the innermost axis."""
    rng = np.random.default_rng(SEED + 153)
    h = rand(rng, (8, 32, 256), DType.float32)
    d = nca.NCDevArray.from_host(h)
    bp, br, bc = bins
    pairs, e = [], None
    with nca.lazy_mode():
        for p in range(bp):
            for r_ in range(br):
                for c_ in range(bc):
                    v = d[p::bp, r_::br, c_::bc]
                    pairs.append((v, h[p::bp, r_::br, c_::bc]))
                    e = v if e is None else e + v
        e = e * (1.0 / (bp * br * bc))
    run(e, pairs, orc, f"binning {bins}")


@pytest.mark.parametrize("layout", ["aligned", "offset", "alternating"])
def test_binning_pairs_on_panels(cuda, orc, layout):
    """The binning views on a table of panels (pointer axis): window loads
    where a panel is on the 16-byte grid, scalar loads where it is not
    (panels starting one element in), chosen per panel at run time."""
    rng = np.random.default_rng(SEED + 154)
    P, R, C = 8, 32, 128
    h = rand(rng, (P, R, C), DType.float32)
    if layout == "aligned":
        panels = [nca.NCDevArray.from_host(h[i]) for i in range(P)]
    else:
        # rows of C + 4 elements (16-byte multiples); a panel starts 0 or 1 element in
        big = np.zeros((P, R, C + 4), np.float32)
        starts = [1] * P if layout == "offset" else [i % 2 for i in range(P)]
        for i in range(P):
            big[i, :, starts[i]:starts[i] + C] = h[i]
        dbig = nca.NCDevArray.from_host(big)
        panels = [dbig[i][:, starts[i]:starts[i] + C] for i in range(P)]
    T = nca.NCDevArray.from_panels(panels)
    pairs, e = [], None
    with nca.lazy_mode():
        for p in range(2):
            for r_ in range(2):
                for c_ in range(2):
                    v = T[p::2, r_::2, c_::2]
                    pairs.append((v, h[p::2, r_::2, c_::2]))
                    e = v if e is None else e + v
        e = e * 0.125
    run(e, pairs, orc, f"panels {layout}")
