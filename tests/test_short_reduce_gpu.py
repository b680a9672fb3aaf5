"""Short inner reductions (one thread per kept position, at most 8 vectors
each, no splits): the form that gathers the operands of 2 (or 3, 4, 8) kept
positions before reducing any of them (default 2) against one position at a
time (NCA_K3_UNITS=1), bit for bit, and both against the oracle.

Cases: the pixel binning as reshape(16, 2, 256, 2, 512, 2).sum((1, 3, 5))
(three reduced dims of 2), rows of 8 and of 6 elements, two reduced dims of
3 x 5, an expression over two operands, and float32 / int32 / bfloat16 /
float64 values; sums, extremes and their indices."""
import os

import numpy as np
import pytest

import ncarray_gb300 as nca
from ncarray_gb300.dtype import DType, RedOp
from tests.helpers import SEED, rand
from tests.test_reduce_gpu import check_reduction

pytestmark = pytest.mark.gpu


def _both(fn, units_many=None):
    got = []
    for units in ("1", units_many):
        old = os.environ.get("NCA_K3_UNITS")
        if units is None:
            os.environ.pop("NCA_K3_UNITS", None)
        else:
            os.environ["NCA_K3_UNITS"] = units
        try:
            got.append([r.to_host() for r in fn()])
        finally:
            if old is None:
                os.environ.pop("NCA_K3_UNITS", None)
            else:
                os.environ["NCA_K3_UNITS"] = old
    return got


@pytest.mark.parametrize("dt", [DType.float32, DType.int32, DType.bfloat16, DType.float64])
def test_short_rows_and_boxes(cuda, orc, dt):
    rng = np.random.default_rng(SEED + 1500 + int(dt))
    cases = [((4, 2, 32, 2, 100, 2), (1, 3, 5)), ((100003, 8), 1), ((7001, 6), 1), ((64, 3, 50, 5), (1, 3))]
    for shape, axes in cases:
        h = rand(rng, shape, dt)
        d = nca.NCDevArray.from_host(h, dt)
        for op in (RedOp.SUM, RedOp.MAX, RedOp.ARGMIN):
            one, many = _both(lambda: d._expr().evaluate(reductions=[(op, axes)]))
            assert one[0].tobytes() == many[0].tobytes(), (shape, op)
            check_reduction(orc, h, dt, op, axes, many[0])
        for units in ("3", "8"):
            one, many = _both(lambda: d._expr().evaluate(reductions=[(RedOp.SUM, axes)]), units)
            assert one[0].tobytes() == many[0].tobytes(), (shape, units)


def test_binning_reshape_full_size(cuda, orc):
    rng = np.random.default_rng(SEED + 1510)
    img = rng.normal(size=(32, 512, 1024)).astype(np.float32)
    d = nca.NCDevArray.from_host(img)
    six = d.reshape(16, 2, 256, 2, 512, 2)
    one, many = _both(lambda: six._expr().evaluate(reductions=[(RedOp.SUM, (1, 3, 5)), (RedOp.MAX, (1, 3, 5))]))
    for a, b in zip(one, many):
        assert a.tobytes() == b.tobytes()
    h6 = img.reshape(16, 2, 256, 2, 512, 2)
    check_reduction(orc, h6, DType.float32, RedOp.SUM, (1, 3, 5), many[0])
    assert np.array_equal(many[1], h6.max(axis=(1, 3, 5)))


def test_expression_of_two_operands(cuda):
    rng = np.random.default_rng(SEED + 1520)
    a = rng.normal(size=(5000, 8)).astype(np.float32)
    b = rng.normal(size=(5000, 8)).astype(np.float32)
    da, db = nca.NCDevArray.from_host(a), nca.NCDevArray.from_host(b)

    def run():
        with nca.lazy_mode():
            e = da * db - da
        return e.evaluate(reductions=[(RedOp.SUM, 1), (RedOp.ARGMAX, 1)])

    one, many = _both(run)
    for x, y in zip(one, many):
        assert x.tobytes() == y.tobytes()
    assert np.array_equal(many[1], (a * b - a).argmax(axis=1))
