"""Pixel binning, the reference's own benchmark workload
(examples/benchmark_binning.cu:34-452): the fused sum of strided views times a
scale, on contiguous data and on a panel-table (pointer-axis) view, and the
reshape-and-sum form, vs the oracle. The fused forms are bit-exact (same tape,
same order); the sums follow tests/test_reduce_gpu.py."""
import numpy as np
import pytest

import ncarray_gb300 as nca
from ncarray_gb300.dtype import DType, RedOp
from tests.helpers import SEED, assert_bits_equal, oracle_eval
from tests.test_reduce_gpu import check_reduction

pytestmark = pytest.mark.gpu


def binned_expr(data, bins):
    bp, br, bc = bins
    e = None
    with nca.lazy_mode():
        for p in range(bp):
            for r in range(br):
                for c in range(bc):
                    v = data[p::bp, r::br, c::bc]
                    e = v if e is None else e + v
        return e * (1.0 / (bp * br * bc))


def host_views(h, bins):
    bp, br, bc = bins
    return [h[p::bp, r::br, c::bc] for p in range(bp) for r in range(br) for c in range(bc)]


@pytest.mark.parametrize("shape,bins", [((8, 64, 128), (2, 2, 2)), ((6, 30, 45), (3, 3, 3)), ((4, 16, 64), (1, 4, 4))])
def test_fused_sum_of_views(cuda, orc, shape, bins):
    rng = np.random.default_rng(SEED + 130)
    h = rng.normal(size=shape).astype(np.float32)
    e = binned_expr(nca.NCDevArray.from_host(h), bins)
    out = nca.NCDevArray(e.shape, e.dtype)
    e.evaluate(out=out)
    assert_bits_equal(out.to_host(), oracle_eval(orc, e, host_views(h, bins)), "binned")


def test_fused_sum_of_views_on_panels(cuda, orc):
    rng = np.random.default_rng(SEED + 131)
    h = rng.normal(size=(8, 64, 128)).astype(np.float32)
    P = nca.NCDevArray.from_panels([nca.NCDevArray.from_host(x) for x in h])
    e = binned_expr(P, (2, 2, 2))
    out = nca.NCDevArray(e.shape, e.dtype)
    e.evaluate(out=out)
    assert_bits_equal(out.to_host(), oracle_eval(orc, e, host_views(h, (2, 2, 2))), "binned panels")


@pytest.mark.parametrize("op", [RedOp.SUM, RedOp.MEAN, RedOp.MAX])
def test_reshape_sum(cuda, orc, op):
    """data.reshape(P/2, 2, R/2, 2, C/2, 2) reduced over axes (1, 3, 5): eight
    elements per output, one thread per output."""
    rng = np.random.default_rng(SEED + 132)
    h = rng.normal(size=(8, 64, 128)).astype(np.float32)
    d = nca.NCDevArray.from_host(h).reshape(4, 2, 32, 2, 64, 2)
    (res,) = d._expr().evaluate(reductions=[(op, (1, 3, 5))])
    check_reduction(orc, h.reshape(4, 2, 32, 2, 64, 2), DType.float32, op, (1, 3, 5), res.to_host())
