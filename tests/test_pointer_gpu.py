"""Operands on a pointer axis (ncarray's NCArray panels: NC semantics, and
PEP 3118 suboffsets: SO semantics) in fused expressions, reductions and
copies, vs the oracle on the stacked logical array. Bit-exact values; float
sums per tests/test_reduce_gpu.py."""
import ctypes

import numpy as np
import pytest

import ncarray_gb300 as nca
from ncarray_gb300 import _lib
from ncarray_gb300.dtype import DType, RedOp
from tests.helpers import SEED, assert_bits_equal, oracle_eval
from tests.test_reduce_gpu import check_reduction

pytestmark = pytest.mark.gpu


def _panels(host):
    return [nca.NCDevArray.from_host(h) for h in host]


def test_fused_expression_over_panels(cuda, orc):
    rng = np.random.default_rng(SEED + 120)
    h = rng.normal(size=(6, 40, 72)).astype(np.float32)
    q = rng.normal(size=(6, 40, 72)).astype(np.float32)
    v = rng.normal(size=72).astype(np.float32)
    P = nca.NCDevArray.from_panels(_panels(h))
    with nca.lazy_mode():
        e = P * nca.NCDevArray.from_host(q) + nca.NCDevArray.from_host(v)
    out = nca.NCDevArray(e.shape, e.dtype)
    e.evaluate(out=out)
    assert_bits_equal(out.to_host(), oracle_eval(orc, e, [h, q, v]), "panels")
    assert_bits_equal(P.to_host(), h, "panels to host")


@pytest.mark.parametrize("op", [RedOp.SUM, RedOp.MAX, RedOp.ARGMAX, RedOp.MIN, RedOp.MEAN])
@pytest.mark.parametrize("axes", [(1, 2), 0, 2, None])
def test_reductions_over_panels(cuda, orc, op, axes):
    rng = np.random.default_rng(SEED + 121)
    h = rng.integers(-50, 50, size=(5, 33, 64)).astype(np.float32)
    P = nca.NCDevArray.from_panels(_panels(h))
    with nca.lazy_mode():
        e = P * 2.0 + 1.0
    (res,) = e.evaluate(reductions=[(op, axes)])
    yr = oracle_eval(orc, e, [h])
    check_reduction(orc, yr, DType.float32, op, axes, res.to_host())


def test_strided_panels_and_slicing(cuda, orc):
    rng = np.random.default_rng(SEED + 122)
    big = rng.integers(-1000, 1000, size=(7, 24, 90)).astype(np.int32)
    d = nca.NCDevArray.from_host(big)
    panels = [d[i, :, ::3] for i in range(7)]            # strided panels (24, 30)
    P = nca.NCDevArray.from_panels(panels)
    h = big[:, :, ::3]
    assert_bits_equal(P.to_host(), h, "strided panels")
    assert_bits_equal(P[1:5].to_host(), h[1:5], "table slice")
    assert_bits_equal(P[::2].to_host(), h[::2], "stepped table (suboffset semantics)")
    assert_bits_equal(P[:, 3:20, ::4].to_host(), h[:, 3:20, ::4], "inner slices")
    assert_bits_equal(P[1:6:2, 5:].to_host(), h[1:6:2, 5:], "stepped table + inner slice")
    assert_bits_equal(P[3].to_host(), h[3], "one panel")
    with nca.lazy_mode():
        e = (P[::2] * 3 + 7) % 11
    out = nca.NCDevArray(e.shape, e.dtype)
    e.evaluate(out=out)
    assert_bits_equal(out.to_host(), oracle_eval(orc, e, [h[::2]]), "int expression over stepped panels")


def test_pointer_axis_not_first_and_suboffsets_abi(cuda):
    """A (2, 3) grid of panels: axis 0 strides the table, axis 1 indexes it
    (NC semantics); and the same data through suboffsets (SO semantics)."""
    import torch
    rng = np.random.default_rng(SEED + 123)
    h = rng.normal(size=(2, 3, 16, 40))
    panels = [[nca.NCDevArray.from_host(h[i, j]) for j in range(3)] for i in range(2)]
    ptrs = np.array([[panels[i][j].ptr for j in range(3)] for i in range(2)], dtype=np.uint64)
    table = nca.NCDevArray.from_host(ptrs)
    out = nca.NCDevArray(h.shape, DType.float64)
    inner = panels[0][0].strides
    v = _lib.make_view(table.ptr, DType.float64, h.shape, (3 * 8, 8) + inner)
    v.pointer_axis = 1
    _lib.call("nca_copy", ctypes.byref(v), ctypes.byref(out.view_struct()), torch.cuda.current_stream().cuda_stream)
    assert_bits_equal(out.to_host(), h, "pointer axis 1")
    # SO: the table holds pointers 64 bytes before each panel; suboffset 64
    ptrs_so = ptrs - np.uint64(64)
    table_so = nca.NCDevArray.from_host(ptrs_so)
    v = _lib.make_view(table_so.ptr, DType.float64, h.shape, (3 * 8, 8) + inner)
    v.pointer_axis = 1
    v.flags = _lib.VIEW_SUBOFFSETS
    v.offsets[1] = 64
    out2 = nca.NCDevArray(h.shape, DType.float64)
    _lib.call("nca_copy", ctypes.byref(v), ctypes.byref(out2.view_struct()), torch.cuda.current_stream().cuda_stream)
    assert_bits_equal(out2.to_host(), h, "suboffsets")
