"""The drop-in engine (include/ncarray_dropin) against ncarray's own code.

Where the reference sources are present, tests/dropin/check_dropin.cu is
compiled with nvcc against ncarray's headers with the drop-in directory first,
linked against libncgb300 (every engine path ncarray's device API takes is
instantiated), and run without a GPU: its descriptors of expressions, a
stencil and reduction-axis sets built by ncarray's own code must equal the
committed fixture that the GPU test replays. Everywhere, the fixture must agree
with the tapes this package's Python layer builds for the same expressions."""
import json

import pytest

from ncarray_gb300.array import DevExpr, lazy_mode
from ncarray_gb300.dtype import DType
from ncarray_gb300.stencil import Stencil, _Slot
from tests.dropin import cases as dropin

FIX = json.loads(dropin.FIXTURE.read_text())


def _by_name(name):
    return next(c for c in FIX if c.get("name") == name)


def test_fixture_matches_ncarray_build(built_lib):
    if not dropin.have_reference():
        pytest.skip("reference sources not present")
    assert dropin.build_and_run() == FIX


def test_reduction_axes_masks():
    """build_reduction_params of {0}, {2}, {1,3}, all, {3} on 4 dims."""
    axes = next(c for c in FIX if c["kind"] == "axes")
    assert axes["masks"] == [0b1, 0b100, 0b1010, 0b1111, 0b1000]


def test_python_layer_builds_the_same_tapes():
    """(k*3+7)%11 and x*v+k: the ncarray-built tapes equal this package's."""
    k = _Slot(2, DType.int32, 4)
    with lazy_mode():
        z = (DevExpr.leaf(k) * 3 + 7) % 11
    want = _by_name("c2_int")["tape"]
    assert z.instrs == want["instrs"]
    # same values; a C++ int literal is int32, the Python binding takes the
    # smallest type that holds the value (uint8): the compute dtype is int32 either way
    assert [s for _, s in z.scalars] == [s for _, s in want["scalars"]]
    assert int(z.expr_dtype) == want["compute"] == int(DType.int32)
    x, v = _Slot(0, DType.float32, 4), _Slot(1, DType.float32, 4)
    with lazy_mode():
        y = x * v + k
    assert y.instrs == _by_name("c2_y")["tape"]["instrs"]


def test_stencil_descriptor_matches_python_stencil():
    offs = [(p, r, c) for p in range(2) for r in range(2) for c in range(2)]

    def binning(views):
        e = DevExpr.leaf(views[0])
        for v in views[1:]:
            e = e + v
        return e * 0.125

    st = Stencil.create(offs, binning, DType.float32)
    want = _by_name("binning_2x2x2")
    assert list(st._ins) == want["tape"]["instrs"]
    assert [v for o in offs for v in o] == want["offsets"]
    assert st._tape.compute_dtype == want["tape"]["compute"]
