"""Expressions and a stencil that ncarray's own code built (through the drop-in
engine, tests/dropin/check_dropin.cu; descriptors in
tests/golden/dropin_cases.json) evaluated on the GPU through the C ABI
(nca_expr_eval, nca_stencil) on seeded data, bit for bit against the oracle
evaluating the same tape over the same logical operand values."""
import ctypes
import json

import numpy as np
import pytest

from ncarray_gb300 import _lib
from ncarray_gb300.dtype import ITEMSIZE, DType
from tests.dropin import cases as dropin
from tests.helpers import SEED

pytestmark = pytest.mark.gpu

FIX = json.loads(dropin.FIXTURE.read_text())
NP = {8: np.int32, 10: np.float32, 11: np.float64}


def _tape(desc):
    ins = (ctypes.c_uint32 * len(desc["instrs"]))(*desc["instrs"])
    sd = (ctypes.c_int32 * max(len(desc["scalars"]), 1))(*[d for d, _ in desc["scalars"]])
    ss = (ctypes.c_uint64 * max(len(desc["scalars"]), 1))(*[v for _, v in desc["scalars"]])
    t = _lib.Tape()
    t.instrs = ctypes.cast(ins, ctypes.POINTER(ctypes.c_uint32))
    t.n_instrs = len(desc["instrs"])
    t.n_scalars = len(desc["scalars"])
    t.scalar_dtypes = ctypes.cast(sd, ctypes.POINTER(ctypes.c_int32))
    t.scalar_slots = ctypes.cast(ss, ctypes.POINTER(ctypes.c_uint64))
    t.compute_dtype = desc["compute"]
    t.result_dtype = desc["result"]
    return t, (ins, sd, ss)


def _view(op, data_ptr):
    v = _lib.make_view(data_ptr, op["dtype"], op["shape"], op["strides"])
    for d, o in enumerate(op["offsets"]):
        v.offsets[d] = o
    v.pointer_axis = op["pointer_axis"]
    v.flags = op["flags"]
    return v


def _seeded(rng, dt, n):
    if dt == 8:
        return rng.integers(-1000, 1000, n).astype(np.int32)
    return rng.normal(size=n).astype(NP[dt])


def _span(op, dims):
    """Bytes a view reaches over `dims` from its start (offsets included)."""
    isz = ITEMSIZE[DType(op["dtype"])]
    return sum(op["offsets"][d] + (op["shape"][d] - 1) * abs(op["strides"][d]) for d in dims) + isz


@pytest.mark.parametrize("name", ["c1_core", "c2_y", "c2_int", "panels"])
def test_ncarray_built_expression(cuda, orc, name):
    torch = cuda
    case = next(c for c in FIX if c.get("name") == name)
    rng = np.random.default_rng(SEED + 500)
    host, dev, keep, views, logical = {}, {}, [], [], []
    for op in case["operands"]:
        nd = len(op["shape"])
        dt, isz = op["dtype"], ITEMSIZE[DType(op["dtype"])]
        pa = op["pointer_axis"]
        if pa < 0:
            b = op["buffer"]
            if b not in host:
                # every view of this buffer in the case must fit it
                need = max(_span(o, range(len(o["shape"]))) for o in case["operands"] if o["buffer"] == b
                           and o["pointer_axis"] < 0)
                host[b] = _seeded(rng, dt, need // isz + 1)
                dev[b] = torch.from_numpy(host[b]).cuda()
            views.append(_view(op, dev[b].data_ptr()))
            start = sum(op["offsets"]) // isz
            logical.append(np.lib.stride_tricks.as_strided(host[b][start:], op["shape"], op["strides"]))
        else:
            # NC pointer axis 0: a table of panel pointers, index offset offsets[0]
            assert pa == 0 and op["flags"] == 0
            n_tab = op["shape"][0] + op["offsets"][0]
            panel_bytes = _span(op, range(1, nd))
            panels = [_seeded(rng, dt, panel_bytes // isz + 1) for _ in range(n_tab)]
            dpan = [torch.from_numpy(p).cuda() for p in panels]
            table = torch.tensor([p.data_ptr() for p in dpan], dtype=torch.int64).cuda()
            keep += dpan + [table]
            views.append(_view(op, table.data_ptr()))
            pstart = sum(op["offsets"][1:]) // isz
            rows = [np.lib.stride_tricks.as_strided(panels[i + op["offsets"][0]][pstart:], op["shape"][1:],
                                                    op["strides"][1:]) for i in range(op["shape"][0])]
            logical.append(np.stack(rows))
    res_dt = case["tape"]["result"]
    out = torch.zeros(int(np.prod(case["out_shape"])), dtype={8: torch.int32, 10: torch.float32,
                                                               11: torch.float64}[res_dt]).cuda()
    isz = ITEMSIZE[DType(res_dt)]
    st, acc = [], isz
    for n in reversed(case["out_shape"]):
        st.append(acc)
        acc *= n
    ov = _lib.make_view(out.data_ptr(), res_dt, case["out_shape"], list(reversed(st)))
    t, _k = _tape(case["tape"])
    arr = (_lib.View * len(views))(*views)
    _lib.call("nca_expr_eval", ctypes.byref(t), arr, len(views), ctypes.byref(ov),
              torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = out.cpu().numpy().reshape(case["out_shape"])
    want = orc.expr_eval(case["tape"]["instrs"], [tuple(s) for s in case["tape"]["scalars"]], case["tape"]["compute"],
                         [(np.ascontiguousarray(a), op["dtype"]) for a, op in zip(logical, case["operands"])],
                         tuple(case["out_shape"]), res_dt)
    assert got.tobytes() == want.tobytes(), name


def test_ncarray_built_stencil(cuda, orc):
    """The binning stencil ncarray's Stencil<3>::create built, applied by
    nca_stencil to a (6, 10, 14) float32 source into (3, 5, 7)."""
    torch = cuda
    case = next(c for c in FIX if c.get("name") == "binning_2x2x2")
    rng = np.random.default_rng(SEED + 501)
    src = rng.normal(size=(6, 10, 14)).astype(np.float32)
    dsrc = torch.from_numpy(src).cuda()
    out = torch.zeros(3 * 5 * 7, dtype=torch.float32).cuda()
    sv = _lib.make_view(dsrc.data_ptr(), 10, (6, 10, 14), (560, 56, 4))
    dv = _lib.make_view(out.data_ptr(), 10, (3, 5, 7), (140, 28, 4))
    offs = case["offsets"]
    n = len(offs) // 3
    c_offs = (ctypes.c_int64 * len(offs))(*offs)
    t, _k = _tape(case["tape"])
    _lib.call("nca_stencil", ctypes.byref(sv), ctypes.byref(dv), c_offs, n, ctypes.byref(t),
              torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    views = []
    for i in range(n):
        o = offs[3 * i: 3 * i + 3]
        views.append((np.ascontiguousarray(src[o[0]:o[0] + 5:2, o[1]:o[1] + 9:2, o[2]:o[2] + 13:2]), 10))
    want = orc.expr_eval(case["tape"]["instrs"], [tuple(s) for s in case["tape"]["scalars"]],
                         case["tape"]["compute"], views, (3, 5, 7), case["tape"]["result"])
    assert out.cpu().numpy().reshape(3, 5, 7).tobytes() == want.tobytes()
