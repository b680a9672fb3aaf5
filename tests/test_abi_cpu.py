"""CPU checks of the C ABI: the library loads without a GPU, exports every
symbol include/ncgb300.h declares, compiles every JIT kernel class with NVRTC
for sm_103a, and rejects malformed requests before touching a device."""
import ctypes
import re
from pathlib import Path

import numpy as np

from ncarray_gb300 import _lib
from ncarray_gb300.dtype import DType, OpCode

HEADER = Path(__file__).resolve().parent.parent / "include" / "ncgb300.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nca_[a-z0-9_]+)\s*\(", text)))


def test_exports_every_declared_symbol(built_lib):
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(built_lib, n)]
    assert not missing, f"not exported: {missing}"
    assert set(_lib.EXPORTS) >= set(names), "python binding lacks declared functions"


def test_version_and_stats(built_lib):
    assert built_lib.nca_version() >= 1000
    c, d, m = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    _lib.call("nca_jit_stats", ctypes.byref(c), ctypes.byref(d), ctypes.byref(m))


def test_nvrtc_compiles_every_kernel_class(built_lib):
    n = ctypes.c_int32(0)
    _lib.call("nca_jit_selftest", b"sm_103a", ctypes.byref(n))
    assert n.value == 132


def _tape(instrs, cdt=DType.float32, rdt=DType.float32):
    arr = (ctypes.c_uint32 * len(instrs))(*instrs)
    t = _lib.Tape()
    t.instrs = ctypes.cast(arr, ctypes.POINTER(ctypes.c_uint32))
    t.n_instrs = len(instrs)
    t.n_scalars = 0
    t.compute_dtype = int(cdt)
    t.result_dtype = int(rdt)
    return t, arr


def _view(shape, dt=DType.float32):
    isz = 4
    st, acc = [], isz
    for n in reversed(shape):
        st.append(acc)
        acc *= n
    return _lib.make_view(0x1000, dt, shape, list(reversed(st)))


def _status(name, *args):
    return getattr(_lib.lib(), name)(*args)


def test_malformed_tapes_rejected(built_lib):
    L = _lib.lib()
    out = _view([4])
    ops = (_lib.View * 1)(_view([4]))
    cases = [
        ([OpCode.ADD << 24], _lib.ERR_INVALID),                                       # underflow
        ([OpCode.LOAD_NCARR << 24, OpCode.LOAD_NCARR << 24], _lib.ERR_INVALID),         # 2 values left
        ([(OpCode.LOAD_NCARR << 24) | 3], _lib.ERR_INVALID),                           # operand 3 of 1
        ([8 << 24], _lib.ERR_UNSUPPORTED),                                             # SZOF
        ([OpCode.LOAD_NCARR << 24, OpCode.LOAD_NCARR << 24, OpCode.BAND << 24], _lib.ERR_DTYPE),
    ]
    for instrs, want in cases:
        t, keep = _tape(instrs)
        rc = L.nca_expr_eval(ctypes.byref(t), ops, 1, ctypes.byref(out), None)
        assert rc == want, (instrs, rc, L.nca_last_error())
        assert L.nca_last_error()


def test_bad_views_rejected(built_lib):
    L = _lib.lib()
    t, keep = _tape([OpCode.LOAD_NCARR << 24])
    out = _view([4])
    bad = _view([5])
    ops = (_lib.View * 1)(bad)
    assert L.nca_expr_eval(ctypes.byref(t), ops, 1, ctypes.byref(out), None) == _lib.ERR_SHAPE
    # pointer axes: accepted on operands, rejected on results, checked for range and flags
    good = (_lib.View * 1)(_view([4]))
    pout = _view([4])
    pout.pointer_axis = 0
    assert L.nca_expr_eval(ctypes.byref(t), good, 1, ctypes.byref(pout), None) == _lib.ERR_UNSUPPORTED
    prange = _view([4])
    prange.pointer_axis = 1
    ops = (_lib.View * 1)(prange)
    assert L.nca_expr_eval(ctypes.byref(t), ops, 1, ctypes.byref(out), None) == _lib.ERR_INVALID
    pflags = _view([4])
    pflags.flags = 1          # suboffset semantics without a pointer axis
    ops = (_lib.View * 1)(pflags)
    assert L.nca_expr_eval(ctypes.byref(t), ops, 1, ctypes.byref(out), None) == _lib.ERR_INVALID
    cplx = _view([4], DType.float32)
    cplx.dtype = 13
    ops = (_lib.View * 1)(cplx)
    assert L.nca_expr_eval(ctypes.byref(t), ops, 1, ctypes.byref(out), None) == _lib.ERR_DTYPE
    big = _view([4])
    big.ndim = 11
    assert L.nca_expr_eval(ctypes.byref(t), ops, 1, ctypes.byref(big), None) == _lib.ERR_LIMIT


def test_reduction_dtype_and_shape_checked(built_lib):
    L = _lib.lib()
    src = _view([4, 6])
    out = _view([6], DType.float64)  # sum of float32 is float32
    assert L.nca_reduce(ctypes.byref(src), 0, 1, ctypes.byref(out), None) == _lib.ERR_DTYPE
    out = _view([5], DType.float32)
    assert L.nca_reduce(ctypes.byref(src), 0, 1, ctypes.byref(out), None) == _lib.ERR_SHAPE


def test_fast_division_magic():
    """The invariant-divisor division used by the ND kernel (q = (umulhi(x, m) + x) >> s)
    is exact for divisors and dividends below 2^31."""
    rng = np.random.default_rng(1)
    divisors = [1, 2, 3, 5, 7, 8, 64, 255, 256, 1000, 65535, 123457, 2**20 + 1, 2**30, 2**31 - 1]
    xs = np.concatenate([rng.integers(0, 2**31, 20000, dtype=np.uint64),
                         np.array([0, 1, 2**31 - 1, 2**31 - 2], dtype=np.uint64)])
    for d in divisors:
        s = 0
        while (1 << s) < d:
            s += 1
        m = ((1 << 32) * ((1 << s) - d)) // d + 1
        m &= 0xFFFFFFFF
        hi = (xs * np.uint64(m)) >> np.uint64(32)
        q = (hi + xs) >> np.uint64(s)
        assert np.array_equal(q, xs // np.uint64(d)), d
