"""nca_reduce_noalloc: the full reduction for callers that cannot allocate
device memory (stream capture without memory nodes, pre-planned real-time
loops, hosts without an allocator for the library).

Runs through the C ABI and compares every op against nca_reduce, the
allocating entry point, on two calls in a row: the second input is smaller
but still spans about 70 CTAs, so a stale partial of the first call would show.
Integer sums, max/min and arg-reductions must match exactly; float sums and
means within |a - b| <= 2^-23 |b| + 1e-12 sum|x|, and against the float64
oracle within the same bound. Float inputs holding +inf, -inf and NaN, and
inputs made only of -inf, only of +inf or of repeated extreme values, must
give what nca_reduce gives (NaN where it gives NaN).
This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes on its own in a fresh process."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OPS = {"sum": 0, "mean": 1, "max": 2, "min": 3, "argmax": 4, "argmin": 5}


def _view(lib_mod, ptr, dt, shape, isz):
    st, acc = [], isz
    for n in reversed(shape):
        st.append(acc)
        acc *= n
    return lib_mod.make_view(ptr, dt, shape, list(reversed(st)))


def _out_dtype(op, dt):
    return {0: dt, 1: 11, 2: dt, 3: dt, 4: 9, 5: 9}[op]


def _run(torch, lib_mod, name, x_dev, dt, isz, shape, op):
    odt = _out_dtype(op, dt)
    tdt = {10: torch.float32, 11: torch.float64, 8: torch.int32, 9: torch.int64}[odt]
    a = torch.zeros(1, dtype=tdt, device="cuda")
    src = _view(lib_mod, x_dev.data_ptr(), dt, shape, isz)
    out = lib_mod.make_view(a.data_ptr(), odt, (), ())
    stream = torch.cuda.current_stream().cuda_stream
    if name == "noalloc":
        lib_mod.call("nca_reduce_noalloc", ctypes.byref(src), op, ctypes.byref(out), stream)
    else:
        mask = (1 << len(shape)) - 1
        lib_mod.call("nca_reduce", ctypes.byref(src), op, mask, ctypes.byref(out), stream)
    torch.cuda.synchronize()
    return a.cpu().item()


@pytest.mark.parametrize("dt", [10, 11, 8, 9])
def test_noalloc_matches_reduce(cuda, dt):
    torch = cuda
    import oracle
    from ncarray_gb300 import _lib
    rng = np.random.default_rng(20261203 + dt)
    npdt = {10: np.float32, 11: np.float64, 8: np.int32, 9: np.int64}[dt]
    isz = np.dtype(npdt).itemsize
    inputs = []
    for shape in [(3, 1000, 337), (7, 40000)]:   # two calls in a row, both multi-CTA
        if dt in (10, 11):
            h = (rng.lognormal(0, 2, shape) * rng.choice([-1, 1], shape)).astype(npdt)
        else:
            h = rng.integers(-10**6, 10**6, shape).astype(npdt)
        inputs.append((shape, h, torch.from_numpy(h.reshape(-1)).cuda()))
    for op_name, op in OPS.items():
        for shape, h, d in inputs:
            got = _run(torch, _lib, "noalloc", d, dt, isz, shape, op)
            want = _run(torch, _lib, "reduce", d, dt, isz, shape, op)
            if dt in (10, 11) and op in (0, 1):
                scale = float(np.abs(h.astype(np.float64)).sum()) / (h.size if op == 1 else 1)
                assert abs(got - want) <= 2.0**-23 * abs(want) + 1e-12 * scale, (op_name, shape, got, want)
                exact = float(oracle.reduce(h, dt, op))
                assert abs(got - exact) <= 2.0**-23 * abs(exact) + 1e-12 * scale, (op_name, shape, got, exact)
            else:
                assert got == want, (op_name, shape, got, want)
            if op == 4:
                assert got == int(np.argmax(h.reshape(-1)))


def test_noalloc_rejects_oversized_and_strided(cuda):
    torch = cuda
    from ncarray_gb300 import _lib
    L = _lib.lib()
    a = torch.zeros(1, dtype=torch.float32, device="cuda")
    out = _lib.make_view(a.data_ptr(), 10, (), ())
    big = _view(_lib, a.data_ptr(), 10, (1 << 16, 1 << 16), 4)   # 2^32 elements: never touched
    assert L.nca_reduce_noalloc(ctypes.byref(big), 0, ctypes.byref(out), None) == _lib.ERR_LIMIT
    assert b"at most" in L.nca_last_error()
    x = torch.zeros(16, dtype=torch.float32, device="cuda")
    strided = _lib.make_view(x.data_ptr(), 10, (8,), (8,))
    assert L.nca_reduce_noalloc(ctypes.byref(strided), 0, ctypes.byref(out), None) == _lib.ERR_UNSUPPORTED


def _same(got, want):
    return (np.isnan(got) and np.isnan(want)) or got == want


@pytest.mark.parametrize("dt", [10, 11])
def test_noalloc_special_values(cuda, dt):
    """Non-finite and all-extreme float inputs, each on a multi-CTA input."""
    torch = cuda
    from ncarray_gb300 import _lib
    npdt = {10: np.float32, 11: np.float64}[dt]
    isz = np.dtype(npdt).itemsize
    rng = np.random.default_rng(77 + dt)
    n = 50_000
    base = rng.normal(size=n).astype(npdt)
    big = np.finfo(npdt).max
    cases = {}
    x = base.copy(); x[12_345] = np.inf; cases["one_pos_inf"] = x
    x = base.copy(); x[40_001] = -np.inf; cases["one_neg_inf"] = x
    x = base.copy(); x[7] = np.inf; x[49_000] = -np.inf; cases["both_inf"] = x
    x = base.copy(); x[30_000] = np.nan; cases["nan"] = x
    cases["all_neg_inf"] = np.full(n, -np.inf, dtype=npdt)
    cases["all_pos_inf"] = np.full(n, np.inf, dtype=npdt)
    x = base.copy(); x[[5, 20_000, 45_000]] = big; x[[6, 20_001, 45_001]] = -big; cases["tied_extremes"] = x
    cases["all_equal"] = np.full(n, 1.5, dtype=npdt)
    # float32 partial sums that overflow to inf while every element is finite
    cases["overflowing_sum"] = np.full(n, big / 4, dtype=npdt)
    for name, h in cases.items():
        d = torch.from_numpy(h).cuda()
        for op_name, op in OPS.items():
            for _ in range(2):   # two calls in a row
                got = _run(torch, _lib, "noalloc", d, dt, isz, (n,), op)
                want = _run(torch, _lib, "reduce", d, dt, isz, (n,), op)
                if name == "overflowing_sum" and op == 1 and dt == 10:
                    # float64 mean of float32 values: whether a float32 partial
                    # overflows first depends on how many elements a thread
                    # adds, which differs between the two entry points; it
                    # must be a positive number or +inf, never NaN
                    assert got > 0 and not np.isnan(got), (name, op_name, got)
                elif op in (0, 1) and np.isfinite(want) and np.isfinite(got):
                    # tied_extremes cancels +-max: only the sum|x|-scaled bound holds
                    scale = float(np.abs(h.astype(np.float64)).sum()) / (n if op == 1 else 1)
                    assert abs(got - want) <= 2.0**-23 * abs(want) + 1e-12 * scale, (name, op_name, got, want)
                else:
                    assert _same(got, want), (name, op_name, got, want)
