"""Fused elementwise expressions on the GPU vs the oracle: bit-exact for every
dtype (float arithmetic rounds after each operation on both sides).

Mirrors the reference's test_gpu_binary_operations.cu / test_gpu_operations.py
cases and adds the strided, permuted and broadcast views of the C2 workload."""
import numpy as np
import pytest

import ncarray_gb300 as nca
from ncarray_gb300.dtype import DType
from tests.helpers import SEED, assert_bits_equal, oracle_eval, rand

pytestmark = pytest.mark.gpu

ALL = [DType.bool, DType.int8, DType.uint8, DType.int16, DType.uint16, DType.int32, DType.uint32,
       DType.int64, DType.uint64, DType.float32, DType.float64, DType.bfloat16, DType.float16]


def dev(h, dt=None):
    return nca.NCDevArray.from_host(h, dt)


def check(orc, expr, host_ops, what=""):
    got = expr.materialize().to_host()
    want = oracle_eval(orc, expr, host_ops)
    assert got.dtype.itemsize == want.dtype.itemsize
    assert_bits_equal(got, want, what)
    return got


def test_c1_expression_f64(cuda, orc):
    """out = a*b + sqrt(abs(c)) - 0.5*a on float64 (128,128,128)."""
    rng = np.random.default_rng(SEED + 0)
    a, b, c = (rng.uniform(-1, 1, (128, 128, 128)) for _ in range(3))
    da, db, dc = dev(a), dev(b), dev(c)
    with nca.lazy_mode():
        e = da * db + nca.sqrt(abs(dc)) - 0.5 * da
    got = check(orc, e, [a, b, c], "C1")
    np.testing.assert_array_equal(got, a * b + np.sqrt(np.abs(c)) - np.float32(0.5) * a)


@pytest.mark.parametrize("shape", [(4, 16, 8, 8), (2, 32, 16, 4), (3, 5, 7, 2)])
def test_c2_strided_broadcast(cuda, orc, shape):
    """y = x.permute(3,1,2,0) * v[None,:,None,None] + k with mixed f32/i32."""
    rng = np.random.default_rng(SEED + 1)
    x = rng.normal(size=shape).astype(np.float32)
    xp = x.transpose(3, 1, 2, 0)
    v = rng.normal(size=(shape[1],)).astype(np.float32)
    k = rng.integers(-1000, 1001, xp.shape).astype(np.int32)
    dx, dv, dk = dev(x).permute(3, 1, 2, 0), dev(v), dev(k)
    vb = dv.reshape(1, shape[1], 1, 1)
    with nca.lazy_mode():
        y = dx * vb + dk
        z = (dk * 3 + 7) % 11
    assert y.dtype == DType.float32 and z.dtype == DType.int32
    got = check(orc, y, [xp, v.reshape(1, -1, 1, 1), k], "C2 y")
    np.testing.assert_array_equal(got, xp * v.reshape(1, -1, 1, 1) + k.astype(np.float32))
    gz = check(orc, z, [k], "C2 int")
    np.testing.assert_array_equal(gz, np.fmod(k * 3 + 7, 11))


@pytest.mark.parametrize("dt", ALL)
def test_dtype_matrix(cuda, orc, dt):
    rng = np.random.default_rng(SEED + 10 + int(dt))
    shape = (7, 33, 5)
    a, b = rand(rng, shape, dt), rand(rng, shape, dt)
    da, db = dev(a, dt), dev(b, dt)
    with nca.lazy_mode():
        exprs = {
            "add": da + db, "sub": da - db, "mul": da * db, "div": da / db, "mod": da % db,
            "gt": da > db, "eq": da == db, "neg": -da, "abs": abs(da),
            "chain": (da + db) * 3 - da, "land": nca.logical_and(da, db),
        }
    for name, e in exprs.items():
        check(orc, e, [a, b][: len(e.arrays)] if len(e.arrays) <= 2 else [a, b, a], f"{dt.name} {name}")


@pytest.mark.parametrize("dt", [DType.float32, DType.float64, DType.int32, DType.uint8])
def test_views(cuda, orc, dt):
    """Negative strides, stepped slices, misaligned starts, broadcasts, 1-element."""
    rng = np.random.default_rng(SEED + 40 + int(dt))
    h = rand(rng, (9, 17, 12), dt)
    d = dev(h, dt)
    cases = [
        (d[::-1, :, ::2], h[::-1, :, ::2]),
        (d[1:, 3:, 1:], h[1:, 3:, 1:]),
        (d.transpose(2, 0, 1), h.transpose(2, 0, 1)),
        (d[:, 5:6, :], h[:, 5:6, :]),
        (d[4:5, 2:3, 7:8], h[4:5, 2:3, 7:8]),
    ]
    for dv, hv in cases:
        with nca.lazy_mode():
            e = dv * 2 + dv
        check(orc, e, [hv], f"view {hv.strides}")
    # broadcast of a row and a column
    r, c = rand(rng, (1, 17, 1), dt), rand(rng, (9, 1, 12), dt)
    with nca.lazy_mode():
        e = dev(r, dt) + dev(c, dt)
    check(orc, e, [r, c], "broadcast")


def test_assign_into_strided_view(cuda, orc):
    rng = np.random.default_rng(SEED + 50)
    base = np.zeros((10, 10), dtype=np.float32)
    d = dev(base)
    d.fill(0.0)
    d[1:3, 1:3] = 5.0
    src = rng.normal(size=(2, 2)).astype(np.float32)
    d[7:9, 7:9] = src
    h = d.to_host()
    assert h[0, 0] == 0.0
    assert np.all(h[1:3, 1:3] == 5.0)
    assert np.array_equal(h[7:9, 7:9], src)
    # expression into a transposed view
    a = rng.normal(size=(6, 8)).astype(np.float32)
    out = nca.NCDevArray((8, 6), DType.float32)
    with nca.lazy_mode():
        e = dev(a) * 2.0
    e.evaluate(out=out.transpose(1, 0))
    np.testing.assert_array_equal(out.to_host(), (a * np.float32(2.0)).T)


def test_iota_and_scalars(cuda, orc):
    with nca.lazy_mode():
        e = nca.iota((3, 4, 5), DType.int64) * 2 + 1
    got = e.materialize().to_host()
    np.testing.assert_array_equal(got, np.arange(60).reshape(3, 4, 5) * 2 + 1)
    rng = np.random.default_rng(SEED + 60)
    a = rand(rng, (5, 6), DType.int16)
    with nca.lazy_mode():
        e = dev(a) * 300 - 70000 + np.int8(-3)
    check(orc, e, [a], "mixed scalars")


def test_reference_semantics(cuda):
    """Known answers of the reference tests (tests/cxx/test_binary_operations.cc,
    test_gpu_binary_operations.cu, tests/python/test_gpu_operations.py)."""
    a = nca.NCDevArray([4, 4, 4], DType.float32).fill(2.0)
    b = nca.NCDevArray([4, 4, 4], DType.float32).fill(4.0)
    assert np.all((a + b).to_host() == 6.0) and np.all((a * b).to_host() == 8.0)
    q = a / b
    assert q.dtype == DType.float64 and np.all(q.to_host() == 0.5)
    m = a > 1.0
    assert m.dtype == DType.bool and np.all(m.to_host())
    x = nca.NCDevArray([100]).fill(10.0)
    x += 5.0
    x *= 2.0
    assert np.all(x.to_host() == 30.0)
    u = nca.NCDevArray.from_host(np.array([7, 8, 9], dtype=np.uint32))
    assert np.array_equal((u % 4).to_host(), np.array([3, 0, 1], dtype=np.uint32))
    z = nca.NCDevArray([10], DType.float32).fill(10.0)
    z[0:5].fill(0.0)
    g = (z > 5.0).to_host()
    assert not g[0] and g[9]


def test_empty_and_zero_division(cuda, orc):
    e0 = nca.NCDevArray([0, 5], DType.float32)
    assert (e0 * 2).to_host().shape == (0, 5)
    a = np.array([1.0, -2.0, 0.0, np.inf, np.nan], dtype=np.float64)
    z = np.zeros(5)
    with nca.lazy_mode():
        e = dev(a) / dev(z)
    got = check(orc, e, [a, z], "x/0")
    assert np.isnan(got[0]) and np.isnan(got[2]) and got[3] == np.inf
    i = np.array([5, -7, 0, 3], dtype=np.int32)
    with nca.lazy_mode():
        e = dev(i) % dev(np.array([0, -1, 3, 2], dtype=np.int32))
    check(orc, e, [i, np.array([0, -1, 3, 2], dtype=np.int32)], "int mod edge")


@pytest.mark.parametrize("dt", [DType.int32, DType.uint8, DType.int64, DType.float32])
def test_opcode_matrix(cuda, orc, dt):
    """Every opcode the device evaluates, alone and mixed with IDX, vs the oracle
    (bit-exact): comparisons, logical and bitwise ops, INC/DEC/NEG, BNOT."""
    rng = np.random.default_rng(SEED + 40 + int(dt))
    shape = (5, 17, 9)
    a, b = rand(rng, shape, dt), rand(rng, shape, dt)
    da, db = dev(a, dt), dev(b, dt)
    with nca.lazy_mode():
        exprs = {
            "ne": da != db, "lt": da < db, "le": da <= db, "ge": da >= db,
            "lor": nca.logical_or(da, db), "lnot": nca.logical_not(da),
            "inc": nca.inc(da), "dec": nca.dec(da), "neg_inc": -nca.inc(db),
            "cmp_chain": nca.logical_and(da < db, db != 0),
            "idx_mix": da + nca.iota(shape, dt),
        }
        if dt != DType.float32:
            exprs.update({"band": da & db, "bor": da | db, "xor": da ^ db, "bnot": ~da,
                          "bit_chain": (da & 7) | (db ^ 3)})
    host = {id(da): a, id(db): b}
    for name, e in exprs.items():
        check(orc, e, [host[id(x)] for x in e.arrays], f"{dt.name} {name}")
