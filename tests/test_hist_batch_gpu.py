"""2-D histogram and batched uneven reductions on the GPU vs the oracle.

Histogram counts (uint64) must be bit-exact; per-bin weight sums are float64
accumulations rounded to float32, so they match the float64 oracle to one
float32 rounding (|got - ref| <= 2^-24 |ref|, plus one ulp of slack).
Batched results are float64: |err| <= 1e-6 |ref| for the mean and both sums
(and <= 1e-9 sum|x| in absolute terms); max is exact."""
import numpy as np
import pytest

import ncarray_gb300 as nca
from ncarray_gb300.batch import Batch
from ncarray_gb300.dtype import DType
from ncarray_gb300.hist import hist2d
from tests.helpers import SEED

pytestmark = pytest.mark.gpu


def mixture_points(rng, n):
    centres = rng.uniform(0, 1, (8, 2))
    sigma = rng.uniform(0.01, 0.1, 8)
    weights = rng.dirichlet(np.full(8, 0.5))
    comp = rng.choice(8, size=n, p=weights)
    pts = centres[comp] + rng.normal(size=(n, 2)) * sigma[comp, None]
    return pts[:, 0].astype(np.float32), pts[:, 1].astype(np.float32)


@pytest.mark.parametrize("n,nb", [(1 << 20, (1024, 1024)), (100003, (37, 61)), (5, (4, 4))])
def test_hist2d_matches_oracle(cuda, orc, n, nb):
    rng = np.random.default_rng(SEED + 5)
    x, y = mixture_points(rng, n)
    x[: min(n, 3)] = [np.nan, -0.5, 1.0][: min(n, 3)]
    w = rng.lognormal(0, 1, n).astype(np.float32)
    nbx, nby = nb
    counts, wsum = hist2d(nca.NCDevArray.from_host(x), nca.NCDevArray.from_host(y), nbx, nby,
                          w=nca.NCDevArray.from_host(w))
    rc, rw = orc.hist2d(x, y, w, nbx, nby, 0.0, 1.0, 0.0, 1.0)
    assert np.array_equal(counts.to_host().reshape(-1), rc)
    got = wsum.to_host().reshape(-1).astype(np.float64)
    ref32 = rw.astype(np.float32).astype(np.float64)
    assert np.all(np.abs(got - ref32) <= 2.0**-23 * np.abs(rw) + 1e-30)
    # counts only (no weights)
    c2, _ = hist2d(nca.NCDevArray.from_host(x), nca.NCDevArray.from_host(y), nbx, nby)
    assert np.array_equal(c2.to_host().reshape(-1), rc)


def _check_hist(x, y, w, nbx, nby, orc, xr=(0.0, 1.0), yr=(0.0, 1.0)):
    counts, wsum = hist2d(nca.NCDevArray.from_host(x), nca.NCDevArray.from_host(y), nbx, nby, xr, yr,
                          w=nca.NCDevArray.from_host(w))
    rc, rw = orc.hist2d(x, y, w, nbx, nby, xr[0], xr[1], yr[0], yr[1])
    assert np.array_equal(counts.to_host().reshape(-1), rc)
    got = wsum.to_host().reshape(-1).astype(np.float64)
    ref32 = rw.astype(np.float32).astype(np.float64)
    assert np.all(np.abs(got - ref32) <= 2.0**-23 * np.abs(rw) + 1e-30)
    return rc, rw


def test_hist2d_bucket_overflow(cuda, orc):
    """The sampled blocks (every 32nd block of 1024 points) spread over the
    grid while all other points crowd into one tile: that tile's bucket
    overflows and its excess goes through the direct atomics."""
    rng = np.random.default_rng(SEED + 6)
    n = (1 << 21) + 777
    x = rng.uniform(0.40, 0.41, n).astype(np.float32)
    y = rng.uniform(0.50, 0.505, n).astype(np.float32)
    idx = np.arange(n)
    sampled = (idx // 1024) % 32 == 0
    x[sampled] = rng.uniform(0, 1, sampled.sum()).astype(np.float32)
    y[sampled] = rng.uniform(0, 1, sampled.sum()).astype(np.float32)
    w = rng.lognormal(0, 1, n).astype(np.float32)
    _check_hist(x, y, w, 1024, 1024, orc)


def test_hist2d_partial_tile_and_ranges(cuda, orc):
    """A grid that is not a whole number of 16384-bin tiles, a range other
    than [0,1)^2, and points outside it."""
    rng = np.random.default_rng(SEED + 7)
    n = (1 << 20) + 12345
    x = rng.normal(0.0, 2.0, n).astype(np.float32)
    y = rng.normal(1.0, 3.0, n).astype(np.float32)
    w = rng.lognormal(0, 1, n).astype(np.float32)
    _check_hist(x, y, w, 1000, 1100, orc, xr=(-4.0, 4.0), yr=(-5.0, 7.0))


def test_hist2d_single_bin(cuda, orc):
    """Every point in one bin (maximal collisions)."""
    n = 1 << 21
    rng = np.random.default_rng(SEED + 8)
    x = np.full(n, 0.5, np.float32)
    y = np.full(n, 0.25, np.float32)
    w = rng.lognormal(0, 1, n).astype(np.float32)
    _check_hist(x, y, w, 512, 512, orc)


def test_hist2d_accumulates_and_empty(cuda, orc):
    from ncarray_gb300.hist import hist2d_into
    rng = np.random.default_rng(SEED + 9)
    x, y = mixture_points(rng, 1 << 20)
    w = rng.lognormal(0, 1, x.size).astype(np.float32)
    dx, dy, dw = (nca.NCDevArray.from_host(a) for a in (x, y, w))
    counts = nca.NCDevArray((256, 256), nca.DType.uint64).fill(0)
    wsum = nca.NCDevArray((256, 256), nca.DType.float32).fill(0.0)
    hist2d_into(dx, dy, counts, (0.0, 1.0), (0.0, 1.0), dw, wsum)
    hist2d_into(dx, dy, counts, (0.0, 1.0), (0.0, 1.0), dw, wsum)
    rc, rw = orc.hist2d(x, y, w, 256, 256, 0.0, 1.0, 0.0, 1.0)
    assert np.array_equal(counts.to_host().reshape(-1), 2 * rc)
    got = wsum.to_host().reshape(-1).astype(np.float64)
    assert np.all(np.abs(got - 2 * rw) <= 2.0**-22 * np.abs(rw) + 1e-30)
    # no points: outputs unchanged
    e = nca.NCDevArray((0,), nca.DType.float32)
    hist2d_into(e, e, counts, (0.0, 1.0), (0.0, 1.0))
    assert np.array_equal(counts.to_host().reshape(-1), 2 * rc)


def make_batch(rng, n, lo=64, hi=1 << 16):
    lens = np.round(np.exp(rng.uniform(np.log(lo), np.log(hi), n))).astype(np.int64)
    lens[:3] = [1, 64, 257][: min(n, 3)]
    arrays, host, dts = [], [], []
    for i, L in enumerate(lens):
        x = (np.exp(rng.normal(0, 2, L)) * rng.choice([-1.0, 1.0], L)).astype(np.float32)
        if i % 2 == 0:
            arrays.append(nca.NCDevArray.from_host(x))
            host.append(x)
            dts.append(10)
        else:
            b = (x.view(np.uint32) >> 16).astype(np.uint16)
            arrays.append(nca.NCDevArray.from_host(b, nca.DType.bfloat16))
            host.append(b)
            dts.append(22)
    return arrays, host, dts


def check_batch(got, ref, host, dts):
    for i in range(len(host)):
        x = host[i]
        xf = (x.astype(np.uint32) << 16).view(np.float32) if dts[i] == 22 else x
        scale = float(np.abs(xf.astype(np.float64)).sum())
        for k in (0, 1, 3):
            assert abs(got[i, k] - ref[i, k]) <= 1e-6 * abs(ref[i, k]) + 1e-9 * scale, (i, k, got[i], ref[i])
        assert got[i, 2] == ref[i, 2]


def test_batch_persistent_graph_plain(cuda, orc):
    rng = np.random.default_rng(SEED + 6)
    arrays, host, dts = make_batch(rng, 300)
    ref = orc.batch_reduce(host, dts, nthreads=4)
    b = Batch(arrays)
    check_batch(b.run().to_host(), ref, host, dts)
    check_batch(b.run().to_host(), ref, host, dts)              # counters reset between launches
    check_batch(b.run(graph=True).to_host(), ref, host, dts)
    check_batch(b.run(graph=True).to_host(), ref, host, dts)
    check_batch(b.run_plain().to_host(), ref, host, dts)
    sched = b.autotune()
    assert sched["chunk_bytes"] > 0 and sched["threads"] in (256, 512)
    check_batch(b.run().to_host(), ref, host, dts)


def test_batch_relative_error_with_cancellation(cuda, orc):
    """Random-sign lognormal(0, 2) sums: the float-float path stays within 1e-6
    of float64 relative to |sum| on every array of the batch."""
    rng = np.random.default_rng(SEED + 7)
    arrays, host, dts = make_batch(rng, 64, lo=1 << 12, hi=1 << 20)
    ref = orc.batch_reduce(host, dts, nthreads=4)
    got = Batch(arrays).run().to_host()
    rel = np.abs(got[:, 0] - ref[:, 0]) / np.abs(ref[:, 0])
    assert rel.max() <= 1e-6, rel.max()


def _edge_case_batch(rng, lens, dts, offset_of):
    """Arrays of the given lengths and dtypes, each a view of a larger device
    buffer starting offset_of(i) elements in (misaligned bodies, head and tail
    elements outside the 16-byte aligned part)."""
    arrays, host, codes = [], [], []
    for i, (L, dt) in enumerate(zip(lens, dts)):
        off = offset_of(i)
        x = (np.exp(rng.normal(0, 2, L + off + 3)) * rng.choice([-1.0, 1.0], L + off + 3)).astype(np.float32)
        if dt == DType.float32:
            h = x
        elif dt == DType.bfloat16:
            h = (x.view(np.uint32) >> 16).astype(np.uint16)
        else:
            h = x.astype(np.float16)
        big = nca.NCDevArray.from_host(h, dt)
        arrays.append(big[off:off + L])
        host.append(np.ascontiguousarray(h[off:off + L]))
        codes.append(int(dt))
    return arrays, host, codes


def _check_edges(got, ref, host, codes):
    lowest = float(np.finfo(np.float32).min)
    for i, x in enumerate(host):
        if x.size == 0:
            assert got[i, 0] == 0.0 and np.isnan(got[i, 1]) and got[i, 2] == lowest and got[i, 3] == 0.0, got[i]
            continue
        if codes[i] == int(DType.bfloat16):
            xf = (x.astype(np.uint32) << 16).view(np.float32)
        else:
            xf = x.astype(np.float32)
        scale = float(np.abs(xf.astype(np.float64)).sum())
        for k in (0, 1, 3):
            assert abs(got[i, k] - ref[i, k]) <= 1e-6 * abs(ref[i, k]) + 1e-9 * scale, (i, x.size, k, got[i], ref[i])
        assert got[i, 2] == ref[i, 2], (i, x.size, got[i, 2], ref[i, 2])


def test_batch_edges(cuda, orc):
    """Lengths around every boundary of the pipeline (16-byte vectors, slabs,
    chunks), empty arrays, all three dtypes, bodies starting 0..7 elements
    past an aligned address, a batch of arrays shorter than 16 bytes, and a
    batch of one array."""
    rng = np.random.default_rng(SEED + 8)
    base = [0, 1, 2, 3, 4, 5, 7, 8, 9, 15, 16, 17, 31, 33, 63, 65, 127, 129, 4095, 4096, 4097,
            65535, 65536, 65537, 131071, 131073, 262143, 262145]
    lens, dts = [], []
    for dt in (DType.float32, DType.bfloat16, DType.float16):
        lens += base
        dts += [dt] * len(base)
    arrays, host, codes = _edge_case_batch(rng, lens, dts, lambda i: i % 8)
    ref = orc.batch_reduce(host, codes, nthreads=4)
    b = Batch(arrays)
    _check_edges(b.run().to_host(), ref, host, codes)
    _check_edges(b.run(graph=True).to_host(), ref, host, codes)
    # only head/tail elements (no 16-byte aligned body)
    lens = [1, 2, 3, 5, 7] * 6
    dts = [DType.float32, DType.bfloat16, DType.float16] * 10
    arrays, host, codes = _edge_case_batch(rng, lens, dts, lambda i: (3 * i) % 8)
    ref = orc.batch_reduce(host, codes, nthreads=4)
    _check_edges(Batch(arrays).run().to_host(), ref, host, codes)
    # one array
    arrays, host, codes = _edge_case_batch(rng, [1 << 20], [DType.float32], lambda i: 5)
    ref = orc.batch_reduce(host, codes, nthreads=4)
    _check_edges(Batch(arrays).run().to_host(), ref, host, codes)
