"""nca_scatter_add on the GPU against the reference's own scatter-add
(golden vectors from host::scatter_add_recursive) and against the oracle
restatement on larger seeded inputs.

Integer destinations must match bit for bit. Float destinations add in the
order the atomics land, so each entry is checked against the float64 sum of
its contributions: |got - exact| <= (k + 1) * eps * sum |contributions| with k
the entry's contribution count and eps = 2^-24 (float32) or 2^-53 (float64)."""
import json
from pathlib import Path

import numpy as np
import pytest

import ncarray_gb300 as nca
from ncarray_gb300.dtype import DType
from tests.helpers import SEED

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden" / "ref_golden.npz"
NP = {4: np.uint32, 5: np.uint64, 8: np.int32, 9: np.int64, 10: np.float32, 11: np.float64}


def _check(got, dest0, dest_dt, idx, src, orc, src_dt):
    """Compares a GPU result with the oracle (integer: exact; float: bound)."""
    want = dest0.copy()
    orc.scatter_add(want, dest_dt, idx, int(DType.int64) if idx.dtype == np.int64 else _dt(idx), src, src_dt)
    if dest_dt not in (10, 11):
        assert got.tobytes() == want.tobytes()
        return
    exact = dest0.astype(np.float64)
    orc.scatter_add(exact, 11, idx, _dt(idx), src, src_dt)
    mag = np.abs(dest0.astype(np.float64))
    cnt = np.zeros(dest0.size, np.float64)
    flat_i = idx.reshape(-1).astype(np.int64) if idx.dtype != np.uint64 else idx.reshape(-1).view(np.int64)
    flat_s = src.reshape(-1).astype(np.float64)
    ok = (flat_i >= 0) & (flat_i < dest0.size)
    np.add.at(mag, flat_i[ok], np.abs(flat_s[ok]))
    np.add.at(cnt, flat_i[ok], 1.0)
    eps = 2.0**-24 if dest_dt == 10 else 2.0**-53
    err = np.abs(got.astype(np.float64) - exact)
    assert np.all(err <= (cnt + 1) * eps * mag + 1e-300), float((err - (cnt + 1) * eps * mag).max())


def _dt(a):
    return {np.dtype(np.int32): 8, np.dtype(np.uint32): 4, np.dtype(np.int64): 9, np.dtype(np.uint64): 5,
            np.dtype(np.float32): 10, np.dtype(np.float64): 11}[a.dtype]


def _run(dest0, dest_dt, idx, src):
    d = nca.NCDevArray.from_host(dest0, DType(dest_dt))
    d.scatter_add(nca.NCDevArray.from_host(idx), nca.NCDevArray.from_host(src))
    return d.to_host()


def test_scatter_add_reference_golden(cuda, orc):
    """The reference's own results (dest x index x source dtypes, 2-D views,
    out-of-range indices): integer dests bit-exact, float dests within bound."""
    z = np.load(GOLDEN)
    meta = json.loads(bytes(z["meta"]).decode())
    n = 0
    for i, m in enumerate(meta):
        if m["kind"] != "scatter":
            continue
        idx, src, want = z[f"x{i}_idx"], z[f"x{i}_src"], z[f"x{i}_dest"]
        got = _run(np.zeros_like(want), m["dest"], idx, src)
        if m["dest"] in (10, 11):
            _check(got, np.zeros_like(want), m["dest"], idx, src, orc, m["src"])
        else:
            assert got.tobytes() == want.tobytes(), m
        n += 1
    assert n == 6


@pytest.mark.parametrize("dest_dt,n_dest,n", [
    (9, 1000, 1 << 20),        # int64, shared-memory copy of the destination
    (10, 3000, 1 << 20),       # float32, shared-memory copy
    (5, 1 << 20, 1 << 22),     # uint64 counts on a 1 Mi grid (global atomics)
    (10, 1 << 20, 1 << 22),    # float32 weights on a 1 Mi grid
    (11, 50_000, 777_777),     # float64, odd sizes
    (8, 17, 100_003),          # int32, tiny destination, heavy collisions
])
def test_scatter_add_skewed_indices(cuda, orc, dest_dt, n_dest, n):
    """Indices from a mixture of narrow Gaussians (a few hot entries take
    most elements), some out of range on both sides."""
    rng = np.random.default_rng(SEED + 300 + dest_dt)
    centres = rng.uniform(0, n_dest, 6)
    sig = rng.uniform(0.5, max(1.0, n_dest / 200), 6)
    comp = rng.choice(6, size=n, p=rng.dirichlet(np.full(6, 0.5)))
    idx = np.floor(centres[comp] + rng.normal(size=n) * sig[comp]).astype(np.int64)
    idx[rng.random(n) < 0.01] = -3
    idx[rng.random(n) < 0.01] = n_dest + 5
    if dest_dt in (10, 11):
        src = rng.lognormal(0, 1, n).astype(np.float32 if dest_dt == 10 else np.float64)
    else:
        src = rng.integers(-1000, 1000, n).astype(np.int32)
    dest0 = np.zeros(n_dest, NP[dest_dt])
    if dest_dt in (9, 8):
        dest0 += rng.integers(-50, 50, n_dest).astype(NP[dest_dt])
    got = _run(dest0, dest_dt, idx, src)
    _check(got, dest0, dest_dt, idx, src, orc, _dt(src))


def test_scatter_add_strided_views_and_index_dtypes(cuda, orc):
    """Transposed index/source views (non-mergeable dims), uint32 / uint64 /
    int32 indices (uint64 values above 2^63 are out of range), and a
    destination with a byte stride of two elements."""
    rng = np.random.default_rng(SEED + 310)
    n_dest = 513
    base_i = rng.integers(-10, n_dest + 10, (64, 48, 5))
    base_s = rng.integers(-100, 100, (64, 48, 5)).astype(np.int64)
    for idt in (np.int32, np.uint32, np.int64, np.uint64):
        idx = base_i.astype(idt)
        if idt == np.uint64:
            idx[0, 0, :] = np.uint64(1 << 63) + np.uint64(3)
        idx_t = np.ascontiguousarray(idx.transpose(2, 0, 1))
        src_t = np.ascontiguousarray(base_s.transpose(2, 0, 1))
        di = nca.NCDevArray.from_host(idx_t).transpose(1, 2, 0)       # (64, 48, 5), strided
        ds = nca.NCDevArray.from_host(src_t).transpose(1, 2, 0)
        big = nca.NCDevArray.from_host(np.zeros(2 * n_dest, np.int64))
        dest = big[::2]
        dest.scatter_add(di, ds)
        got = big.to_host()[::2].copy()
        want = np.zeros(n_dest, np.int64)
        orc.scatter_add(want, 9, idx, _dt(idx), base_s, 9)
        assert np.array_equal(got, want), idt
        assert not big.to_host()[1::2].any()


def test_scatter_add_casts_and_empty(cuda, orc):
    """bool, bfloat16 and float64 sources cast into float32 / int64
    destinations; empty inputs and empty destinations are no-ops."""
    rng = np.random.default_rng(SEED + 311)
    n, n_dest = 100_000, 257
    idx = rng.integers(0, n_dest, n).astype(np.int64)
    b = rng.integers(0, 2, n).astype(np.bool_)
    got = _run(np.zeros(n_dest, np.int64), 9, idx, b)
    want = np.zeros(n_dest, np.int64)
    orc.scatter_add(want, 9, idx, 9, b, 0)
    assert np.array_equal(got, want)
    f = rng.normal(size=n).astype(np.float32)
    bf = (f.view(np.uint32) >> 16).astype(np.uint16)
    d = nca.NCDevArray.from_host(np.zeros(n_dest, np.float32))
    d.scatter_add(nca.NCDevArray.from_host(idx), nca.NCDevArray.from_host(bf, DType.bfloat16))
    widened = (bf.astype(np.uint32) << 16).view(np.float32)
    _check(d.to_host(), np.zeros(n_dest, np.float32), 10, idx, widened, orc, 10)
    e = nca.NCDevArray.from_host(np.zeros(4, np.float32))
    e.scatter_add(nca.NCDevArray.from_host(np.zeros(0, np.int64)), nca.NCDevArray.from_host(np.zeros(0, np.float32)))
    assert not e.to_host().any()
