"""Histogram counts on the partitioned (tile) path and the direct-atomics
path against the oracle, bit-exact:

* grids from 1x1 to 1024x1024 (odd sizes), point counts that are not
  multiples of four;
* hot bins that take a large share of the points (a single-bin grid takes
  all of them), within one call and across calls that add to one output;
* both paths give the same counts for the same points."""
import os

import numpy as np
import pytest

import ncarray_gb300 as nca
from ncarray_gb300.dtype import DType
from ncarray_gb300.hist import hist2d_into
from tests.helpers import SEED

pytestmark = pytest.mark.gpu


def _counts(path, x, y, nbx, nby, out=None):
    old = os.environ.get("NCA_HIST_PATH")
    os.environ["NCA_HIST_PATH"] = path
    try:
        c = out if out is not None else nca.NCDevArray((nby, nbx), DType.uint64).fill(0)
        hist2d_into(nca.NCDevArray.from_host(x), nca.NCDevArray.from_host(y), c, (0.0, 1.0), (0.0, 1.0))
        return c
    finally:
        if old is None:
            del os.environ["NCA_HIST_PATH"]
        else:
            os.environ["NCA_HIST_PATH"] = old


def _mixture(rng, n):
    centres = rng.uniform(0, 1, (8, 2))
    sigma = rng.uniform(0.01, 0.1, 8)
    comp = rng.choice(8, size=n, p=rng.dirichlet(np.full(8, 0.5)))
    pts = centres[comp] + rng.normal(size=(n, 2)) * sigma[comp, None]
    return pts[:, 0].astype(np.float32), pts[:, 1].astype(np.float32)


@pytest.mark.parametrize("path", ["tile", "direct"])
@pytest.mark.parametrize("n,nbx,nby", [(1 << 21, 1024, 1024), (1_000_003, 999, 1001), (1 << 20, 1, 1),
                                       (1_048_579, 37, 61)])
def test_counts_match_oracle(cuda, orc, path, n, nbx, nby):
    rng = np.random.default_rng(SEED + 900 + n % 97)
    x, y = _mixture(rng, n)
    x[:3] = [np.nan, -0.5, 1.0]
    want, _ = orc.hist2d(x, y, None, nbx, nby, 0.0, 1.0, 0.0, 1.0)
    got = _counts(path, x, y, nbx, nby).to_host().reshape(-1)
    assert np.array_equal(got, want)


def test_hot_bins_and_accumulation(cuda, orc):
    """3 Mi points: 40 % in one bin, 20 % in another, the rest spread."""
    rng = np.random.default_rng(SEED + 910)
    n = 3 << 20
    x, y = _mixture(rng, n)
    hot = rng.random(n)
    x[hot < 0.4], y[hot < 0.4] = np.float32(0.5001), np.float32(0.25001)
    sel = (hot >= 0.4) & (hot < 0.6)
    x[sel], y[sel] = np.float32(0.0), np.float32(0.99999)
    want, _ = orc.hist2d(x, y, None, 1024, 1024, 0.0, 1.0, 0.0, 1.0)
    c = _counts("tile", x, y, 1024, 1024)
    assert np.array_equal(c.to_host().reshape(-1), want)
    _counts("tile", x, y, 1024, 1024, out=c)   # a second call adds to the same output
    assert np.array_equal(c.to_host().reshape(-1), 2 * want)


def test_paths_agree(cuda):
    rng = np.random.default_rng(SEED + 920)
    n = (1 << 21) + 5
    x, y = _mixture(rng, n)
    got = {p: _counts(p, x, y, 1024, 1024).to_host() for p in ("tile", "direct")}
    assert np.array_equal(got["tile"], got["direct"])
    assert int(got["tile"].sum()) <= n
