"""Host <-> device copies of strided views (nca_copy_host) vs numpy slicing:
bit-exact, both directions, numpy and pinned torch host buffers."""
import numpy as np
import pytest

import ncarray_gb300 as nca
from ncarray_gb300 import _lib
from tests.helpers import SEED

pytestmark = pytest.mark.gpu


def test_chunk_views_both_directions(cuda):
    import torch
    rng = np.random.default_rng(SEED + 90)
    x = rng.normal(size=(16, 64, 32, 8)).astype(np.float32)
    d = nca.NCDevArray(x.shape, nca.DType.float32).fill(0.0)
    for b0 in range(0, 64, 16):
        d[:, b0:b0 + 16].copy_from(x[:, b0:b0 + 16])
    torch.cuda.synchronize()
    assert np.array_equal(d.to_host(), x)
    # device -> pinned host, chunk by chunk, on a side stream
    h = torch.zeros(x.shape, dtype=torch.float32).pin_memory()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        for b0 in range(0, 64, 32):
            d[:, b0:b0 + 32].copy_to(h[:, b0:b0 + 32])
    s.synchronize()
    assert np.array_equal(h.numpy(), x)


def test_inner_slices_and_every_rank(cuda):
    rng = np.random.default_rng(SEED + 91)
    a = rng.integers(-100, 100, size=(5, 7, 9, 12)).astype(np.int32)
    d = nca.NCDevArray.from_host(a)
    out = np.zeros((5, 3, 9, 4), np.int32)
    d[:, 2:5, :, 3:7].copy_to(out)      # innermost run of 4 elements, three outer axes
    import torch
    torch.cuda.synchronize()
    assert np.array_equal(out, a[:, 2:5, :, 3:7])
    v = np.arange(12, dtype=np.int32)
    e = nca.NCDevArray((12,), nca.DType.int32).copy_from(v)
    torch.cuda.synchronize()
    assert np.array_equal(e.to_host(), v)


def test_rejected_views(cuda):
    d = nca.NCDevArray((4, 8), nca.DType.float32)
    with pytest.raises(Exception):
        d.copy_from(np.zeros((4, 9), np.float32))            # shape differs
    with pytest.raises(Exception):
        d.transpose(1, 0).copy_from(np.zeros((8, 4), np.float32))   # innermost axis strided on the device
    with pytest.raises(Exception):
        d.copy_from(np.zeros((4, 8), np.float64))            # itemsize differs
