"""3-D stencils on the GPU vs the float64 oracle.

float64 grids: max |gpu - oracle| <= 1e-12 max|oracle| (fused multiply-adds in a
different order). float32 grids: relative L2 error <= 2e-6 and max error
<= 1e-5 max|oracle| after the stated iterations. Shapes cover the TMA path
(x extent a multiple of 4, partial tiles at every edge) and the direct path."""
import numpy as np
import pytest

import ncarray_gb300 as nca
from ncarray_gb300.stencil import Stencil3D, device_status, laplacian7, laplacian27
from tests.helpers import SEED

pytestmark = pytest.mark.gpu

SHAPES = [(20, 36, 68), (33, 17, 132), (9, 40, 64), (7, 11, 13), (5, 6, 30)]


def run(u, w, dt, iters, dtype):
    a = nca.NCDevArray.from_host(u.astype(dtype))
    b = nca.NCDevArray(u.shape, a.dtype)
    res = Stencil3D(w, dt).iterate(a, b, iters)
    out = res.to_host()
    assert device_status() == 0
    return out


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("kind", ["7", "27", "random"])
def test_stencil_f64(cuda, orc, shape, kind):
    rng = np.random.default_rng(SEED + 3)
    u = rng.normal(size=shape)
    w = {"7": laplacian7(), "27": laplacian27(), "random": rng.normal(size=(3, 3, 3))}[kind].reshape(27)
    for iters in (1, 2, 3):
        ref = orc.stencil3d_f64(u, w, 0.1, iters)
        got = run(u, w, 0.1, iters, np.float64)
        assert np.max(np.abs(got - ref)) <= 1e-12 * max(np.max(np.abs(ref)), 1.0), (shape, kind, iters)


@pytest.mark.parametrize("shape", SHAPES[:3])
@pytest.mark.parametrize("kind", ["7", "27", "random"])
def test_stencil_f32_error_vs_f64(cuda, orc, shape, kind):
    """7-point (star kernel), isotropic 27-point (centre/face/corner sums) and
    arbitrary 27 weights (general kernel)."""
    rng = np.random.default_rng(SEED + 3)
    u = rng.normal(size=shape).astype(np.float32)
    w = {"7": laplacian7(), "27": laplacian27(), "random": rng.normal(size=(3, 3, 3)) / 8}[kind].reshape(27)
    iters = 3 if kind == "random" else 10
    ref = orc.stencil3d_f64(u.astype(np.float64), w, 0.1, iters)
    got = run(u, w, 0.1, iters, np.float32).astype(np.float64)
    rel_l2 = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert rel_l2 <= 2e-6, rel_l2
    assert np.max(np.abs(got - ref)) <= 1e-5 * np.max(np.abs(ref))


def test_stencil_zero_weights_copy_and_validation(cuda):
    rng = np.random.default_rng(SEED + 4)
    u = rng.normal(size=(8, 8, 64)).astype(np.float32)
    got = run(u, np.zeros(27), 0.1, 1, np.float32)
    assert np.array_equal(got, u)
    a = nca.NCDevArray.from_host(u)
    with pytest.raises(nca.NcaError):
        Stencil3D(laplacian7(), 0.1).apply(a, a)          # source and destination overlap
    with pytest.raises(nca.NcaError):
        Stencil3D(laplacian7(), 0.1).apply(a, nca.NCDevArray((8, 8, 32), nca.DType.float32))
