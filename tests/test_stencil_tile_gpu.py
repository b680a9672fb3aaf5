"""The tiled form of nca_stencil (shared-memory planes, a register window
along z) against the view form (one strided view per offset through the
expression kernels) and the oracle, bit for bit: both forms evaluate the same
tape with the same operand conversion and the same operations in the same
order.

Cases: the 7- and 27-point Laplacians on zero-padded float32 and float64
grids whose extents are not multiples of the tile; an int32 tape with DIV and
GT over asymmetric offsets; bfloat16 (staged by plain loads, not cp.async);
2-D and 1-D sets; strided sources and a transposed destination; many z chunks
with a ragged last one; every tile shape the planner can pick and a few more
set through NCA_STENCIL_TILE_CFG. NCA_STENCIL_TILE=2 makes the call fail when
the tiled form does not apply, so every case here is known to run on it."""
import contextlib
import os

import numpy as np
import pytest

import ncarray_gb300 as nca
from ncarray_gb300.dtype import DType
from ncarray_gb300.stencil import Stencil, laplacian7, laplacian27
from tests.helpers import SEED
from tests.test_stencil_general_gpu import oracle_stencil

pytestmark = pytest.mark.gpu


@contextlib.contextmanager
def _env(**kv):
    old = {k: os.environ.get(k) for k in kv}
    try:
        for k, v in kv.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
        yield
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def _both(st, src, dest_shape, dest_dt, cfg=None):
    """(tiled result, view-form result) as host arrays."""
    out = []
    for mode in ("2", "0"):
        d = nca.NCDevArray(dest_shape, dest_dt)
        with _env(NCA_STENCIL_TILE=mode, NCA_STENCIL_TILE_CFG=cfg):
            st.apply(src, d)
        out.append(d.to_host())
    return out


def _laplacian_stencil(w, dt, scale):
    wl = [float(v) for v in np.asarray(w).reshape(27)]
    used = [t for t in range(27) if wl[t] != 0.0]
    offs = [(t // 9, (t // 3) % 3, t % 3) for t in used]
    cast = np.float64 if dt == DType.float64 else np.float32
    centre = used.index(13)

    def lap(v):
        acc = None
        for k, t in enumerate(used):
            term = nca.DevExpr.leaf(v[k]) * cast(wl[t])
            acc = term if acc is None else acc + term
        return nca.DevExpr.leaf(v[centre]) + acc * cast(scale)

    return Stencil.create(offs, lap, dt)


@pytest.mark.parametrize("dt", [DType.float32, DType.float64])
@pytest.mark.parametrize("w", ["7", "27"])
@pytest.mark.parametrize("shape", [(37, 45, 70), (5, 130, 257), (300, 11, 40)])
def test_laplacians_on_padded_grids(cuda, orc, dt, w, shape):
    rng = np.random.default_rng(SEED + 1400 + shape[0] + int(dt))
    nz, ny, nx = shape
    npdt = np.float32 if dt == DType.float32 else np.float64
    pad = np.zeros((nz + 2, ny + 2, nx + 2), npdt)
    pad[1:-1, 1:-1, 1:-1] = rng.normal(size=shape)
    st = _laplacian_stencil(laplacian7() if w == "7" else laplacian27(), dt, 0.1)
    src = nca.NCDevArray.from_host(pad)
    tiled, view = _both(st, src, shape, dt)
    assert tiled.tobytes() == view.tobytes()
    if shape[0] <= 40:
        want = oracle_stencil(orc, st, pad, int(dt), shape, int(dt))
        assert tiled.tobytes() == want.tobytes()


def test_int32_tape_asymmetric_offsets(cuda, orc):
    rng = np.random.default_rng(SEED + 1410)
    src_h = rng.integers(-1000, 1000, (40, 33, 75)).astype(np.int32)
    offs = [(0, 0, 0), (1, 2, 3), (2, 0, 1), (0, 3, 2), (1, 1, 0)]

    def f(v):
        return (v[0] * v[1] - v[2] / 7 + (v[3] > v[4]) * 3) % 1001 - v[4]

    st = Stencil.create(offs, f, DType.int32)
    dest_shape = (38, 30, 72)
    tiled, view = _both(st, nca.NCDevArray.from_host(src_h), dest_shape, st.result_dtype)
    assert tiled.tobytes() == view.tobytes()
    want = oracle_stencil(orc, st, src_h, int(DType.int32), dest_shape, int(st.result_dtype))
    assert tiled.tobytes() == want.tobytes()


def test_bfloat16_plain_load_staging(cuda, orc):
    """2-byte elements are staged by plain loads (cp.async takes 4, 8 or 16)."""
    rng = np.random.default_rng(SEED + 1420)
    f = rng.normal(size=(18, 40, 90)).astype(np.float32)
    hb = (f.view(np.uint32) >> 16).astype(np.uint16)       # bfloat16 bit patterns
    src = nca.NCDevArray.from_host(hb, DType.bfloat16)
    st = _laplacian_stencil(laplacian7(), DType.bfloat16, 0.25)
    tiled, view = _both(st, src, (16, 38, 88), st.result_dtype)
    assert tiled.tobytes() == view.tobytes()
    want = oracle_stencil(orc, st, hb, int(DType.bfloat16), (16, 38, 88), int(st.result_dtype))
    assert tiled.tobytes() == want.tobytes()


def test_two_and_one_dims(cuda, orc):
    rng = np.random.default_rng(SEED + 1430)
    h2 = rng.normal(size=(131, 260)).astype(np.float32)
    st2 = Stencil.create([(1, 1), (0, 1), (2, 1), (1, 0), (1, 2)],
                         lambda v: v[0] * np.float32(-4.0) + v[1] + v[2] + v[3] + v[4], DType.float32)
    tiled, view = _both(st2, nca.NCDevArray.from_host(h2), (129, 258), DType.float32)
    assert tiled.tobytes() == view.tobytes()
    assert tiled.tobytes() == oracle_stencil(orc, st2, h2, 10, (129, 258), 10).tobytes()
    h1 = rng.normal(size=5000)
    st1 = Stencil.create([(0,), (2,), (4,)], lambda v: (v[0] - v[1] * 2.0 + v[2]) / 3.0, DType.float64)
    tiled, view = _both(st1, nca.NCDevArray.from_host(h1), (4996,), DType.float64)
    assert tiled.tobytes() == view.tobytes()
    assert tiled.tobytes() == oracle_stencil(orc, st1, h1, 11, (4996,), 11).tobytes()


def test_strided_source_and_transposed_destination(cuda, orc):
    rng = np.random.default_rng(SEED + 1440)
    big = rng.normal(size=(24, 30, 2 * 66)).astype(np.float32)
    src = nca.NCDevArray.from_host(big)[:, :, ::2]          # x stride 8 bytes
    sh = np.ascontiguousarray(big[:, :, ::2])
    st = _laplacian_stencil(laplacian27(), DType.float32, 0.5)
    dest_shape = (22, 28, 64)
    want = oracle_stencil(orc, st, sh, 10, dest_shape, 10)
    tiled, view = _both(st, src, dest_shape, DType.float32)
    assert tiled.tobytes() == view.tobytes() == want.tobytes()
    # the destination as a transposed view of a (64, 28, 22) array
    for mode in ("2", "0"):
        base = nca.NCDevArray((64, 28, 22), DType.float32)
        with _env(NCA_STENCIL_TILE=mode):
            st.apply(src, base.permute(2, 1, 0))
        assert np.ascontiguousarray(base.to_host().transpose(2, 1, 0)).tobytes() == want.tobytes()


@pytest.mark.parametrize("cfg", ["1,1,4,2,7", "2,2,8,3,16", "4,1,16,5,5", "1,4,8,4,128", "2,1,8,8,1", "1,8,8,3,32,2",
                                 "1,2,2,1,9,8"])
def test_tile_shapes(cuda, cfg):
    rng = np.random.default_rng(SEED + 1450)
    shape = (45, 70, 150)
    pad = np.zeros((shape[0] + 2, shape[1] + 2, shape[2] + 2), np.float32)
    pad[1:-1, 1:-1, 1:-1] = rng.normal(size=shape)
    src = nca.NCDevArray.from_host(pad)
    for w in (laplacian7(), laplacian27()):
        st = _laplacian_stencil(w, DType.float32, 0.1)
        tiled, view = _both(st, src, shape, DType.float32, cfg=cfg)
        assert tiled.tobytes() == view.tobytes()


def test_where_the_tiled_form_does_not_apply(cuda):
    """A source/destination ratio other than 1, a pointer-axis source and a
    destination over the source take the view form; forced, they fail."""
    h = np.zeros((8, 16, 32), np.float32)
    src = nca.NCDevArray.from_host(h)
    st = Stencil.create([(0, 0, 0), (1, 1, 1)], lambda v: v[0] + v[1], DType.float32)
    with _env(NCA_STENCIL_TILE="2"):
        with pytest.raises(nca.NcaError, match="ratio"):
            st.apply(src, nca.NCDevArray((4, 8, 16), DType.float32))
        with pytest.raises(nca.NcaError, match="overlaps"):
            st.apply(src, src[:7, :15, :31])
        P = nca.NCDevArray.from_panels([nca.NCDevArray.from_host(h[i]) for i in range(8)])
        with pytest.raises(nca.NcaError, match="pointer"):
            st.apply(P, nca.NCDevArray((7, 15, 31), DType.float32))
    # the default mode falls back to the view form for the same calls
    out = nca.NCDevArray((7, 15, 31), DType.float32)
    st.apply(P, out)
    assert np.array_equal(out.to_host(), np.zeros((7, 15, 31), np.float32))


@pytest.mark.parametrize("w", ["7", "27"])
def test_column_pairs_opt_in(cuda, orc, w):
    """NCA_STENCIL_TILE_PK=1: float32 tapes evaluated on column pairs in packed
    f32x2 fused multiply-adds, bit for bit the view form and the oracle."""
    rng = np.random.default_rng(SEED + 1460 + int(w))
    shape = (21, 70, 150)
    pad = np.zeros((shape[0] + 2, shape[1] + 2, shape[2] + 2), np.float32)
    pad[1:-1, 1:-1, 1:-1] = rng.normal(size=shape)
    st = _laplacian_stencil(laplacian7() if w == "7" else laplacian27(), DType.float32, 0.1)
    src = nca.NCDevArray.from_host(pad)
    with _env(NCA_STENCIL_TILE_PK="1"):
        tiled, view = _both(st, src, shape, DType.float32)
    assert tiled.tobytes() == view.tobytes()
    assert tiled.tobytes() == oracle_stencil(orc, st, pad, 10, shape, 10).tobytes()
    # a tape with division, negation and absolute value
    st2 = Stencil.create([(0, 0, 0), (1, 1, 1), (2, 2, 2)], lambda v: -abs(v[0] - v[1]) / (v[2] * np.float32(3.0) + 7.0),
                         DType.float32)
    with _env(NCA_STENCIL_TILE_PK="1"):
        tiled, view = _both(st2, src, shape, st2.result_dtype)
    assert tiled.tobytes() == view.tobytes()
