"""nca_stencil (ncarray's Stencil<NDIM>: any offsets, any dims, a source /
destination shape ratio, pointer-axis sources) on the GPU.

Every case is compared bit for bit with the oracle evaluating the same tape
in the same compute dtype over numpy views of the same offsets (the kernels
round after every operation, as the oracle does), and the 3-D Laplacian cases
also with the reference's own stack VM over shifted views of a zero-padded
grid (the golden vectors of tests/golden/ref_golden.npz)."""
import json
from pathlib import Path

import numpy as np
import pytest

import ncarray_gb300 as nca
from ncarray_gb300.dtype import DType
from ncarray_gb300.stencil import Stencil
from tests.helpers import SEED

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden" / "ref_golden.npz"


def oracle_stencil(orc, st: Stencil, src: np.ndarray, src_dt: int, dest_shape, dest_dt: int):
    """The stencil evaluated by the oracle: one numpy view per offset."""
    step = [s // d for s, d in zip(src.shape, dest_shape)]
    offs = np.ctypeslib.as_array(st._offs).reshape(st.n, st.ndim)
    views = []
    for o in offs:
        sl = tuple(slice(int(o[d]), int(o[d]) + (dest_shape[d] - 1) * step[d] + 1, step[d]) for d in range(st.ndim))
        views.append((src[sl], src_dt))
    instrs = list(st._ins)
    scalars = [(int(st._sd[i]), int(st._ss[i])) for i in range(st._tape.n_scalars)]
    return orc.expr_eval(instrs, scalars, st._tape.compute_dtype, views, tuple(dest_shape), dest_dt)


def test_stencil_matches_reference_vm_goldens(cuda):
    """The zero-padded Laplacian cases the reference's VM produced: one
    nca_stencil call per Jacobi step over the padded grid (offsets 0..2 on
    each axis, the same tape), float64, bit-exact."""
    z = np.load(GOLDEN)
    meta = json.loads(bytes(z["meta"]).decode())
    n = 0
    for i, m in enumerate(meta):
        if m["kind"] != "stencil":
            continue
        u = z[f"s{i}_in"]
        w = z[f"s{i}_w"]
        offs = [(1, 1, 1)]
        for o in range(27):
            if w[o] != 0.0:
                offs.append((o // 9, (o // 3) % 3, o % 3))

        def expr(v, w=w):
            acc = None
            k = 1
            for o in range(27):
                if w[o] == 0.0:
                    continue
                t = nca.DevExpr.const(np.float64(w[o])) * v[k]
                acc = t if acc is None else acc + t
                k += 1
            return v[0] + nca.DevExpr.const(np.float64(m["dt"])) * acc

        st = Stencil.create(offs, expr, DType.float64)
        nz, ny, nx = u.shape
        for _ in range(m["iters"]):
            pad = np.zeros((nz + 2, ny + 2, nx + 2))
            pad[1:-1, 1:-1, 1:-1] = u
            out = nca.NCDevArray(u.shape, DType.float64)
            st.apply(nca.NCDevArray.from_host(pad), out)
            u = out.to_host()
        assert u.tobytes() == z[f"s{i}_out"].tobytes(), m["name"]
        n += 1
    assert n == 3


def test_pixel_binning_stencil(cuda, orc):
    """The reference benchmark's binning stencil (examples/benchmark_binning.cu:
    343-377): offsets {p, r, c} for p, r, c in 0..1 on a (32, 512, 1024)
    float32 array into (16, 256, 512), sum of the views times a scale."""
    rng = np.random.default_rng(SEED + 400)
    src = rng.normal(size=(32, 512, 1024)).astype(np.float32)
    offs = [(p, r, c) for p in range(2) for r in range(2) for c in range(2)]

    def binning(views):
        e = nca.DevExpr.leaf(views[0])
        for v in views[1:]:
            e = e + v
        return e * np.float32(0.125)

    st = Stencil.create(offs, binning, DType.float32, is_pointer_axis=[0, 0, 0])
    out = nca.NCDevArray((16, 256, 512), DType.float32)
    st.apply(nca.NCDevArray.from_host(src), out)
    want = oracle_stencil(orc, st, src, 10, (16, 256, 512), 10)
    assert out.to_host().tobytes() == want.tobytes()


@pytest.mark.parametrize("dt", [DType.float32, DType.float64, DType.int32])
def test_random_offsets_ops_and_ratio(cuda, orc, dt):
    """Offsets anywhere in range, a source/destination ratio of (2, 1, 3),
    and the reference's stencil operators ADD, SUB, MUL, DIV, GT."""
    rng = np.random.default_rng(SEED + 401 + int(dt))
    src_shape, dest_shape = (22, 17, 61), (10, 14, 19)
    if dt == DType.int32:
        src = rng.integers(-1000, 1000, src_shape).astype(np.int32)
    else:
        src = rng.normal(size=src_shape).astype(np.float32 if dt == DType.float32 else np.float64)
    offs = [(0, 0, 0), (1, 2, 3), (2, 0, 1), (0, 3, 2), (1, 1, 0)]

    def f(v):
        return (v[0] * v[1] - v[2] / 2.5 + (v[3] > v[4]) * 3) - v[4]

    st = Stencil.create(offs, f, dt)
    d = nca.NCDevArray(dest_shape, st.result_dtype)
    st.apply(nca.NCDevArray.from_host(src), d)
    want = oracle_stencil(orc, st, src, int(dt), dest_shape, int(st.result_dtype))
    got = d.to_host()
    assert got.tobytes() == want.tobytes()


def test_stencil_on_pointer_axis_source(cuda, orc):
    """A source made of 12 separate panels (axis 0 is a pointer axis): a
    2x2x2 binning across panels (step 2 along the table), and a shifted
    stencil that starts at panel 1."""
    rng = np.random.default_rng(SEED + 402)
    panels_h = [rng.normal(size=(64, 96)).astype(np.float32) for _ in range(12)]
    P = nca.NCDevArray.from_panels([nca.NCDevArray.from_host(p) for p in panels_h])
    full = np.stack(panels_h)
    offs = [(p, r, c) for p in range(2) for r in range(2) for c in range(2)]

    def binning(views):
        e = nca.DevExpr.leaf(views[0])
        for v in views[1:]:
            e = e + v
        return e

    st = Stencil.create(offs, binning, DType.float32, is_pointer_axis=[1, 0, 0])
    out = nca.NCDevArray((6, 32, 48), DType.float32)
    st.apply(P, out)
    assert out.to_host().tobytes() == oracle_stencil(orc, st, full, 10, (6, 32, 48), 10).tobytes()
    st2 = Stencil.create([(1, 0, 2), (2, 1, 0)], lambda v: v[0] - v[1] * 2.0, DType.float32)
    out2 = nca.NCDevArray((10, 63, 94), st2.result_dtype)
    st2.apply(P, out2)
    want = oracle_stencil(orc, st2, full, 10, (10, 63, 94), int(st2.result_dtype))
    assert out2.to_host().tobytes() == want.tobytes()


def test_stencil_rejects_reads_outside_source(cuda):
    src = nca.NCDevArray.from_host(np.zeros((8, 8), np.float32))
    dest = nca.NCDevArray((8, 8), DType.float32)
    st = Stencil.create([(0, 1)], lambda v: v[0] + 1.0, DType.float32)
    with pytest.raises(nca.NcaError, match="leaves the source"):
        st.apply(src, dest)
    st = Stencil.create([(0, -1)], lambda v: v[0], DType.float32)
    with pytest.raises(nca.NcaError, match="leaves the source"):
        st.apply(src, nca.NCDevArray((8, 7), DType.float32))
