"""The workloads at their full sizes (C1 128^3, C2 (8,256,256,64), C3 512^3,
C4 2^27 points, C5 20,000 arrays) and beyond 2^31 elements. Where the oracle
would take too long the checks are exact independent computations (numpy
fmod/argmax, separately rounded float32 multiply-then-add, a float64
convolution) or size-independent properties (point totals, mean = sum/len);
C1 and C4 run the oracle itself."""
import numpy as np
import pytest

import ncarray_gb300 as nca
from ncarray_gb300.dtype import DType, RedOp
from tests.helpers import SEED, assert_bits_equal

pytestmark = pytest.mark.gpu


def test_c2_full_size(cuda):
    import torch
    rng = np.random.default_rng(SEED + 200)
    x = rng.normal(size=(64, 256, 256, 8)).astype(np.float32)
    v = rng.normal(size=256).astype(np.float32)
    k = rng.integers(-1000, 1001, size=(8, 256, 256, 64)).astype(np.int32)
    dx, dv, dk = nca.NCDevArray.from_host(x), nca.NCDevArray.from_host(v), nca.NCDevArray.from_host(k)
    with nca.lazy_mode():
        y = dx.permute(3, 1, 2, 0) * dv.reshape(1, 256, 1, 1) + dk
        z = (dk * 3 + 7) % 11
    out = nca.NCDevArray(y.shape, y.dtype)
    mx, am = y.evaluate(out=out, reductions=[(RedOp.MAX, 2), (RedOp.ARGMAX, 2)])
    zo = nca.NCDevArray(z.shape, z.dtype)
    z.evaluate(out=zo)
    # float32 multiply then add, each rounded once (no contraction): torch's
    # separate kernels round the same way
    tx = torch.from_numpy(x).cuda().permute(3, 1, 2, 0)
    ty = tx * torch.from_numpy(v).cuda().view(1, 256, 1, 1)
    ty = ty + torch.from_numpy(k).cuda().float()
    yh = ty.cpu().numpy()
    assert_bits_equal(out.to_host(), yh, "C2 y at full size")
    assert_bits_equal(mx.to_host(), yh.max(axis=2), "C2 max at full size")
    assert np.array_equal(am.to_host(), yh.argmax(axis=2)), "C2 argmax (first index) at full size"
    assert np.array_equal(zo.to_host(), np.fmod(k * 3 + 7, 11)), "C2 int expression at full size"


def test_c1_full_size_oracle(cuda, orc):
    from tests.helpers import oracle_eval
    rng = np.random.default_rng(SEED + 201)
    a, b, c = (rng.uniform(-1, 1, (128, 128, 128)) for _ in range(3))
    da, db, dc = (nca.NCDevArray.from_host(t) for t in (a, b, c))
    with nca.lazy_mode():
        e = da * db + nca.sqrt(abs(dc)) - 0.5 * da
    out = nca.NCDevArray(e.shape, e.dtype)
    s0, mx = e.evaluate(out=out, reductions=[(RedOp.SUM, 0), (RedOp.MAX, 0)])
    ref = oracle_eval(orc, e, [a, b, c])
    assert_bits_equal(out.to_host(), ref, "C1 out")
    assert_bits_equal(mx.to_host(), orc.reduce(ref, int(DType.float64), int(RedOp.MAX), 0), "C1 axis-0 max")
    want = orc.reduce(ref, int(DType.float64), int(RedOp.SUM), 0)
    assert np.all(np.abs(s0.to_host() - want) <= 1e-12 * np.abs(ref).sum(axis=0) + 1e-300)


@pytest.mark.parametrize("kind", ["7", "27"])
def test_c3_full_size_f64_vs_convolution(cuda, kind):
    """512^3 float64, 2 Jacobi steps, against torch's float64 conv3d (an
    independent implementation): |diff| <= 1e-12 max|u|."""
    import torch
    from ncarray_gb300.stencil import Stencil3D, laplacian7, laplacian27
    w = (laplacian7() if kind == "7" else laplacian27()).reshape(3, 3, 3)
    g = torch.Generator(device="cuda").manual_seed(SEED + 202)
    u0 = torch.randn((512, 512, 512), generator=g, device="cuda", dtype=torch.float64)
    a = nca.NCDevArray((512, 512, 512), DType.float64)
    a._buf.view(torch.float64).copy_(u0.reshape(-1))
    b = nca.NCDevArray((512, 512, 512), DType.float64)
    res = Stencil3D(w.reshape(27), 0.1).iterate(a, b, 2)
    got = res._buf[res._offset: res._offset + res.nbytes].view(torch.float64).view(512, 512, 512)
    ker = torch.from_numpy(np.ascontiguousarray(w)).cuda().view(1, 1, 3, 3, 3)
    u = u0
    for _ in range(2):
        u = u + 0.1 * torch.nn.functional.conv3d(u.view(1, 1, 512, 512, 512), ker, padding=1).view(512, 512, 512)
    assert float((got - u).abs().max()) <= 1e-12 * float(u.abs().max())


def test_c4_full_size_counts_oracle(cuda, orc):
    from ncarray_gb300.hist import hist2d
    rng = np.random.default_rng(SEED + 203)
    n = 1 << 27
    centres = rng.uniform(0, 1, (8, 2))
    sigma = rng.uniform(0.01, 0.1, 8)
    comp = rng.choice(8, size=n, p=rng.dirichlet(np.full(8, 0.5)))
    pts = (centres[comp] + rng.normal(size=(n, 2)) * sigma[comp, None]).astype(np.float32)
    x, y = np.ascontiguousarray(pts[:, 0]), np.ascontiguousarray(pts[:, 1])
    del pts, comp
    counts, _ = hist2d(nca.NCDevArray.from_host(x), nca.NCDevArray.from_host(y), 1024, 1024)
    rc, _ = orc.hist2d(x, y, None, 1024, 1024, 0.0, 1.0, 0.0, 1.0)
    got = counts.to_host().reshape(-1)
    assert np.array_equal(got, rc)
    inside = int(np.count_nonzero((x >= 0) & (x < 1) & (y >= 0) & (y < 1)))
    assert int(got.sum()) == inside


def test_c4_full_size_weighted_oracle(cuda, orc):
    """2^27 mixture points with lognormal(0, 1) weights: counts bit-exact and
    per-bin float32 weight sums within one float32 rounding of the float64
    oracle (|got - ref| <= 2^-23 |ref|)."""
    from ncarray_gb300.hist import hist2d
    rng = np.random.default_rng(SEED + 206)
    n = 1 << 27
    centres = rng.uniform(0, 1, (8, 2))
    sigma = rng.uniform(0.01, 0.1, 8)
    comp = rng.choice(8, size=n, p=rng.dirichlet(np.full(8, 0.5)))
    pts = (centres[comp] + rng.normal(size=(n, 2)) * sigma[comp, None]).astype(np.float32)
    x, y = np.ascontiguousarray(pts[:, 0]), np.ascontiguousarray(pts[:, 1])
    del pts, comp
    w = rng.lognormal(0, 1, n).astype(np.float32)
    counts, wsum = hist2d(nca.NCDevArray.from_host(x), nca.NCDevArray.from_host(y), 1024, 1024,
                          w=nca.NCDevArray.from_host(w))
    rc, rw = orc.hist2d(x, y, w, 1024, 1024, 0.0, 1.0, 0.0, 1.0)
    assert np.array_equal(counts.to_host().reshape(-1), rc)
    got = wsum.to_host().reshape(-1).astype(np.float64)
    assert np.all(np.abs(got - rw) <= 2.0**-23 * np.abs(rw) + 1e-30)


@pytest.mark.parametrize("kind", ["7", "27"])
def test_c3_full_size_f32_vs_f64_oracle(cuda, orc, kind):
    """512^3 float32 grid, 10 Jacobi steps u <- u + 0.1 L(u) with zero halo,
    against the float64 oracle from the same (float32) start: relative L2
    error <= 1e-6 and max |err| <= 1e-5 max|u64|."""
    import torch
    from ncarray_gb300.stencil import Stencil3D, laplacian7, laplacian27
    w = (laplacian7() if kind == "7" else laplacian27()).reshape(27)
    rng = np.random.default_rng(SEED + 207)
    u0 = rng.standard_normal((512, 512, 512), dtype=np.float32)
    a = nca.NCDevArray.from_host(u0)
    b = nca.NCDevArray((512, 512, 512), DType.float32)
    res = Stencil3D(w, 0.1).iterate(a, b, 10)
    got = res.to_host().astype(np.float64)
    torch.cuda.synchronize()
    want = orc.stencil3d_f64(u0, w, 0.1, 10)
    err = got - want
    rel_l2 = float(np.sqrt((err * err).sum() / (want * want).sum()))
    assert rel_l2 <= 1e-6, rel_l2
    assert float(np.abs(err).max()) <= 1e-5 * float(np.abs(want).max())


def test_c5_full_size_sampled(cuda, orc):
    """20,000 uneven arrays (log-uniform lengths in [64, 2^22], float32 and
    bfloat16 alternately): 300 sampled arrays against the oracle, and
    mean == sum / length for all."""
    import torch
    from ncarray_gb300.batch import Batch
    rng = np.random.default_rng(SEED + 204)
    n_arrays = 20000
    lens = np.round(np.exp(rng.uniform(np.log(64), np.log(2 ** 22), n_arrays))).astype(np.int64)
    g = torch.Generator(device="cuda").manual_seed(SEED + 204)
    arrays = []
    for i, L in enumerate(lens):
        t = torch.exp(torch.randn(int(L), generator=g, device="cuda") * 2.0)
        t *= torch.where(torch.rand(int(L), generator=g, device="cuda") < 0.5, -1.0, 1.0)
        if i % 2:
            t = t.to(torch.bfloat16)
        a = nca.NCDevArray((int(L),), DType.bfloat16 if i % 2 else DType.float32)
        a._buf.copy_(t.view(torch.uint8).reshape(-1))
        arrays.append(a)
    res = Batch(arrays).run(graph=True).to_host()
    assert np.allclose(res[:, 1], res[:, 0] / lens, rtol=1e-15, atol=0.0)
    pick = rng.choice(n_arrays, 300, replace=False)
    host = []
    for i in pick:
        raw = arrays[i]._buf[: arrays[i].nbytes].cpu().numpy()
        host.append(raw.view(np.float32) if i % 2 == 0 else raw.view(np.uint16))
    ref = orc.batch_reduce(host, [10 if i % 2 == 0 else 22 for i in pick], nthreads=8)
    got = res[pick]
    for j, i in enumerate(pick):
        x = host[j]
        xf = (x.astype(np.uint32) << 16).view(np.float32) if i % 2 else x
        scale = float(np.abs(xf.astype(np.float64)).sum())
        for c in (0, 1, 3):
            assert abs(got[j, c] - ref[j, c]) <= 1e-6 * abs(ref[j, c]) + 1e-9 * scale
        assert got[j, 2] == ref[j, 2]


def test_beyond_2_31_elements(cuda):
    """A full reduction and an expression over 2^31 + 7 int8 elements (the
    64-bit index paths)."""
    import torch
    n = (1 << 31) + 7
    g = torch.Generator(device="cuda").manual_seed(SEED + 205)
    t = torch.randint(-128, 128, (n,), generator=g, device="cuda", dtype=torch.int8)
    a = nca.NCDevArray((n,), DType.int8)
    a._buf.copy_(t.view(torch.uint8))
    s = a.sum()
    want = int(t.to(torch.int64).sum())
    assert int(np.asarray(s.to_host() if hasattr(s, "to_host") else s).reshape(-1)[0]) == want
    with nca.lazy_mode():
        e = a + 1
    out = nca.NCDevArray((n,), e.dtype)
    e.evaluate(out=out)
    ot = out._buf[: out.nbytes].view(torch.int64 if e.dtype == DType.int64 else torch.int16)
    assert int(ot.to(torch.int64).sum()) == want + n
    assert int(ot[-1]) == int(t[-1]) + 1 and int(ot[0]) == int(t[0]) + 1
