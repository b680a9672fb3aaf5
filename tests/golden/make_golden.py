"""Generates tests/golden/ref_golden.npz from ncarray's OWN host code.

Run where the reference sources are present (the oracle Makefile compiles them
into oracle/_ref/libncref.so):  python tests/golden/make_golden.py
Every case stores its seeded inputs and the reference's output, so the oracle
restatement can be pinned on machines without the reference.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402

OUT = Path(__file__).resolve().parent / "ref_golden.npz"
I = lambda op, i=0: (op << 24) | i  # noqa: E731

# ncarray dtype numbers
B, U8, U16, U32, U64, I8, I16, I32, I64, F32, F64 = 0, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11
NP = {B: np.bool_, U8: np.uint8, U16: np.uint16, U32: np.uint32, U64: np.uint64, I8: np.int8,
      I16: np.int16, I32: np.int32, I64: np.int64, F32: np.float32, F64: np.float64}


def data(rng, shape, dt):
    if dt == B:
        return rng.integers(0, 2, shape).astype(np.bool_)
    if dt in (F32, F64):
        return rng.normal(size=shape).astype(NP[dt])
    info = np.iinfo(NP[dt])
    lo, hi = max(info.min, -1000), min(info.max, 1000)
    return rng.integers(lo, hi + 1, shape).astype(NP[dt])


def slot(value, dt):
    raw = np.array([value]).astype(NP[dt]).tobytes()
    b = np.zeros(8, dtype=np.uint8)
    b[: len(raw)] = np.frombuffer(raw, dtype=np.uint8)
    return int(b.view(np.uint64)[0])


def promote(a, b):
    return max(a, b)


SUM = {B: U64, U8: U64, U16: U64, I8: I64, I16: I64}


def res_dtype(op, w):
    if op in (20, 21, 22, 23, 24, 25, 26, 27, 12):
        return B
    if op == 14:
        return SUM.get(w, w)
    if op == 15:
        return I64 if w in (B, U8, U16, I8, I16) else w
    if op == 17:
        return F64
    return w


def stencil_weights(kind, rng):
    w = np.zeros((3, 3, 3))
    if kind == "7":
        w[1, 1, 1] = -6.0
        for dz, dy, dx in ((0, 1, 1), (2, 1, 1), (1, 0, 1), (1, 2, 1), (1, 1, 0), (1, 1, 2)):
            w[dz, dy, dx] = 1.0
    elif kind == "27":
        for dz in range(3):
            for dy in range(3):
                for dx in range(3):
                    far = (dz != 1) + (dy != 1) + (dx != 1)
                    w[dz, dy, dx] = {0: -128.0, 1: 14.0, 2: 3.0, 3: 1.0}[far] / 30.0
    else:   # no symmetry, a few zero weights
        w = rng.normal(size=(3, 3, 3)) * (rng.random((3, 3, 3)) < 0.8)
    return w.reshape(27)


def ref_stencil_step(u, w27, dt):
    """One step u + dt * sum_o w[o] u[. + o] with zero halo, evaluated by the
    reference's stack VM over 27 shifted views of a zero-padded copy (the
    shifted-view pattern of examples/benchmark_binning.cc:36-110). The terms
    are added in (dz, dy, dx) order, zero weights left out."""
    nz, ny, nx = u.shape
    pad = np.zeros((nz + 2, ny + 2, nx + 2))
    pad[1:-1, 1:-1, 1:-1] = u
    views, scalars = [], [(F64, slot(dt, F64))]
    centre = len(views)
    views.append((pad[1:1 + nz, 1:1 + ny, 1:1 + nx], F64))
    instrs = [I(2, centre), I(4, 0)]
    first = True
    for o in range(27):
        if w27[o] == 0.0:
            continue
        dz, dy, dx = o // 9, (o // 3) % 3, o % 3
        views.append((pad[dz:dz + nz, dy:dy + ny, dx:dx + nx], F64))
        scalars.append((F64, slot(w27[o], F64)))
        instrs += [I(4, len(scalars) - 1), I(2, len(views) - 1), I(16)]
        if not first:
            instrs.append(I(14))
        first = False
    instrs += [I(16), I(14)]
    return oracle.ref_expr_eval(instrs, scalars, F64, F64, views, u.shape)


def hist_bins(x, y, nbx, nby, xr, yr):
    """Bin index of every point (-1 = dropped) by the float32 rule of
    nca_hist2d: floor((x - lo) * s) with s = float32(nb / (hi - lo))."""
    sx, sy = np.float32(nbx / (xr[1] - xr[0])), np.float32(nby / (yr[1] - yr[0]))
    fx = np.floor((x - np.float32(xr[0])) * sx)
    fy = np.floor((y - np.float32(yr[0])) * sy)
    ok = (fx >= 0) & (fx < nbx) & (fy >= 0) & (fy < nby)
    return np.where(ok, np.where(ok, fy, 0).astype(np.int64) * nbx + np.where(ok, fx, 0).astype(np.int64), -1)


def add_path_cases(store, meta):
    """Stencil, histogram, batched-reduction and scatter-add cases from the
    reference's own code (its VM, host::scatter_add_recursive and ArrayImpl
    reductions), with their own seed so that the cases above stay as they were."""
    rng = np.random.default_rng(20261204)
    for kind, shape, iters in (("7", (5, 6, 7), 2), ("27", (4, 9, 8), 3), ("rand", (6, 5, 4), 1)):
        u0 = rng.normal(size=shape)
        w = stencil_weights(kind, rng)
        u = u0
        for _ in range(iters):
            u = ref_stencil_step(u, w, 0.1)
        i = len(meta)
        store[f"s{i}_in"], store[f"s{i}_w"], store[f"s{i}_out"] = u0, w, u
        meta.append({"kind": "stencil", "name": kind, "dt": 0.1, "iters": iters})
    for n, nbx, nby, xr, yr in ((6000, 16, 12, (0.0, 1.0), (0.0, 1.0)), (4000, 7, 9, (-0.5, 1.5), (0.25, 0.75))):
        centres = rng.uniform(0, 1, (8, 2))
        sigma = rng.uniform(0.01, 0.1, 8)
        comp = rng.choice(8, size=n, p=rng.dirichlet(np.full(8, 0.5)))
        pts = (centres[comp] + rng.normal(size=(n, 2)) * sigma[comp, None]).astype(np.float32)
        x, y = np.ascontiguousarray(pts[:, 0]), np.ascontiguousarray(pts[:, 1])
        x[:5] = np.array([np.nan, -0.0, 1.0, np.inf, -1e-8], dtype=np.float32)
        w = rng.lognormal(0, 1, n).astype(np.float32)
        b = hist_bins(x, y, nbx, nby, xr, yr)
        counts = np.zeros(nbx * nby, dtype=np.uint64)
        wsum = np.zeros(nbx * nby, dtype=np.float64)
        oracle.ref_scatter_add(counts, U64, b, I64, np.ones(n, dtype=np.uint64), U64)
        oracle.ref_scatter_add(wsum, F64, b, I64, w, F32)
        i = len(meta)
        store[f"h{i}_x"], store[f"h{i}_y"], store[f"h{i}_w"] = x, y, w
        store[f"h{i}_counts"], store[f"h{i}_wsum"] = counts, wsum
        meta.append({"kind": "hist", "nbx": nbx, "nby": nby, "xr": list(xr), "yr": list(yr)})
    # batched reductions: per array the reference's ArrayImpl::sum / mean / max
    # and the sum of its VM's x*x - x (bfloat16 arrays widened exactly to float32:
    # the reference has no bfloat16)
    lens = np.round(np.exp(rng.uniform(np.log(64), np.log(5000), 12))).astype(np.int64)
    for j, L in enumerate(lens):
        xf = (np.exp(rng.normal(size=L) * 2.0) * rng.choice([-1.0, 1.0], L)).astype(np.float32)
        dt = F32
        if j % 2:
            raw = (xf.view(np.uint32) >> 16).astype(np.uint16)
            xf = (raw.astype(np.uint32) << 16).view(np.float32)
            dt = 22
        res = {}
        for name, op in (("sum", 0), ("mean", 1), ("max", 2)):
            val, odt = oracle.ref_reduce_full(xf, F32, op)
            res[name] = [float(val), odt]
        sq = oracle.ref_expr_eval([I(2, 0), I(2, 0), I(16), I(2, 0), I(15)], [], F32, F32, [(xf, F32)], xf.shape)
        val, odt = oracle.ref_reduce_full(sq, F32, 0)
        res["sum_sq_m"] = [float(val), odt]
        i = len(meta)
        store[f"b{i}_x"] = raw if dt == 22 else xf
        meta.append({"kind": "batch", "dtype": dt, "ref": res})
    # scatter-add: dest dtype x index dtype x src dtype, ragged 2-D index/src views
    for ddt, idt, sdt in ((I64, I64, I32), (U64, I32, U64), (F32, I64, F32), (F64, I32, F32), (I32, U32, I32),
                          (F64, I64, F64)):
        shape = (int(rng.integers(3, 9)), int(rng.integers(5, 40)))
        n_dest = int(rng.integers(5, 200))
        idx = rng.integers(-5, n_dest + 5, shape).astype(NP[idt] if idt != U32 else np.uint32)
        src = (rng.normal(size=shape) * 50).astype(NP[sdt]) if sdt in (F32, F64) else \
            rng.integers(-1000, 1000, shape).astype(NP[sdt])
        dest = np.zeros(n_dest, dtype=NP[ddt])
        oracle.ref_scatter_add(dest, ddt, idx, idt, src, sdt)
        i = len(meta)
        store[f"x{i}_idx"], store[f"x{i}_src"], store[f"x{i}_dest"] = idx, src, dest
        meta.append({"kind": "scatter", "dest": ddt, "idx": idt, "src": sdt})


def main():
    if oracle.ref() is None:
        oracle.build(with_ref=True)
    assert oracle.ref() is not None, "reference host code not built"
    rng = np.random.default_rng(20261203)
    store, meta = {}, []

    def add_expr(name, instrs, scalars, operands, work, expr):
        out_shape = np.broadcast_shapes(*[a.shape for a, _ in operands])
        ops = [(np.ascontiguousarray(np.broadcast_to(a, out_shape)), d) for a, d in operands]
        y = oracle.ref_expr_eval(instrs, scalars, work, expr, ops, out_shape)
        i = len(meta)
        for k, (a, d) in enumerate(ops):
            store[f"e{i}_op{k}"] = a
        store[f"e{i}_out"] = y
        meta.append({"kind": "expr", "name": name, "instrs": instrs, "scalars": scalars,
                     "op_dtypes": [d for _, d in ops], "work": work, "expr": expr})

    # C1 without the ops the reference lacks: a*b + c - 0.5*a (float64)
    a, b, c = (rng.uniform(-1, 1, (6, 8, 10)) for _ in range(3))
    add_expr("c1_core", [I(2, 0), I(2, 1), I(16), I(2, 2), I(14), I(4, 0), I(2, 0), I(16), I(15)],
             [(F32, slot(0.5, F32))], [(a, F64), (b, F64), (c, F64)], F64, F64)
    # C2 fusion on a permuted view and a broadcast vector (float32 with int32)
    x = rng.normal(size=(4, 16, 8, 8)).astype(np.float32).transpose(3, 1, 2, 0)
    v = rng.normal(size=(1, 16, 1, 1)).astype(np.float32)
    k = rng.integers(-1000, 1001, x.shape).astype(np.int32)
    add_expr("c2_y", [I(2, 0), I(2, 1), I(16), I(2, 2), I(14)], [], [(x, F32), (v, F32), (k, I32)], F32, F32)
    add_expr("c2_int", [I(2, 0), I(4, 0), I(16), I(4, 1), I(14), I(4, 2), I(18)],
             [(U8, 3), (U8, 7), (U8, 11)], [(k, I32)], I32, I32)
    # random tapes over the integer and float dtypes
    binops = [14, 15, 16, 17, 18, 20, 21, 22, 23, 24, 25, 26, 27]
    # LNOT is left out: the reference VM skips it (dynamicmvnode.hh:203-204), a
    # defect the library does not reproduce (LNOT negates here).
    unops = [5, 6, 7]
    for t in range(40):
        dt1 = int(rng.choice([B, U8, U16, U32, U64, I8, I16, I32, I64, F32, F64]))
        dt2 = int(rng.choice([dt1, I32, F32, U8]))
        shape = (3, 5, 4)
        p, q = data(rng, shape, dt1), data(rng, shape, dt2)
        op = int(rng.choice(binops))
        work = promote(dt1, dt2)
        instrs = [I(2, 0), I(2, 1), I(op)]
        expr = res_dtype(op, work)
        if rng.random() < 0.5:
            u = int(rng.choice(unops))
            instrs.append(I(u))
            expr = B if u == 12 else work  # unary ops take the work dtype (mvnode.hh:339-369)
        if op in (18,) and dt1 not in (F32, F64) and work not in (F32, F64):
            q = np.where(q == 0, 1, q).astype(q.dtype)
            if work in (I8, I16, I32, I64):
                q = np.where(q == -1, 2, q).astype(q.dtype)
        compute = work if expr == B else expr
        if compute in (I8, I16, I32, I64, U8, U16, U32, U64, B) and op == 17:
            continue
        add_expr(f"rand{t}", instrs, [], [(p, dt1), (q, dt2)], work, expr)
    # reductions
    for dt in (B, U8, I16, I32, U32, I64, F32, F64):
        h = data(rng, (5, 6, 7), dt)
        i = len(meta)
        store[f"r{i}_in"] = h
        full = {}
        for op in (0, 1, 2, 3, 4, 5):
            val, odt = oracle.ref_reduce_full(h, dt, op)
            full[op] = [val.item() if hasattr(val, "item") else val, odt]
        axes = {}
        for mask_axes in ([0], [1], [2], [0, 2], [1, 2]):
            for op in (0, 2, 3):
                y, odt = oracle.ref_reduce_axes(h, dt, op, mask_axes)
                key = f"{op}_{'_'.join(map(str, mask_axes))}"
                store[f"r{i}_ax_{key}"] = y
                axes[key] = odt
        meta.append({"kind": "reduce", "dtype": dt, "full": {str(k): v for k, v in full.items()}, "axes": axes})
    add_path_cases(store, meta)
    store["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(OUT, **store)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(meta)} cases)")


if __name__ == "__main__":
    main()
