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
    store["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(OUT, **store)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(meta)} cases)")


if __name__ == "__main__":
    main()
