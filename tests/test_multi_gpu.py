"""nca_expr_multi / evaluate_many: several expressions over shared operands.

The results must equal the expressions evaluated one call after another
(bit for bit: the same tapes, the same compute dtypes). Where the views fit
the TMA-staged pass (the C2 shape: a transposed float32 operand, an int32
operand in the output's layout, 4-byte outputs) every output comes from one
launch; elsewhere (outputs that overlap an operand, 8-byte outputs, operands
that need no staging, no reductions) the calls run one after another."""
import numpy as np
import pytest

import ncarray_gb300 as nca
from ncarray_gb300 import _lib
from ncarray_gb300.dtype import DType, RedOp
from tests.helpers import SEED

pytestmark = pytest.mark.gpu


def _c2_like(rng, shape=(64, 32, 48, 8)):
    x = rng.normal(size=shape).astype(np.float32)
    v = rng.normal(size=shape[1]).astype(np.float32)
    k = rng.integers(-1000, 1001, (shape[3], shape[1], shape[2], shape[0])).astype(np.int32)
    return x, v, k


def _exprs(dx, dv, dk, b):
    with nca.lazy_mode():
        y = dx.permute(3, 1, 2, 0) * dv.reshape(1, b, 1, 1) + dk
        z = (dk * 3 + 7) % 11
        w = dk + 1
        u = dx.permute(3, 1, 2, 0) - dv.reshape(1, b, 1, 1)
    return y, z, w, u


def _separate(exprs, reds):
    y = exprs[0]
    oy = nca.NCDevArray(y.shape, y.dtype)
    r = y.evaluate(out=oy, reductions=reds) if reds else (y.evaluate(out=oy) or [])
    outs = [oy.to_host()]
    for e in exprs[1:]:
        o = nca.NCDevArray(e.shape, e.dtype)
        e.evaluate(out=o)
        outs.append(o.to_host())
    return outs, [a.to_host() for a in r]


def _fused(exprs, reds):
    outs = [nca.NCDevArray(e.shape, e.dtype) for e in exprs]
    n0 = _lib.lib().nca_launch_count()
    r = nca.evaluate_many(list(zip(exprs, outs)), reductions=reds)
    n1 = _lib.lib().nca_launch_count()
    return [o.to_host() for o in outs], [a.to_host() for a in r], n1 - n0


REDS = [(RedOp.MAX, 2), (RedOp.ARGMAX, 2)]


@pytest.mark.parametrize("n_extra", [1, 2, 3])
def test_c2_shape_one_launch(cuda, n_extra):
    rng = np.random.default_rng(SEED + 1300 + n_extra)
    x, v, k = _c2_like(rng)
    dx, dv, dk = (nca.NCDevArray.from_host(a) for a in (x, v, k))
    exprs = list(_exprs(dx, dv, dk, x.shape[1]))[: 1 + n_extra]
    want, want_r = _separate(exprs, REDS)
    got, got_r, launches = _fused(exprs, REDS)
    for g, w in zip(got, want):
        assert g.tobytes() == w.tobytes()
    for g, w in zip(got_r, want_r):
        assert g.tobytes() == w.tobytes()
    assert launches == 1
    # the int32 output against numpy (C's truncating remainder)
    assert np.array_equal(got[1], np.fmod(k * 3 + 7, 11))


def test_extra_over_the_staged_operand_and_scalars(cuda):
    """An extra tape that reads the transposed operand and has constants of
    its own (the scalar words follow the first tape's)."""
    rng = np.random.default_rng(SEED + 1310)
    x, v, k = _c2_like(rng, (32, 16, 64, 4))
    dx, dv, dk = (nca.NCDevArray.from_host(a) for a in (x, v, k))
    with nca.lazy_mode():
        y = dx.permute(3, 1, 2, 0) * dv.reshape(1, 16, 1, 1) + dk * 0.5
        z = dx.permute(3, 1, 2, 0) * 2.5 - 1.25
    want, want_r = _separate([y, z], [(RedOp.SUM, 2), (RedOp.MIN, 2)])
    got, got_r, launches = _fused([y, z], [(RedOp.SUM, 2), (RedOp.MIN, 2)])
    assert all(g.tobytes() == w.tobytes() for g, w in zip(got, want))
    assert all(g.tobytes() == w.tobytes() for g, w in zip(got_r, want_r))
    assert launches == 1


def test_fallbacks_match_separate_calls(cuda):
    rng = np.random.default_rng(SEED + 1320)
    x, v, k = _c2_like(rng)
    dx, dv, dk = (nca.NCDevArray.from_host(a) for a in (x, v, k))
    y, z, _, _ = _exprs(dx, dv, dk, x.shape[1])
    # an 8-byte extra output: no staged store for it, two launches
    with nca.lazy_mode():
        z64 = (dk * 3 + 7) % 11 + nca.NCDevArray.from_host(np.zeros(1, np.int64))
    want, want_r = _separate([y, z64], REDS)
    got, got_r, launches = _fused([y, z64], REDS)
    assert all(g.tobytes() == w.tobytes() for g, w in zip(got, want))
    assert all(g.tobytes() == w.tobytes() for g, w in zip(got_r, want_r))
    assert launches >= 2
    # no reductions: one call per expression
    want, _ = _separate([y, z], [])
    got, _, _ = _fused([y, z], [])
    assert all(g.tobytes() == w.tobytes() for g, w in zip(got, want))
    # contiguous operands (no staging): separate launches, same results
    a = rng.normal(size=(64, 96)).astype(np.float32)
    da = nca.NCDevArray.from_host(a)
    with nca.lazy_mode():
        e1 = da * 2.0
        e2 = da + 1.0
    want, want_r = _separate([e1, e2], [(RedOp.SUM, 0)])
    got, got_r, _ = _fused([e1, e2], [(RedOp.SUM, 0)])
    assert all(g.tobytes() == w.tobytes() for g, w in zip(got, want))
    assert all(g.tobytes() == w.tobytes() for g, w in zip(got_r, want_r))


def test_output_overlapping_an_operand_runs_in_order(cuda):
    """z written over k itself: the first expression must still read the
    original k (the calls run one after another)."""
    rng = np.random.default_rng(SEED + 1330)
    x, v, k = _c2_like(rng)
    dx, dv, dk = (nca.NCDevArray.from_host(a) for a in (x, v, k))
    y, z, _, _ = _exprs(dx, dv, dk, x.shape[1])
    oy = nca.NCDevArray(y.shape, y.dtype)
    mx, am = nca.evaluate_many([(y, oy), (z, dk)], reductions=REDS)
    xp = np.transpose(x, (3, 1, 2, 0))
    want_y = xp * v.reshape(1, -1, 1, 1) + k.astype(np.float32)
    assert oy.to_host().tobytes() == want_y.astype(np.float32).tobytes()
    assert np.array_equal(dk.to_host(), np.fmod(k * 3 + 7, 11))
    assert np.array_equal(mx.to_host(), want_y.max(axis=2))
    assert np.array_equal(am.to_host(), want_y.argmax(axis=2))


def test_shared_operand_given_twice(cuda):
    """The same array reached through two leaves of different expressions and
    a tape that loads one array twice: the operand list is merged."""
    rng = np.random.default_rng(SEED + 1340)
    x, v, k = _c2_like(rng)
    dx, dv = nca.NCDevArray.from_host(x), nca.NCDevArray.from_host(v)
    dk1 = nca.NCDevArray.from_host(k)
    with nca.lazy_mode():
        y = dx.permute(3, 1, 2, 0) * dv.reshape(1, x.shape[1], 1, 1) + dk1
        z = dk1 * dk1 - dk1
    want, want_r = _separate([y, z], REDS)
    got, got_r, launches = _fused([y, z], REDS)
    assert all(g.tobytes() == w.tobytes() for g, w in zip(got, want))
    assert all(g.tobytes() == w.tobytes() for g, w in zip(got_r, want_r))
    assert launches == 1


def test_idx_tape_falls_back(cuda):
    """An extra tape reading the element index (IDX) is not fused: the calls
    run in order with the same results."""
    rng = np.random.default_rng(SEED + 1350)
    x, v, k = _c2_like(rng)
    dx, dv, dk = (nca.NCDevArray.from_host(a) for a in (x, v, k))
    y, _, _, _ = _exprs(dx, dv, dk, x.shape[1])
    with nca.lazy_mode():
        zi = dk + nca.iota(dk, DType.int32)
    want, want_r = _separate([y, zi], REDS)
    got, got_r, launches = _fused([y, zi], REDS)
    assert all(g.tobytes() == w.tobytes() for g, w in zip(got, want))
    assert all(g.tobytes() == w.tobytes() for g, w in zip(got_r, want_r))
    assert launches >= 2
