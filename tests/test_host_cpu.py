"""Host logic without a GPU: dtype promotion (the reference's rules), scalar
typing, and the multi-rank aggregation of bench.py on world_size-2 gloo."""
import os
import socket
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from ncarray_gb300.dtype import DType, OpCode, compute_dtype, promote, result_dtype, scalar_dtype  # noqa: E402


def test_promotion_follows_reference_rules():
    # work dtype = the numerically larger DType (interface.hh:91-100)
    assert promote(DType.float32, DType.int32) == DType.float32
    assert promote(DType.int32, DType.float32) == DType.float32
    assert promote(DType.uint8, DType.int16) == DType.int16
    assert promote(DType.float32, DType.float64) == DType.float64
    # ADD/MUL -> sum_type: <= 16-bit ints and bool widen to 64-bit (op_traits.hh:72-76)
    assert result_dtype(OpCode.ADD, DType.int16) == DType.int64
    assert result_dtype(OpCode.ADD, DType.uint8) == DType.uint64
    assert result_dtype(OpCode.ADD, DType.int32) == DType.int32
    assert result_dtype(OpCode.ADD, DType.float32) == DType.float32
    # DIV -> truediv_type = double for every real type
    assert result_dtype(OpCode.DIV, DType.int32) == DType.float64
    assert result_dtype(OpCode.DIV, DType.float32) == DType.float64
    # MOD keeps the type; comparisons give bool
    assert result_dtype(OpCode.MOD, DType.int32) == DType.int32
    assert result_dtype(OpCode.GT, DType.float64) == DType.bool
    # bool results compute in the work dtype, others in the result dtype
    assert compute_dtype(DType.bool, DType.float32) == DType.float32
    assert compute_dtype(DType.float64, DType.int32) == DType.float64


def test_c2_expression_dtypes():
    # y = x_f32 * v_f32 + k_i32 -> float32; (k*3+7)%11 stays int32
    w = promote(promote(DType.float32, DType.float32), DType.int32)
    assert w == DType.float32 and result_dtype(OpCode.ADD, w) == DType.float32
    assert scalar_dtype(3) in (DType.uint8, DType.int8, DType.int16, DType.int32, DType.int64)
    wi = promote(DType.int32, scalar_dtype(3))
    assert wi == DType.int32
    assert result_dtype(OpCode.MOD, result_dtype(OpCode.ADD, result_dtype(OpCode.MUL, wi))) == DType.int32


def test_scalar_typing_mirrors_binding():
    # Python ints take the smallest unsigned type that holds them, then signed;
    # floats are float32 (the pybind variant order of the reference binding)
    assert scalar_dtype(7) == DType.uint8
    assert scalar_dtype(300) == DType.uint16
    assert scalar_dtype(-1) == DType.int8
    assert scalar_dtype(0.5) == DType.float32


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, ms, out):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    value, ms_step = bench.job_throughput(ms[rank], 10, world, 1e9,
                                          lambda v: bench.all_reduce_max(dist, torch, v, "cpu"))
    out.put((rank, value, ms_step))
    dist.barrier()
    dist.destroy_process_group()


def test_multirank_throughput_takes_slowest_rank_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ms = [10.0, 20.0]
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, ms, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # slowest rank: 20 ms for 10 steps -> 2 ms/step; 2 ranks x 1 GB per step
    for _, value, ms_step in res:
        assert ms_step == pytest.approx(2.0)
        assert value == pytest.approx(2 * 1e9 / 2e-3 / 1e9)


def test_reference_arm_other_ranks_print_nothing(capsys):
    import bench

    class A:
        steps, warmup, gpus = 1, 3, 2
    bench.run_reference(A(), rank=1)
    assert capsys.readouterr().out == ""


def test_evaluate_many_merges_operands(monkeypatch):
    """evaluate_many on the host: equal operand views of the expressions
    become one operand, every tape's loads are renumbered into the merged
    list, and one nca_expr_multi call carries all tapes and outputs (the C ABI
    is replaced by a recorder: no GPU)."""
    torch = pytest.importorskip("torch")
    import ncarray_gb300 as nca
    import ncarray_gb300.array as arr_mod
    from ncarray_gb300 import _lib
    from ncarray_gb300.dtype import ITEMSIZE, RedOp

    def mk(shape, dt):
        n = max(int(np.prod(shape)) * ITEMSIZE[dt], 1)
        return nca.NCDevArray(shape, dt, _buf=torch.empty(n, dtype=torch.uint8))

    x, v, k = mk((4, 2, 3, 8), DType.float32), mk((2,), DType.float32), mk((8, 2, 3, 4), DType.int32)
    with nca.lazy_mode():
        y = x.permute(3, 1, 2, 0) * v.reshape(1, 2, 1, 1) + k
        z = (k * 3 + 7) % 11
        w = k * k - k
    outs = [mk(y.shape, y.dtype), mk(z.shape, z.dtype), mk(w.shape, w.dtype)]
    mx = mk((8, 2, 4), DType.float32)
    calls = []
    monkeypatch.setattr(_lib, "call", lambda name, *a: calls.append((name, a)) or 0)
    monkeypatch.setattr(arr_mod, "current_stream", lambda: 0)
    res = nca.evaluate_many([(y, outs[0]), (z, outs[1]), (w, outs[2])], reductions=[(RedOp.MAX, 2)], red_out=[mx])
    assert res == [mx]
    assert [c[0] for c in calls] == ["nca_expr_multi"]
    tarr, nt, ops, nops, oarr, rarr, nred, stream = calls[0][1]
    assert (nt, nops, nred) == (3, 3, 1)
    assert [ops[i].data for i in range(3)] == [x.ptr, v.ptr, k.ptr]
    assert [oarr[i].data for i in range(3)] == [o.ptr for o in outs]

    def loads(t):
        return sorted({int(t.instrs[i]) & 0xFFFFFF for i in range(t.n_instrs) if int(t.instrs[i]) >> 24 == OpCode.LOAD_NCARR})

    assert loads(tarr[0]) == [0, 1, 2]
    assert loads(tarr[1]) == [2] and loads(tarr[2]) == [2]
    assert rarr[0].op == int(RedOp.MAX) and rarr[0].axes_mask == 1 << 2
    # shapes must agree
    with pytest.raises(ValueError):
        nca.evaluate_many([(y, outs[0]), (z, mk((8, 2, 3, 5), DType.int32))])
