"""Benchmark of the GB300 device path (one JSON line on rank 0).

Headline workload (strided/broadcast fusion, float32 + int32):
  x  float32 (64,256,256,8) ~ N(0,1), viewed with axes permuted (3,1,2,0)
  v  float32 (256,) ~ N(0,1), broadcast as v[None,:,None,None]
  k  int32 (8,256,256,64) ~ U{-1000..1000}
  one step = y = x_perm * v + k (stored) with y.max(axis 2) and y.argmax(axis 2)
             in the same pass, and z = (k*3 + 7) % 11 (on a second stream).
Inputs are resident in HBM when the timed region starts; the working set
(~640 MB) is larger than L2, so no flush is needed between steps.

`value` = algorithmic bytes of a step / device time of a step (GB/s, whole job);
          the step's C-ABI calls are captured once into a CUDA graph and the
          timed region replays it K times.
`e2e`   = the same bytes through the C-ABI calls with pinned HOST buffers:
          each step copies x, v, k in and y, max, argmax, z out.
`--impl reference` times the CPU restatement of the reference path (the
oracle port) on a bounded sample of the same workload on the host cores.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "HBM GB/s & % of GB300 peak per op; batched-vs-plain speedup at ≤1e-6 rel err"
SEED = 20261203
C2_SHAPE = (64, 256, 256, 8)  # x as stored; the view is (8,256,256,64)


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---- clocks ---------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "50",
                 "-i", str(self.index)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---- workload ---------------------------------------------------------------------
def c2_host(scale_l0: int = 8):
    """Seeded host inputs; scale_l0 < 8 takes the leading view slices (a sample)."""
    rng = np.random.default_rng(SEED + 1)
    x = rng.standard_normal(C2_SHAPE, dtype=np.float32)
    v = rng.standard_normal(256, dtype=np.float32)
    k = rng.integers(-1000, 1001, (8, 256, 256, 64), dtype=np.int32)
    return x, v, k


def c2_bytes(n: int) -> dict:
    """Algorithmic bytes over n = elements of the view: per kernel, and for
    the whole step the bytes it must move once -- read x and k, write y and z
    (4 bytes each), read v, write the axis-2 max (4 B) and argmax (8 B) per
    kept position. k feeds both expressions but counts once."""
    fused = 12 * n + (4 + 8) * (n // 256) + 1024
    intexpr = 8 * n
    step = 16 * n + (4 + 8) * (n // 256) + 1024
    return {"fused": fused, "int": intexpr, "step": step}


# NCA_C2_STEP=forked runs the step as two calls (the fused expression and the
# int32 expression on two forked streams) instead of one nca_expr_multi pass
C2_FORKED = os.environ.get("NCA_C2_STEP", "") == "forked"


class C2Step:
    """One step through the public API (lazy tape -> fused kernel) on device arrays."""

    def __init__(self, nca, dx, dv, dk):
        self.nca = nca
        with nca.lazy_mode():
            self.y_expr = dx.permute(3, 1, 2, 0) * dv.reshape(1, 256, 1, 1) + dk
            self.z_expr = (dk * 3 + 7) % 11
        self.y = nca.NCDevArray(self.y_expr.shape, self.y_expr.dtype)
        self.z = nca.NCDevArray(self.z_expr.shape, self.z_expr.dtype)
        self.red = [(nca.RedOp.MAX, 2), (nca.RedOp.ARGMAX, 2)]
        kept = (self.y.shape[0], self.y.shape[1], self.y.shape[3])
        self.mx = nca.NCDevArray(kept, nca.DType.float32)
        self.am = nca.NCDevArray(kept, nca.DType.int64)

    def fused(self):
        self.y_expr.evaluate(out=self.y, reductions=self.red, red_out=[self.mx, self.am])

    def intexpr(self):
        self.z_expr.evaluate(out=self.z)

    def multi(self):
        """Both expressions in one pass (nca_expr_multi): x and k read once."""
        self.nca.evaluate_many([(self.y_expr, self.y), (self.z_expr, self.z)], reductions=self.red,
                               red_out=[self.mx, self.am])

    def __call__(self):
        if C2_FORKED:
            self.fused()
            self.intexpr()
        else:
            self.multi()

    def forked(self, torch, side):
        """The step with the two expressions on two streams (they share only the
        input k): each kernel fills the other's start and tail."""
        cur = torch.cuda.current_stream()
        side.wait_stream(cur)
        self.fused()
        with torch.cuda.stream(side):
            self.intexpr()
        cur.wait_stream(side)


def make_graph(torch, fn):
    """Captures fn() (a sequence of C-ABI calls on the current stream) into a
    CUDA graph; the kernels are compiled beforehand by eager calls."""
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        fn()
        fn()
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        fn()
    torch.cuda.synchronize()
    return g


def time_events(torch, fn, reps: int) -> float:
    """Average ms of fn() over reps, CUDA events on the current stream."""
    s = torch.cuda.current_stream()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(s)
    for _ in range(reps):
        fn()
    b.record(s)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def cpu_baseline_c2(nthreads: int | None = None, sample_l0: int = 1):
    """The oracle port (C restatement of the reference's VM and host
    reductions) on the first `sample_l0` of the 8 view slices along axis 0."""
    import oracle
    x, v, k = c2_host()
    xp = x.transpose(3, 1, 2, 0)[:sample_l0]
    ks = np.ascontiguousarray(k[:sample_l0])
    vb = v.reshape(1, 256, 1, 1)
    n = xp.size
    if nthreads:
        os.environ["OMP_NUM_THREADS"] = str(nthreads)
    I = lambda op, i=0: (op << 24) | i  # noqa: E731
    t0 = time.perf_counter()
    y = oracle.expr_eval([I(2, 0), I(2, 1), I(16), I(2, 2), I(14)], [], 10, [(xp, 10), (vb, 10), (ks, 8)],
                         xp.shape, 10)
    oracle.reduce(y, 10, 2, [2])
    oracle.reduce(y, 10, 4, [2])
    oracle.expr_eval([I(2, 0), I(4, 0), I(16), I(4, 1), I(14), I(4, 2), I(18)], [(2, 3), (2, 7), (2, 11)], 8,
                     [(ks, 8)], ks.shape, 8)
    dt = time.perf_counter() - t0
    gbs = c2_bytes(n)["step"] / dt / 1e9
    return gbs, n, dt


# ---- per-op measurements of the other workloads -----------------------------------
def flush_l2(torch, buf):
    """Evicts the op's data from L2: a 512 MiB write (> L2), then a 256 MiB read,
    so that the flush's own dirty lines are written back here and not during the
    timed op."""
    buf.fill_(1)
    buf[: buf.numel() // 2].view(torch.float32).sum()


def timed_flushed(torch, fn, reps, flush_buf):
    """Average device ms of fn() with an L2 flush before every rep (flush not timed)."""
    s = torch.cuda.current_stream()
    total = 0.0
    for _ in range(reps):
        flush_l2(torch, flush_buf)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        fn()
        b.record(s)
        torch.cuda.synchronize()
        total += a.elapsed_time(b)
    return total / reps


def op_entry(bytes_, ms, peak, elements=None, **extra):
    gbs = bytes_ / (ms * 1e-3) / 1e9
    d = {"GB/s": round(gbs, 1), "frac_of_measured": round(gbs / peak, 4), "ms": round(ms, 4)}
    if elements:
        d["Gelements/s"] = round(elements / (ms * 1e-3) / 1e9, 3)
    d.update(extra)
    return d


def cpu_entry(fn, bytes_, elements, sample, threads, reps=3):
    """The oracle port timed on the host cores: best of `reps` wall-clock runs
    of fn() over a bounded sample of the workload (`bytes_` algorithmic bytes,
    `elements` units of work in that sample). A reported baseline, not a target."""
    best = float("inf")
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        best = min(best, time.perf_counter() - t0)
    return {"GB/s": round(bytes_ / best / 1e9, 3), "Gelements/s": round(elements / best / 1e9, 4),
            "s": round(best, 4), "cores": threads, "kind": "port", "sample": sample}


def _orc_tape(e):
    """(instrs, scalars, compute dtype) of a DevExpr for the oracle."""
    from ncarray_gb300.dtype import compute_dtype
    return list(e.instrs), [(int(d), v) for d, v in e.scalars], int(compute_dtype(e.expr_dtype, e.work))


def measure_c1(torch, nca, peak, flush_buf, reps=20):
    """C1: out = a*b + sqrt(abs(c)) - 0.5*a on float64 (128,128,128), with the
    axis-0 sum and max in the same pass, then the full sum and max."""
    rng = np.random.default_rng(SEED + 0)
    a, b, c = (rng.uniform(-1, 1, (128, 128, 128)) for _ in range(3))
    da, db, dc = (nca.NCDevArray.from_host(v) for v in (a, b, c))
    with nca.lazy_mode():
        e = da * db + nca.sqrt(abs(dc)) - 0.5 * da
    out = nca.NCDevArray(e.shape, e.dtype)
    res = {}

    def step():
        s0, m0 = e.evaluate(out=out, reductions=[(nca.RedOp.SUM, 0), (nca.RedOp.MAX, 0)])
        res["s"] = s0._expr().evaluate(reductions=[(nca.RedOp.SUM, None)])[0]
        res["m"] = m0._expr().evaluate(reductions=[(nca.RedOp.MAX, None)])[0]

    for _ in range(3):
        step()
    # device time of the step: replays of a graph of its C-ABI calls (the eager
    # calls' host side, about 0.1 ms for three evaluates, is reported beside it)
    ms_eager = timed_flushed(torch, step, reps, flush_buf)
    g = make_graph(torch, step)
    g.replay()
    ms = timed_flushed(torch, g.replay, reps, flush_buf)
    n = a.size
    ref = a * b + np.sqrt(np.abs(c)) - np.float32(0.5) * a
    exact = bool(np.array_equal(out.to_host(), ref))
    rel = abs(float(res["s"].to_host()) - float(np.sum(ref))) / abs(float(np.sum(ref)))
    import oracle
    ins, sc, cdt = _orc_tape(e)
    ops = [(a, 11), (b, 11), (c, 11)]

    def cpu_step():
        y = oracle.expr_eval(ins, sc, cdt, ops, a.shape, 11)
        oracle.reduce(y, 11, 0, [0])
        oracle.reduce(y, 11, 2, [0])
        oracle.reduce(y, 11, 0)
        oracle.reduce(y, 11, 2)

    cpu = cpu_entry(cpu_step, 32 * n + 2 * 8 * 128 * 128, n, "the whole step (128^3)", omp_threads())
    return op_entry(32 * n + 2 * 8 * 128 * 128, ms, peak, elements=n, cpu_baseline=cpu,
                    bound_note="float64 ALU (GB300 FP64 rate) rather than HBM",
                    eager_ms=round(ms_eager, 4), launch="CUDA-graph replay of the step's three evaluate calls",
                    out_bit_exact=exact, sum_rel_err_vs_f64=rel, max_exact=bool(float(res["m"].to_host()) == ref.max()),
                    l2="flushed before every rep (512 MiB write, then 256 MiB read: no dirty lines left)")


def gst_used(w):
    """Offsets (flat 3x3x3 indices) of the non-zero weights."""
    return [t for t in range(27) if float(w.reshape(27)[t]) != 0.0]


def general_laplacian(nca, w, scale=0.1):
    """u + scale * sum_t w_t u[o_t] as ncarray's Stencil<3> over the shifted
    views of a zero-padded source (offsets 0..2 per axis, one per non-zero
    weight), float32."""
    from ncarray_gb300.stencil import Stencil
    wl = [float(v) for v in w.reshape(27)]
    used = gst_used(w)
    centre = used.index(13)

    def lap(views):
        acc = None
        for k, t in enumerate(used):
            term = nca.DevExpr.leaf(views[k]) * np.float32(wl[t])
            acc = term if acc is None else acc + term
        return nca.DevExpr.leaf(views[centre]) + acc * np.float32(scale)

    offs = [(t // 9, (t // 3) % 3, t % 3) for t in used]
    return Stencil.create(offs, lap, nca.DType.float32, is_pointer_axis=[0, 0, 0])


def measure_c3(torch, nca, peak, iters=10):
    """C3: 7- and 27-point Laplacian, 512^3 float32, zero halo, 10 Jacobi steps
    u <- u + 0.1 L(u); error vs the float64 run of the same steps."""
    from ncarray_gb300.stencil import Stencil3D, laplacian7, laplacian27, device_status
    g = torch.Generator(device="cuda").manual_seed(SEED + 2)
    n = 512 ** 3
    u64 = torch.randn((512, 512, 512), generator=g, device="cuda", dtype=torch.float64)
    out = {}
    for name, w in (("7pt", laplacian7()), ("27pt", laplacian27())):
        st = Stencil3D(w, 0.1)
        a = nca.NCDevArray((512, 512, 512), nca.DType.float32)
        b = nca.NCDevArray((512, 512, 512), nca.DType.float32)
        src32 = u64.float().contiguous()
        a._buf.view(torch.float32).view(512, 512, 512).copy_(src32)
        st.iterate(a, b, 2)
        a._buf.view(torch.float32).view(512, 512, 512).copy_(src32)
        s = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        res = st.iterate(a, b, iters)
        e1.record(s)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / iters
        status = device_status()
        # float64 run of the same steps on the device
        a64 = nca.NCDevArray((512, 512, 512), nca.DType.float64)
        b64 = nca.NCDevArray((512, 512, 512), nca.DType.float64)
        a64._buf.view(torch.float64).view(512, 512, 512).copy_(src32.double())
        r64 = st.iterate(a64, b64, iters)
        t32 = res._buf.view(torch.float32).double()
        t64 = r64._buf.view(torch.float64)
        rel_l2 = float(torch.linalg.vector_norm(t32 - t64) / torch.linalg.vector_norm(t64))
        max_rel = float((t32 - t64).abs().max() / t64.abs().max())
        import oracle
        sample = src32[:64].cpu().numpy()
        cpu = cpu_entry(lambda: oracle.stencil3d_f64(sample, w.reshape(27), 0.1, 1), 8 * sample.size, sample.size,
                        "one float64 iteration on 64 of the 512 z-planes (bytes counted as float32 in/out)",
                        omp_threads(), reps=2)
        out[name] = op_entry(8 * n, ms, peak, elements=n, per="iteration", rel_l2_err_vs_f64=rel_l2,
                             max_err_rel_to_max=max_rel, status=status, cpu_baseline=cpu)
        # the same iteration through the general stencil (Stencil.create: the
        # shifted views of a zero-padded (514, 514, 514) source, one fused
        # expression per point), against the TMA kernel's first iteration;
        # timed in the tiled form (the default) and in the view form
        gst = general_laplacian(nca, w)
        pad = nca.NCDevArray((514, 514, 514), nca.DType.float32).fill(0.0)
        pad._buf.view(torch.float32).view(514, 514, 514)[1:513, 1:513, 1:513].copy_(src32)
        dst = nca.NCDevArray((512, 512, 512), nca.DType.float32)
        gms = {}
        for form, mode in (("view", "0"), ("tiled", "1")):
            os.environ["NCA_STENCIL_TILE"] = mode
            gst.apply(pad, dst)
            e0.record(s)
            for _ in range(5):
                gst.apply(pad, dst)
            e1.record(s)
            torch.cuda.synchronize()
            gms[form] = e0.elapsed_time(e1) / 5
        os.environ.pop("NCA_STENCIL_TILE", None)
        one = nca.NCDevArray((512, 512, 512), nca.DType.float32)
        a1 = nca.NCDevArray((512, 512, 512), nca.DType.float32)
        a1._buf.view(torch.float32).view(512, 512, 512).copy_(src32)
        r1 = st.iterate(a1, one, 1)
        tg = dst._buf.view(torch.float32).double()
        tt = r1._buf.view(torch.float32).double()
        gbytes = 4 * (514 ** 3 + n)
        out["general_" + name] = op_entry(gbytes, gms["tiled"], peak, elements=n, per="iteration",
                                          offsets=len(gst_used(w)),
                                          kernel="nca_stencil_tile (shared-memory planes, register window along z)",
                                          view_form={"ms": round(gms["view"], 4), "GB/s": round(gbytes / gms["view"] / 1e6, 1),
                                                     "kernel": "nca_nd (one strided view per offset)"},
                                          max_diff_rel_to_max_vs_tma=float((tg - tt).abs().max() / tt.abs().max()))
        del a, b, a64, b64, t32, t64, pad, dst, one, a1, tg, tt
    return out


def c4_points(torch, nca, P=1 << 27):
    """P = 2^27 (x, y) float32 points from a mixture of 8 Gaussians (centres
    uniform in [0,1)^2, sigma 0.01-0.1, Dirichlet(0.5) weights) and lognormal
    weights, generated on the device from a seed."""
    rng = np.random.default_rng(SEED + 3)
    centres = rng.uniform(0, 1, (8, 2))
    sigma = rng.uniform(0.01, 0.1, 8)
    mix = rng.dirichlet(np.full(8, 0.5))
    g = torch.Generator(device="cuda").manual_seed(SEED + 3)
    comp = torch.multinomial(torch.tensor(mix, device="cuda", dtype=torch.float32), P, replacement=True, generator=g)
    cen = torch.tensor(centres, device="cuda", dtype=torch.float32)[comp]
    sig = torch.tensor(sigma, device="cuda", dtype=torch.float32)[comp]
    pts = cen + torch.randn((P, 2), generator=g, device="cuda") * sig[:, None]
    wts = torch.exp(torch.randn(P, generator=g, device="cuda"))
    x = nca.NCDevArray((P,), nca.DType.float32)
    y = nca.NCDevArray((P,), nca.DType.float32)
    w = nca.NCDevArray((P,), nca.DType.float32)
    x._buf.view(torch.float32).copy_(pts[:, 0].contiguous())
    y._buf.view(torch.float32).copy_(pts[:, 1].contiguous())
    w._buf.view(torch.float32).copy_(wts)
    del comp, cen, sig, pts, wts
    return x, y, w


def measure_c4(torch, nca, peak, reps=5):
    """C4: 2^27 (x, y) float32 points from 8 Gaussians into 1024 x 1024 bins on
    [0,1)^2; uint64 counts (exact) and float32 weighted sums (float32
    compensated per tile, float64 across tiles)."""
    from ncarray_gb300.hist import hist2d_into
    P = 1 << 27
    x, y, w = c4_points(torch, nca)
    counts = nca.NCDevArray((1024, 1024), nca.DType.uint64)
    wsum = nca.NCDevArray((1024, 1024), nca.DType.float32)

    def run(weighted):
        counts.fill(0)
        if weighted:
            wsum.fill(0.0)
        hist2d_into(x, y, counts, (0.0, 1.0), (0.0, 1.0), w if weighted else None, wsum if weighted else None)

    out = {}
    for weighted in (False, True):
        run(weighted)
        s = torch.cuda.current_stream()
        tot = 0.0
        for _ in range(reps):
            counts.fill(0)
            if weighted:
                wsum.fill(0.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            hist2d_into(x, y, counts, (0.0, 1.0), (0.0, 1.0), w if weighted else None, wsum if weighted else None)
            e1.record(s)
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1)
        ms = tot / reps
        byts = (12 * P + 16 * 1024 * 1024) if weighted else (8 * P + 8 * 1024 * 1024)
        import oracle
        ns = 1 << 23
        xs = x._buf[: 4 * ns].cpu().numpy().view(np.float32)
        ys = y._buf[: 4 * ns].cpu().numpy().view(np.float32)
        ws = w._buf[: 4 * ns].cpu().numpy().view(np.float32) if weighted else None
        cpu = cpu_entry(lambda: oracle.hist2d(xs, ys, ws, 1024, 1024, 0.0, 1.0, 0.0, 1.0),
                        (12 if weighted else 8) * ns + (16 if weighted else 8) * 1024 * 1024, ns,
                        "the first 2^23 of the 2^27 points, one thread", 1, reps=2)
        out["weighted" if weighted else "counts"] = op_entry(byts, ms, peak, elements=P, points=P, cpu_baseline=cpu)
    total = int(counts._buf.view(torch.int64).sum().item())
    out["counts_total"] = total
    return out


def measure_binning(torch, nca, peak, flush_buf, reps=20):
    """Pixel binning, the reference's own benchmark (examples/benchmark_binning.cu):
    a (32, 512, 1024) float32 image binned 2 x 2 x 2 into (16, 256, 512) as the
    fused sum of 8 strided views times 1/8, on contiguous data and on a
    32-panel pointer-axis view, and as reshape(16,2,256,2,512,2).sum((1,3,5)).
    64 MB read + 8 MB written per call; L2 flushed before every call (the image
    fits in L2); eager calls and CUDA-graph replays."""
    shape, bins = (32, 512, 1024), (2, 2, 2)
    g = torch.Generator(device="cuda").manual_seed(SEED + 7)
    data = nca.NCDevArray(shape, nca.DType.float32)
    data._buf.view(torch.float32).copy_(torch.rand(32 * 512 * 1024, generator=g, device="cuda"))
    panels = [data[i].copy() for i in range(32)]
    P = nca.NCDevArray.from_panels(panels)

    def fused(src):
        e = None
        with nca.lazy_mode():
            for a in range(2):
                for b in range(2):
                    for c in range(2):
                        v = src[a::2, b::2, c::2]
                        e = v if e is None else e + v
            return e * 0.125

    e_c, e_p = fused(data), fused(P)
    out = nca.NCDevArray((16, 256, 512), nca.DType.float32)
    six = data.reshape(16, 2, 256, 2, 512, 2)._expr()
    bytes_per = 32 * 512 * 1024 * 4 + 16 * 256 * 512 * 4
    forms = {"fused_views": lambda: e_c.evaluate(out=out),
             "fused_views_panels": lambda: e_p.evaluate(out=out),
             "reshape_sum": lambda: six.evaluate(reductions=[(nca.RedOp.SUM, (1, 3, 5))], red_out=[out])}
    s = torch.cuda.current_stream()
    res = {}
    for name, fn in forms.items():
        fn()
        fn()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            fn()
        for mode, call in (("eager", fn), ("graph", graph.replay)):
            call()
            tot = 0.0
            for _ in range(reps):
                flush_l2(torch, flush_buf)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(s)
                call()
                e1.record(s)
                torch.cuda.synchronize()
                tot += e0.elapsed_time(e1)
            ms = tot / reps
            gbs = bytes_per / (ms * 1e-3) / 1e9
            res[f"{name}_{mode}"] = {"GB/s": round(gbs, 1), "frac_of_measured": round(gbs / peak, 4),
                                     "us": round(ms * 1e3, 2)}
    # all forms agree (sums of eight values: the reduction may round differently)
    e_c.evaluate(out=out)
    a = out.to_host().copy()
    e_p.evaluate(out=out)
    b = out.to_host().copy()
    six.evaluate(reductions=[(nca.RedOp.SUM, (1, 3, 5))], red_out=[out])
    c = out.to_host() * np.float32(0.125)
    import oracle
    img = data.to_host()
    ins, sc, cdt = _orc_tape(e_c)
    views = [(img[i::2, j::2, k::2], 10) for i in range(2) for j in range(2) for k in range(2)]
    res["cpu_baseline"] = cpu_entry(lambda: oracle.expr_eval(ins, sc, cdt, views, (16, 256, 512), 10), bytes_per,
                                    16 * 256 * 512, "the whole binning (fused sum of 8 strided views)", omp_threads())
    res["Gelements/s_fused_views_graph"] = round(16 * 256 * 512 / (res["fused_views_graph"]["us"] * 1e-6) / 1e9, 3)
    res["panels_bit_exact_vs_contiguous"] = bool(np.array_equal(a, b))
    res["reshape_sum_max_rel_diff"] = float(np.max(np.abs(c - a) / np.maximum(np.abs(a), 1e-30)))
    res["l2"] = "flushed before every call (512 MiB write, then 256 MiB read: no dirty lines left)"
    return res


def measure_reductions(torch, nca, peak, reps=50):
    """Plain axis and global reductions of 256 MB float32 arrays (inputs larger
    than L2; CUDA-graph replays of one evaluate call each): the reduction
    kinds on their own, checked against numpy on the host."""
    cases = [
        ("global_sum", (64 << 20,), [(nca.RedOp.SUM, None)]),
        ("global_max", (64 << 20,), [(nca.RedOp.MAX, None)]),
        ("sum_last_axis_4096x16384", (4096, 16384), [(nca.RedOp.SUM, 1)]),
        ("sum_last_axis_1Mx64", (1 << 20, 64), [(nca.RedOp.SUM, 1)]),
        ("sum_axis0_4096x16384", (4096, 16384), [(nca.RedOp.SUM, 0)]),
        ("max_axis1_256x256x1024", (256, 256, 1024), [(nca.RedOp.MAX, 1)]),
        ("argmax_last_axis_4096x16384", (4096, 16384), [(nca.RedOp.ARGMAX, 1)]),
    ]
    res = {}
    gen = torch.Generator(device="cuda").manual_seed(SEED + 9)
    for name, shape, red in cases:
        x = torch.randn(int(np.prod(shape)), device="cuda", dtype=torch.float32, generator=gen)
        d = nca.NCDevArray(shape, nca.DType.float32, _buf=x.view(torch.uint8))
        e = d._expr()
        outs = e.evaluate(reductions=red)
        g = make_graph(torch, lambda: e.evaluate(reductions=red))
        for _ in range(3):
            g.replay()
        ms = time_events(torch, g.replay, reps)
        nbytes = x.numel() * 4
        op, axes = red[0]
        xh = x.view(shape).cpu().numpy()
        got = outs[0].to_host()
        if op == nca.RedOp.SUM:
            want = xh.astype(np.float64).sum(axis=axes)
            ok = bool(np.all(np.abs(got - want) <= 1e-6 * np.abs(xh).astype(np.float64).sum(axis=axes) + 1e-30))
        elif op == nca.RedOp.MAX:
            ok = bool(np.array_equal(got, xh.max(axis=axes)))
        else:
            ok = bool(np.array_equal(got, xh.argmax(axis=axes)))
        res[name] = {"GB/s": round(nbytes / ms / 1e6, 1), "frac_of_measured": round(nbytes / ms / 1e6 / peak, 4),
                     "us": round(ms * 1e3, 2), "Gelements/s": round(x.numel() / ms / 1e6, 3), "matches_numpy": ok}
        if name in ("global_sum", "sum_axis0_4096x16384", "argmax_last_axis_4096x16384"):
            import oracle
            part = xh.reshape(-1)[: 1 << 24].reshape((-1,) + tuple(shape[1:])) if len(shape) > 1 else \
                xh.reshape(-1)[: 1 << 24]
            ax = None if axes is None else [axes]
            res[name]["cpu_baseline"] = cpu_entry(lambda: oracle.reduce(part, 10, int(op), ax), part.nbytes,
                                                  part.size, "the first 2^24 elements, one thread (the "
                                                  "reference's host reductions are single-threaded)", 1, reps=2)
        del x, d, e, g, outs
        torch.cuda.empty_cache()
    res["l2"] = "inputs 256 MB > L2; no flush"
    return res


def c5_arrays(torch, nca, n_arrays):
    """n_arrays 1-D device arrays with lengths log-uniform in [64, 2^22],
    alternately float32 and bfloat16, x = exp(N(0, 2)) with random signs,
    generated on the device from a seed (views into two large buffers)."""
    rng = np.random.default_rng(SEED + 4)
    lens = np.round(np.exp(rng.uniform(np.log(64), np.log(2 ** 22), n_arrays))).astype(np.int64)
    is16 = np.arange(n_arrays) % 2 == 1
    g = torch.Generator(device="cuda").manual_seed(SEED + 4)
    tot32, tot16 = int(lens[~is16].sum()), int(lens[is16].sum())
    buf32 = torch.empty(tot32, device="cuda", dtype=torch.float32)
    buf16 = torch.empty(tot16, device="cuda", dtype=torch.bfloat16)
    for buf, tot in ((buf32, tot32), (buf16, tot16)):
        step = 1 << 28
        for o in range(0, tot, step):
            m = min(step, tot - o)
            v = torch.exp(torch.randn(m, generator=g, device="cuda") * 2.0)
            v *= torch.where(torch.rand(m, generator=g, device="cuda") < 0.5, -1.0, 1.0)
            buf[o:o + m].copy_(v)
            del v
    arrays, o32, o16 = [], 0, 0
    b32 = buf32.view(torch.uint8)
    b16 = buf16.view(torch.uint8)
    for i, L in enumerate(lens):
        L = int(L)
        if is16[i]:
            arrays.append(nca.NCDevArray((L,), nca.DType.bfloat16, _buf=b16, _offset=2 * o16))
            o16 += L
        else:
            arrays.append(nca.NCDevArray((L,), nca.DType.float32, _buf=b32, _offset=4 * o32))
            o32 += L
    return rng, lens, arrays, tot32, tot16


def measure_c5(torch, nca, peak, n_arrays=20000):
    """C5: 20,000 1-D arrays, lengths log-uniform in [64, 2^22], half float32 and
    half bfloat16, x = s * exp(N(0, 2)) with random signs; per array sum, mean,
    max and sum(x*x - x): one persistent graph-replayed launch vs the plain
    per-array per-op float64 launches."""
    import oracle
    from ncarray_gb300.batch import Batch
    rng, lens, arrays, tot32, tot16 = c5_arrays(torch, nca, n_arrays)
    nbytes = 4 * tot32 + 2 * tot16
    B = Batch(arrays)
    sched = B.autotune()
    B.run(graph=True)
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()

    def timeit(fn, reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(reps):
            fn()
        e1.record(s)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    ms_b = timeit(lambda: B.run(graph=True), 5)
    got = B.run(graph=True).to_host().copy()
    ms_p = timeit(B.run_plain, 1)
    plain = B.results.to_host().copy()
    # accuracy vs float64 on a sample of arrays (copied to the host)
    pick = rng.choice(n_arrays, size=min(400, n_arrays), replace=False)
    host, dts = [], []
    for i in pick:
        a = arrays[i]
        raw = a._buf[a._offset: a._offset + a.nbytes].cpu().numpy()
        host.append(raw.view(np.float32) if a.dtype == nca.DType.float32 else raw.view(np.uint16))
        dts.append(10 if a.dtype == nca.DType.float32 else 22)
    t0 = time.perf_counter()
    ref = oracle.batch_reduce(host, dts, nthreads=omp_threads())
    cpu_s = time.perf_counter() - t0
    sbytes = sum(h.nbytes for h in host)
    selems = sum(h.size for h in host)
    cpu = {"GB/s": round(sbytes / cpu_s / 1e9, 3), "Gelements/s": round(selems / cpu_s / 1e9, 4), "s": round(cpu_s, 4),
           "cores": omp_threads(), "kind": "port", "sample": f"{len(pick)} of the {n_arrays} arrays, four results each"}
    g_ = got[pick]
    p_ = plain[pick]
    rel = lambda a_, b_: float(np.max(np.abs(a_ - b_) / np.maximum(np.abs(b_), 1e-300)))  # noqa: E731
    # the general form (any tapes and reductions per array) on the same four outputs
    from ncarray_gb300.batch import BatchExpr
    outs = [(None, nca.RedOp.SUM), (None, nca.RedOp.MEAN), (None, nca.RedOp.MAX), (lambda x: x * x - x, nca.RedOp.SUM)]
    G = BatchExpr([(a, outs) for a in arrays])
    G.launch(graph=True)
    torch.cuda.synchronize()
    ms_g = timeit(lambda: G.launch(graph=True), 5)
    gv, _ = G.run(graph=True)
    general = op_entry(nbytes, ms_g, peak, elements=int(lens.sum()), info=G.info(),
                       max_rel_err={"sum": rel(gv[pick, 0], ref[:, 0]), "mean": rel(gv[pick, 1], ref[:, 1]),
                                    "sum_x_times_x_minus_x": rel(gv[pick, 3], ref[:, 3]),
                                    "max_exact": bool(np.array_equal(gv[pick, 2], ref[:, 2]))},
                       note="x*x - x rounded as the tape says (two float32 roundings), then summed")
    del G
    return op_entry(nbytes, ms_b, peak, elements=int(lens.sum()), arrays=n_arrays, bytes=nbytes, cpu_baseline=cpu,
                    general_form=general,
                    plain_ms=round(ms_p, 3),
                    speedup_vs_plain=round(ms_p / ms_b, 2), schedule=sched,
                    batched_max_rel_err={"sum": rel(g_[:, 0], ref[:, 0]), "mean": rel(g_[:, 1], ref[:, 1]),
                                         "sum_x2_minus_x": rel(g_[:, 3], ref[:, 3]),
                                         "max_exact": bool(np.array_equal(g_[:, 2], ref[:, 2]))},
                    plain_max_rel_err={"sum": rel(p_[:, 0], ref[:, 0]), "sum_x2_minus_x": rel(p_[:, 3], ref[:, 3])},
                    sample_checked=len(pick))


def profile_op(torch, nca, op: str, steps: int) -> None:
    """Runs one op `steps` times at the bench size, with no timing or JSON:
    the target of small, self-terminating profiler captures."""
    if op in ("c2-fused", "c2-int", "c2-multi"):
        x, v, k = c2_host()
        step = C2Step(nca, nca.NCDevArray.from_host(x), nca.NCDevArray.from_host(v), nca.NCDevArray.from_host(k))
        fn = {"c2-fused": step.fused, "c2-int": step.intexpr, "c2-multi": step.multi}[op]
    elif op in ("c3-7", "c3-27"):
        from ncarray_gb300.stencil import Stencil3D, laplacian7, laplacian27
        st = Stencil3D(laplacian7() if op == "c3-7" else laplacian27(), 0.1)
        a = nca.NCDevArray((512, 512, 512), nca.DType.float32)
        b = nca.NCDevArray((512, 512, 512), nca.DType.float32)
        a._buf.view(torch.float32).normal_()
        fn = lambda: st.apply(a, b)  # noqa: E731
    elif op == "c1":
        rng = np.random.default_rng(SEED)
        da, db, dc = (nca.NCDevArray.from_host(rng.uniform(-1, 1, (128, 128, 128))) for _ in range(3))
        with nca.lazy_mode():
            e = da * db + nca.sqrt(abs(dc)) - 0.5 * da
        out = nca.NCDevArray(e.shape, e.dtype)
        fn = lambda: e.evaluate(out=out, reductions=[(nca.RedOp.SUM, 0), (nca.RedOp.MAX, 0)])  # noqa: E731
    elif op in ("c4", "c4-counts", "c4-small", "c4-counts-small"):
        # the small forms: 2^25 points (128 MB per array, above L2) for full captures
        from ncarray_gb300.hist import hist2d_into
        x, y, w = c4_points(torch, nca, (1 << 25) if op.endswith("small") else (1 << 27))
        counts = nca.NCDevArray((1024, 1024), nca.DType.uint64).fill(0)
        wsum = nca.NCDevArray((1024, 1024), nca.DType.float32).fill(0.0)
        if not op.startswith("c4-counts"):
            fn = lambda: hist2d_into(x, y, counts, (0.0, 1.0), (0.0, 1.0), w, wsum)  # noqa: E731
        else:
            fn = lambda: hist2d_into(x, y, counts, (0.0, 1.0), (0.0, 1.0))  # noqa: E731
    elif op == "binning":
        # the fused sum of eight strided views of a (32, 512, 1024) image (2x2x2 bins)
        data = nca.NCDevArray((32, 512, 1024), nca.DType.float32)
        data._buf.view(torch.float32).copy_(torch.rand(32 * 512 * 1024, device="cuda"))
        e = None
        with nca.lazy_mode():
            for a in range(2):
                for b in range(2):
                    for c in range(2):
                        v = data[a::2, b::2, c::2]
                        e = v if e is None else e + v
            e = e * 0.125
        out = nca.NCDevArray((16, 256, 512), nca.DType.float32)
        fn = lambda: e.evaluate(out=out)  # noqa: E731
    elif op == "binning-reshape":
        # the same binning as reshape(16, 2, 256, 2, 512, 2).sum((1, 3, 5))
        data = nca.NCDevArray((32, 512, 1024), nca.DType.float32)
        data._buf.view(torch.float32).copy_(torch.rand(32 * 512 * 1024, device="cuda"))
        six = data.reshape(16, 2, 256, 2, 512, 2)._expr()
        out = nca.NCDevArray((16, 256, 512), nca.DType.float32)
        fn = lambda: six.evaluate(reductions=[(nca.RedOp.SUM, (1, 3, 5))], red_out=[out])  # noqa: E731
    elif op in ("red-global-sum", "red-rows64"):
        # plain reductions of 256 MB float32: a global sum, a sum over rows of 64
        shape, red = ((64 << 20,), [(nca.RedOp.SUM, None)]) if op == "red-global-sum" else \
            ((1 << 20, 64), [(nca.RedOp.SUM, 1)])
        x = torch.randn(int(np.prod(shape)), device="cuda", dtype=torch.float32)
        e = nca.NCDevArray(shape, nca.DType.float32, _buf=x.view(torch.uint8))._expr()
        fn = lambda: e.evaluate(reductions=red)  # noqa: E731
    elif op == "c5-small":
        # the batched reduction on 1,000 of the uneven arrays (about 1 GB)
        from ncarray_gb300.batch import Batch
        _, _, arrays, _, _ = c5_arrays(torch, nca, 1000)
        B = Batch(arrays)
        B.run(graph=False)
        fn = lambda: B.run(graph=False)  # noqa: E731
    elif op == "c2-multi-small":
        # the one-pass C2 step on half of the b axis: x (64,128,256,8), k (8,128,256,64)
        # (x, k, y, z 64 MiB each, above L2), for full profiler captures
        rng = np.random.default_rng(SEED + 12)
        x = rng.standard_normal((64, 128, 256, 8), dtype=np.float32)
        v = rng.standard_normal(128, dtype=np.float32)
        k = rng.integers(-1000, 1001, (8, 128, 256, 64), dtype=np.int32)
        dx, dv, dk = (nca.NCDevArray.from_host(a) for a in (x, v, k))
        with nca.lazy_mode():
            ye = dx.permute(3, 1, 2, 0) * dv.reshape(1, 128, 1, 1) + dk
            ze = (dk * 3 + 7) % 11
        y, z = nca.NCDevArray(ye.shape, ye.dtype), nca.NCDevArray(ze.shape, ze.dtype)
        red = [(nca.RedOp.MAX, 2), (nca.RedOp.ARGMAX, 2)]
        fn = lambda: nca.evaluate_many([(ye, y), (ze, z)], reductions=red)  # noqa: E731
    elif op == "c1-variants":
        # the C1 expression and its parts (x, a*b, sqrt(abs(c)), 0.5*a, all) on
        # float64 (128,128,128), each with the axis-0 sum and max, the sum, the
        # max: float64 instruction counts per part
        rng = np.random.default_rng(SEED)
        da, db, dc = (nca.NCDevArray.from_host(rng.uniform(-1, 1, (128, 128, 128))) for _ in range(3))
        with nca.lazy_mode():
            parts = [da._expr(), da * db, nca.sqrt(abs(dc)), 0.5 * da, da * db + nca.sqrt(abs(dc)) - 0.5 * da]
        outs = [nca.NCDevArray(e.shape, e.dtype) for e in parts]
        reds = ([(nca.RedOp.SUM, 0), (nca.RedOp.MAX, 0)], [(nca.RedOp.SUM, 0)], [(nca.RedOp.MAX, 0)])

        def fn():
            for e, o in zip(parts, outs):
                for r in reds:
                    e.evaluate(out=o, reductions=r)
    elif op == "red-global-sum-noalloc":
        # the global sum of 64 Mi float32 (256 MB) through nca_reduce_noalloc
        import ctypes
        from ncarray_gb300 import _lib
        x = torch.randn(64 << 20, device="cuda", dtype=torch.float32)
        res = torch.zeros(1, dtype=torch.float32, device="cuda")
        src = _lib.make_view(x.data_ptr(), int(nca.DType.float32), (64 << 20,), (4,))
        dst = _lib.make_view(res.data_ptr(), int(nca.DType.float32), (), ())
        fn = lambda: _lib.call("nca_reduce_noalloc", ctypes.byref(src), 0, ctypes.byref(dst),  # noqa: E731
                               torch.cuda.current_stream().cuda_stream)
    elif op == "c5-general-small":
        # the general batched form (any tapes and reductions) on 1,000 of the uneven arrays
        from ncarray_gb300.batch import BatchExpr
        _, _, arrays, _, _ = c5_arrays(torch, nca, 1000)
        outs = [(None, nca.RedOp.SUM), (None, nca.RedOp.MEAN), (None, nca.RedOp.MAX),
                (lambda x: x * x - x, nca.RedOp.SUM)]
        G = BatchExpr([(a, outs) for a in arrays])
        G.launch(graph=False)
        fn = lambda: G.launch(graph=False)  # noqa: E731
    elif op == "red-axis0":
        # float32 (4096, 16384) summed over axis 0 (256 MB read, 64 KB written)
        x = torch.randn(4096 * 16384, device="cuda", dtype=torch.float32)
        e = nca.NCDevArray((4096, 16384), nca.DType.float32, _buf=x.view(torch.uint8))._expr()
        fn = lambda: e.evaluate(reductions=[(nca.RedOp.SUM, 0)])  # noqa: E731
    elif op == "scatter-add":
        # 2^26 float32 values scattered into 2^20 float32 entries by int64 indices
        # drawn from 8 narrow Gaussians (768 MB read)
        g = torch.Generator(device="cuda").manual_seed(SEED + 11)
        n, nd = 1 << 26, 1 << 20
        cen = torch.randint(0, nd, (8,), generator=g, device="cuda").float()
        comp = torch.randint(0, 8, (n,), generator=g, device="cuda")
        idx = (cen[comp] + torch.randn(n, generator=g, device="cuda") * 2000.0).long().clamp_(0, nd - 1)
        src = torch.rand(n, generator=g, device="cuda")
        di = nca.NCDevArray((n,), nca.DType.int64, _buf=idx.view(torch.uint8))
        ds = nca.NCDevArray((n,), nca.DType.float32, _buf=src.view(torch.uint8))
        dest = nca.NCDevArray((nd,), nca.DType.float32).fill(0.0)
        fn = lambda: dest.scatter_add(di, ds)  # noqa: E731
    elif op in ("stencil-general-7", "stencil-general-27"):
        # the 7- / 27-point Laplacian through the general stencil on a
        # zero-padded (322, 322, 322) float32 grid (133 MB in, 131 MB out)
        from ncarray_gb300.stencil import laplacian7, laplacian27
        st = general_laplacian(nca, laplacian7() if op.endswith("-7") else laplacian27())
        src = nca.NCDevArray((322, 322, 322), nca.DType.float32)
        src._buf.view(torch.float32).normal_()
        out = nca.NCDevArray((320, 320, 320), nca.DType.float32)
        fn = lambda: st.apply(src, out)  # noqa: E731
    elif op == "stencil-binning":
        # the pixel-binning stencil of the reference's benchmark through the
        # general stencil: 8 offset views of a (32, 512, 1024) float32 image
        from ncarray_gb300.stencil import Stencil
        src = nca.NCDevArray((32, 512, 1024), nca.DType.float32)
        src._buf.view(torch.float32).copy_(torch.rand(32 * 512 * 1024, device="cuda"))
        offs = [(p, r, c) for p in range(2) for r in range(2) for c in range(2)]

        def binning(views):
            e = nca.DevExpr.leaf(views[0])
            for v in views[1:]:
                e = e + v
            return e * np.float32(0.125)

        st = Stencil.create(offs, binning, nca.DType.float32, is_pointer_axis=[0, 0, 0])
        out = nca.NCDevArray((16, 256, 512), nca.DType.float32)
        fn = lambda: st.apply(src, out)  # noqa: E731
    else:
        raise SystemExit(f"unknown --profile-op {op}")
    for _ in range(steps):
        fn()
    torch.cuda.synchronize()
    print(f"profile-op {op}: {steps} runs ok")


def all_reduce_max(dist, torch, v: float, device: str) -> float:
    """The maximum of v over the ranks of the default process group."""
    t = torch.tensor([v], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(ms_total: float, steps: int, world: int, bytes_per_step: float, reduce_max):
    """Whole-job GB/s: every rank processes bytes_per_step per step (weak
    scaling); the job's time is the slowest rank's. Returns (GB/s, ms/step)."""
    ms_step = reduce_max(ms_total) / steps
    return world * bytes_per_step / (ms_step * 1e-3) / 1e9, ms_step


def omp_threads() -> int:
    try:
        return int(os.environ.get("OMP_NUM_THREADS", "")) or os.cpu_count() or 1
    except ValueError:
        return os.cpu_count() or 1


def run_reference(args, rank: int):
    if rank != 0:
        return
    import oracle
    oracle.build(with_ref=False)
    threads = omp_threads()
    vals = []
    for _ in range(max(args.warmup, 0)):
        cpu_baseline_c2(threads)
    for _ in range(args.steps):
        gbs, n, dt = cpu_baseline_c2(threads)
        vals.append((gbs, dt))
    gbs = statistics.median(v[0] for v in vals)
    sample = f"view slice 0 of 8 along axis 0: {n} elements of the step (1/8 of the workload)"
    line = {
        "impl": "reference", "metric": METRIC, "value": round(gbs, 3), "unit": "GB/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(statistics.median(v[1] for v in vals) * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+i32", "data": "synthetic",
        "config": {"workload": "strided/broadcast fusion f32 (8,256,256,64) permuted view * bcast v + i32; "
                               "max+argmax axis 2; (k*3+7)%11", "sample_of_workload": 1 / 8},
        "cpu_baseline": {"value": round(gbs, 3), "unit": "GB/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(gbs, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--headline-only", action="store_true", help="skip the per-op measurements of the other workloads")
    ap.add_argument("--only", default=None, choices=["c1", "c3", "c4", "c5", "binning", "reductions"],
                    help="measure one per-op workload and print its figures (no headline line)")
    ap.add_argument("--profile-op", default=None, help="run one op --steps times for a profiler capture")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if args.only:
        import torch
        import ncarray_gb300 as nca
        peak, _ = peaks()
        flush_buf = torch.empty(512 << 20, dtype=torch.uint8, device="cuda") if args.only in ("c1", "binning") else None
        fn = {"c1": lambda: measure_c1(torch, nca, peak, flush_buf), "c3": lambda: measure_c3(torch, nca, peak),
              "c4": lambda: measure_c4(torch, nca, peak), "c5": lambda: measure_c5(torch, nca, peak),
              "binning": lambda: measure_binning(torch, nca, peak, flush_buf),
              "reductions": lambda: measure_reductions(torch, nca, peak)}[args.only]
        print(json.dumps({args.only: fn()}), flush=True)
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from ncarray_gb300 import build as nbuild
    nbuild.build()
    import ncarray_gb300 as nca
    from ncarray_gb300 import _lib
    if args.profile_op:
        profile_op(torch, nca, args.profile_op, args.steps)
        return

    x, v, k = c2_host()
    n = int(np.prod(k.shape))
    by = c2_bytes(n)
    dx = nca.NCDevArray.from_host(x)
    dv = nca.NCDevArray.from_host(v)
    dk = nca.NCDevArray.from_host(k)
    step = C2Step(nca, dx, dv, dk)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # correctness spot check against the host formula on one slice
    y0 = step.y[0].to_host()
    ref0 = x.transpose(3, 1, 2, 0)[0] * v.reshape(256, 1, 1) + k[0].astype(np.float32)
    if not np.array_equal(y0, ref0):
        raise SystemExit("bench: y differs from the host formula")
    if not np.array_equal(step.am.to_host()[0], np.argmax(ref0, axis=1)):
        raise SystemExit("bench: argmax differs from the host formula")

    # one step = one replay of the captured graph of the step's C-ABI calls
    l0 = _lib.lib().nca_launch_count()
    step()
    torch.cuda.synchronize()
    per_step_launches = _lib.lib().nca_launch_count() - l0
    side = torch.cuda.Stream()
    g_step = make_graph(torch, (lambda: step.forked(torch, side)) if C2_FORKED else step.multi)
    g_fused = make_graph(torch, step.fused)
    g_int = make_graph(torch, step.intexpr)
    for _ in range(args.warmup):
        g_step.replay()
    torch.cuda.synchronize()
    dev_index = int(os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[0] or 0) if world == 1 else local
    sampler = ClockSampler(dev_index)
    sampler.start()
    time.sleep(0.15)
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0.record(s)
    for _ in range(args.steps):
        g_step.replay()
    e1.record(s)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms_total = e0.elapsed_time(e1)
    launches = per_step_launches * args.steps
    # per-kernel timing for the roofline: the dominant kernel is the one-pass
    # kernel (the whole step) or, for the forked step, the fused pass
    ms_fused = time_events(torch, g_fused.replay, args.steps)
    ms_int = time_events(torch, g_int.replay, args.steps)
    ms_dom = ms_fused if C2_FORKED else time_events(torch, g_step.replay, args.steps)
    bytes_dom = by["fused"] if C2_FORKED else by["step"]
    clocks = sampler.stop()
    value, ms_step = job_throughput(ms_total, args.steps, world, by["step"],
                                    (lambda v: all_reduce_max(dist, torch, v, "cuda")) if dist else (lambda v: v))
    peak, peak_kind = peaks()
    fused_gbs = by["fused"] / (ms_fused * 1e-3) / 1e9
    int_gbs = by["int"] / (ms_int * 1e-3) / 1e9
    dom_gbs = bytes_dom / (ms_dom * 1e-3) / 1e9

    # end to end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        hx = torch.from_numpy(x).pin_memory()
        hv = torch.from_numpy(v).pin_memory()
        hk = torch.from_numpy(k).pin_memory()
        hy = torch.empty(n, dtype=torch.float32).pin_memory()
        hz = torch.empty(n, dtype=torch.int32).pin_memory()
        hm = torch.empty(n // 256, dtype=torch.float32).pin_memory()
        ha = torch.empty(n // 256, dtype=torch.int64).pin_memory()
        h2d = x.nbytes + v.nbytes + k.nbytes
        d2h = 4 * n * 2 + 12 * (n // 256)

        def bytes_view(a):
            return a._buf[a._offset: a._offset + a.nbytes]

        def e2e_step():
            bytes_view(dx).copy_(hx.view(-1).view(torch.uint8), non_blocking=True)
            bytes_view(dv).copy_(hv.view(torch.uint8), non_blocking=True)
            bytes_view(dk).copy_(hk.view(-1).view(torch.uint8), non_blocking=True)
            step()
            hy.view(torch.uint8).copy_(bytes_view(step.y), non_blocking=True)
            hz.view(torch.uint8).copy_(bytes_view(step.z), non_blocking=True)
            hm.view(torch.uint8).copy_(bytes_view(step.mx), non_blocking=True)
            ha.view(torch.uint8).copy_(bytes_view(step.am), non_blocking=True)

        for _ in range(3):
            e2e_step()
        reps = max(5, min(args.steps, 50))
        ms_serial = time_events(torch, e2e_step, reps)

        # the same step in NCH chunks along axis 1 (b), pipelined over three
        # streams: host->device copies of chunk i+1, the fused and int32
        # expressions of chunk i and device->host copies of chunk i-1 overlap
        # (host<->device copies of strided chunk views through nca_copy_host)
        NCH = int(os.environ.get("NCA_E2E_CHUNKS", "2"))
        NCS = int(os.environ.get("NCA_E2E_COPY_STREAMS", "1"))
        bc = 256 // NCH
        hx4, hk4 = hx.view(64, 256, 256, 8), hk.view(8, 256, 256, 64)
        hy4, hz4 = hy.view(8, 256, 256, 64), hz.view(8, 256, 256, 64)
        hm3, ha3 = hm.view(8, 256, 64), ha.view(8, 256, 64)
        red = [(nca.RedOp.MAX, 2), (nca.RedOp.ARGMAX, 2)]

        def chunk_parts(bx, bv, bk, by_, bz, bm, ba):
            """the NCH chunk views of one set of device buffers"""
            out = []
            for i in range(NCH):
                b0, b1 = i * bc, (i + 1) * bc
                dxc, dvc, dkc = bx[:, b0:b1], bv[b0:b1], bk[:, b0:b1]
                with nca.lazy_mode():
                    ye = dxc.permute(3, 1, 2, 0) * dvc.reshape(1, bc, 1, 1) + dkc
                    ze = (dkc * 3 + 7) % 11
                out.append(dict(dx=dxc, dv=dvc, dk=dkc, ye=ye, ze=ze, y=by_[:, b0:b1], z=bz[:, b0:b1],
                                mx=bm[:, b0:b1], am=ba[:, b0:b1], hx=hx4[:, b0:b1], hv=hv[b0:b1],
                                hk=hk4[:, b0:b1], hy=hy4[:, b0:b1], hz=hz4[:, b0:b1], hm=hm3[:, b0:b1],
                                ha=ha3[:, b0:b1]))
            return out

        # two sets of device buffers: consecutive steps alternate between them,
        # so a step waits only for the step two back to release its buffers
        sets = [chunk_parts(dx, dv, dk, step.y, step.z, step.mx, step.am)]
        sets.append(chunk_parts(nca.NCDevArray(dx.shape, dx.dtype), nca.NCDevArray(dv.shape, dv.dtype),
                                nca.NCDevArray(dk.shape, dk.dtype), nca.NCDevArray(step.y.shape, step.y.dtype),
                                nca.NCDevArray(step.z.shape, step.z.dtype), nca.NCDevArray(step.mx.shape, step.mx.dtype),
                                nca.NCDevArray(step.am.shape, step.am.dtype)))
        s_ins = [torch.cuda.Stream() for _ in range(NCS)]
        s_outs = [torch.cuda.Stream() for _ in range(NCS)]
        s_cmp = torch.cuda.Stream()
        ev_in = [[torch.cuda.Event() for _ in range(NCH)] for _ in sets]
        ev_cmp = [[torch.cuda.Event() for _ in range(NCH)] for _ in sets]
        ev_out = [[torch.cuda.Event() for _ in range(NCH)] for _ in sets]

        def e2e_pipelined(cross_step=True, nsteps=1):
            """nsteps steps, each copying all its inputs in and all its results
            out; step r uses buffer set r % 2. With cross_step the first steps
            also wait for a previous call's use of their set (later steps always
            wait for the step two back)."""
            cur = torch.cuda.current_stream()
            for st in s_ins + s_outs + [s_cmp]:
                st.wait_stream(cur)
            for r in range(nsteps):
                S = r % 2 if nsteps > 1 else 0
                cross = cross_step or r >= 2
                for i, c in enumerate(sets[S]):
                    s_in, s_out = s_ins[i % NCS], s_outs[i % NCS]
                    with torch.cuda.stream(s_in):
                        if cross:
                            s_in.wait_event(ev_cmp[S][i])   # the step before is done reading chunk i of set S
                        c["dx"].copy_from(c["hx"])
                        c["dv"].copy_from(c["hv"])
                        c["dk"].copy_from(c["hk"])
                        ev_in[S][i].record(s_in)
                    with torch.cuda.stream(s_cmp):
                        s_cmp.wait_event(ev_in[S][i])
                        if cross:
                            s_cmp.wait_event(ev_out[S][i])  # and its results in set S are on the host
                        if C2_FORKED:
                            c["ye"].evaluate(out=c["y"], reductions=red, red_out=[c["mx"], c["am"]])
                            c["ze"].evaluate(out=c["z"])
                        else:
                            nca.evaluate_many([(c["ye"], c["y"]), (c["ze"], c["z"])], reductions=red,
                                              red_out=[c["mx"], c["am"]])
                        ev_cmp[S][i].record(s_cmp)
                    with torch.cuda.stream(s_out):
                        s_out.wait_event(ev_cmp[S][i])
                        c["y"].copy_to(c["hy"])
                        c["z"].copy_to(c["hz"])
                        c["mx"].copy_to(c["hm"])
                        c["am"].copy_to(c["ha"])
                        ev_out[S][i].record(s_out)
            for st in s_ins + s_outs + [s_cmp]:
                cur.wait_stream(st)

        for _ in range(3):
            e2e_pipelined()
        torch.cuda.synchronize()
        ms_eager = time_events(torch, e2e_pipelined, reps)
        # GS pipelined steps captured in one CUDA graph: the host->device copies
        # of step r + 1 overlap the device->host copies of step r (replays of
        # one graph on one stream never overlap, so the first step of a replay
        # needs no cross-step waits)
        GS = int(os.environ.get("NCA_E2E_GRAPH_STEPS", "8"))
        g_e2e = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g_e2e):
            e2e_pipelined(cross_step=False, nsteps=GS)
        torch.cuda.synchronize()
        for _ in range(3):
            g_e2e.replay()
        ms_e2e = time_events(torch, g_e2e.replay, max(2, reps // GS)) / GS
        # the pipelined step computes the same results as the serial one
        hy_ref = hy.clone()
        e2e_step()
        torch.cuda.synchronize()
        hy.zero_()
        g_e2e.replay()
        torch.cuda.synchronize()
        same = bool(torch.equal(hy, hy_ref))
        e2e = {"value": round(by["step"] / (ms_e2e * 1e-3) / 1e9, 3), "unit": "GB/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "ms_per_step": round(ms_e2e, 4),
               "how": f"CUDA-graph replays of {GS} consecutive steps, each in {NCH} chunks along axis 1 "
                      f"pipelined over {NCS} copy-in, 1 compute and {NCS} copy-out streams (pinned host "
                      "buffers, nca_copy_host + " + ("evaluate" if C2_FORKED else "evaluate_many") +
                      " on chunk views; every step copies all its inputs in "
                      "and all its results out)",
               "serial_ms_per_step": round(ms_serial, 4), "eager_pipelined_ms_per_step": round(ms_eager, 4),
               "matches_serial": same}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = omp_threads()
        gbs, ns, dt = cpu_baseline_c2(threads)
        cpu = {"value": round(gbs, 3), "unit": "GB/s", "cores": threads, "kind": "port",
               "sample": f"view slice 0 of 8 along axis 0 ({ns} elements), one step, {dt:.2f} s"}

    per_op = {"c2_fused_expr_max_argmax": {"GB/s": round(fused_gbs, 1), "frac_of_measured": round(fused_gbs / peak, 4),
                                           "ms": round(ms_fused, 5), "note": "the first expression alone"},
              "c2_int_expr": {"GB/s": round(int_gbs, 1), "frac_of_measured": round(int_gbs / peak, 4),
                              "ms": round(ms_int, 5), "note": "the int32 expression alone"}}
    if not args.headline_only:
        del step, dx, dv, dk
        torch.cuda.empty_cache()
        flush_buf = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
        for name, fn in (("c1_fused_f64", lambda: measure_c1(torch, nca, peak, flush_buf)),
                         ("c3_stencil_f32", lambda: measure_c3(torch, nca, peak)),
                         ("c4_hist2d", lambda: measure_c4(torch, nca, peak)),
                         ("c5_batched", lambda: measure_c5(torch, nca, peak)),
                         ("binning", lambda: measure_binning(torch, nca, peak, flush_buf)),
                         ("reductions", lambda: measure_reductions(torch, nca, peak))):
            try:
                per_op[name] = fn()
            except Exception as ex:  # a failed side measurement must not hide the headline
                per_op[name] = {"error": f"{type(ex).__name__}: {ex}"[:300]}
            torch.cuda.empty_cache()

    traffic = None
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists():
        t = json.loads(tf.read_text()).get("c2_fused" if C2_FORKED else "c2_multi")
        if t:
            traffic = t.get("bytes_per_launch")
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_step, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+i32", "data": "synthetic (seeded numpy)",
        "config": {"workload": "strided/broadcast fusion: x f32 (64,256,256,8) viewed (3,1,2,0) * v[None,:,None,None]"
                               " + k i32 (8,256,256,64); y stored + max/argmax axis 2 in one pass; (k*3+7)%11",
                   "elements": n, "bytes_per_step": by["step"], "l2": "working set 640 MB > L2; no flush",
                   "launch": ("each step is one replay of a CUDA graph of its C-ABI calls (the fused and the "
                              "int32 expressions on two forked streams)") if C2_FORKED else
                             ("each step is one replay of a CUDA graph of one nca_expr_multi call: y, z, max and "
                              "argmax from one TMA-staged pass that reads x and k once"),
                   "parallelism": f"replicas x{world}"},
        "roofline": {"bound": "hbm", "achieved": round(dom_gbs, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(dom_gbs / peak, 4), "traffic": traffic, "peak_kind": peak_kind,
                     "kernel": ("nca_staged_async: TMA-staged fused expression + axis-2 max/argmax") if C2_FORKED else
                               ("nca_staged_async with an extra output: y = x.permute * v + k stored, max/argmax "
                                "over axis 2, z = (k*3+7)%11 stored, one pass"),
                     "bytes_per_launch": bytes_dom, "ms_per_launch": round(ms_dom, 5)},
        "per_op": per_op,
        "gpu_launches": int(launches),
        "clocks": clocks,
        "e2e": e2e,
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
