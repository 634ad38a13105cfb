"""Benchmark: direct Biot-Savart velocity, 1,000,000 particles, Gaussian core (one GB300).

Workload (the precision configuration): 1M particles, positions ~ N(0, 0.25^2 I) in FP32,
strength proportional to exp(-r^2/0.125) normalised to total 1, core radius 0.005, Gaussian
("exponential") core, thick targets = the particles themselves.  One step = one full
N x N velocity evaluation (10^12 interactions, self pair included) through the engine.

  value : compensated-FP32 Ginteractions/s, device-resident inputs, main + reduce kernels,
          CUDA events on the launching stream, L2 flushed between steps;
  e2e   : the same evaluation through the host-pointer C ABI call (host arrays in, host
          arrays out, copies inside the timed region);
  plain : the plain-FP32 drop-in kernel measured the same way;
  precision : max / RMS relative error of both modes against the FP64 oracle on a seeded
          1024-target subset (measured outside the timed region).

``--impl reference`` times the reference's CPU implementation of the same call (its own
compiled code where available, else the C restatement with the same arithmetic: float pairs,
double accumulators, OpenMP over targets) on all host cores, on a bounded target subset.
Under torchrun each rank evaluates its own copy of the workload (targets shard naturally;
no collective on the data path) and rank 0 reports the aggregate.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N = 1_000_000
SIGMA = 0.005
SEED = 2
METRIC = "Ginteractions/s @N=1M, compensated vs plain fp32 @err\u22641e-6 vs fp64; adjoint/fwd"
UNIT = "Ginteractions/s"
FLOPS_PER_PAIR = 19        # flopsu_0v_0b for the exponential core (src/Kernels.h:79 + src/CoreFunc.h:145)
FMA_PER_CLK_PER_SM = 128   # FP32 lanes per SM per clock


def make_workload(seed=SEED, n=None):
    n = N if n is None else n          # N is set from --n at run time
    rng = np.random.default_rng(seed)
    x, y = rng.normal(0.0, 0.25, (2, n)).astype(np.float32)
    g = np.exp(-(x.astype(np.float64) ** 2 + y.astype(np.float64) ** 2) / 0.125)
    s = (g / g.sum()).astype(np.float32)
    r = np.full(n, SIGMA, np.float32)
    return x, y, r, s


ADJ_NS = 500_000          # differentiation workload: sources uniform in [-1,1]^2, core 0.01, Gaussian
ADJ_GRID = 100            # probes on a 100 x 100 grid over [-0.5,0.5]^2; loss = sum |u_probe|^2


def make_adjoint_workload(seed=4):
    rng = np.random.default_rng(seed)
    sx, sy = rng.uniform(-1.0, 1.0, (2, ADJ_NS)).astype(np.float32)
    ss = rng.normal(0.0, 1.0 / np.sqrt(ADJ_NS), ADJ_NS).astype(np.float32)
    sr = np.full(ADJ_NS, 0.01, np.float32)
    g = np.linspace(-0.5, 0.5, ADJ_GRID, dtype=np.float32)
    px, py = [a.ravel().astype(np.float32) for a in np.meshgrid(g, g)]
    return sx, sy, sr, ss, px, py


def time_adjoint(og, torch, ctx, stream, dev, flush, steps, warmup):
    """Forward (finalized probe velocities) and hand-written backward (dL/d source x, y, G of
    L = sum u^2 + v^2 over the probes), both compensated, device-resident inputs, CUDA events on
    the launching stream, L2 flushed before each timed call.  Returns timings, the backward's
    launch count and, for the precision check, the host arrays and the device results."""
    sx, sy, sr, ss, px, py = make_adjoint_workload()
    SX, SY, SR, SS, PX, PY = [torch.from_numpy(a).to(dev) for a in (sx, sy, sr, ss, px, py)]
    npb = px.size
    PU = torch.zeros(npb, device=dev)
    PV = torch.zeros(npb, device=dev)
    GX, GY, GS = [torch.zeros(ADJ_NS, device=dev) for _ in range(3)]

    def fwd():
        PU.zero_()
        PV.zero_()
        og.points_affect_points_dev(ctx, og.CORE_GAUSSIAN, og.VELONLY, og.COMPENSATED, SX, SY, SR, SS, PX, PY, None,
                                    PU, PV, finalize=True)

    def bwd():
        GX.zero_()
        GY.zero_()
        GS.zero_()
        og.points_affect_points_vjp_dev(ctx, og.CORE_GAUSSIAN, og.COMPENSATED, SX, SY, SR, SS, PX, PY, None,
                                        2.0 * PU, 2.0 * PV, GX, GY, GS)

    def timed(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        tot = 0.0
        l0 = ctx.launches
        for _ in range(steps):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            tot += e0.elapsed_time(e1)
        ctx.synchronize()
        return tot / steps, ctx.launches - l0

    f_ms, f_l = timed(fwd)
    fwd()
    b_ms, b_l = timed(bwd)
    pairs = float(ADJ_NS) * npb
    res = {"workload": f"{ADJ_NS} sources U[-1,1]^2, core 0.01, Gaussian; {npb} probes on a "
                       f"{ADJ_GRID}x{ADJ_GRID} grid over [-0.5,0.5]^2; loss sum |u|^2 (no freestream)",
           "forward_ms": f_ms, "backward_ms": b_ms, "adjoint_over_forward": b_ms / f_ms,
           "forward_ginter_s": pairs / (f_ms * 1e-3) / 1e9, "backward_ginter_s": pairs / (b_ms * 1e-3) / 1e9}
    host = (sx, sy, sr, ss, px, py, PU.cpu().numpy(), PV.cpu().numpy(), GX.cpu().numpy(), GY.cpu().numpy(),
            GS.cpu().numpy())
    return res, f_l + b_l, host


def max_over_ranks(value: float, device=None) -> float:
    """The largest of one float over all ranks (the identity on one process)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank: float, world_size: int, max_ms: float) -> float:
    """Whole-job throughput in G-units/s: every rank's units over the slowest rank's time."""
    return world_size * units_per_rank / (max_ms * 1e-3) / 1e9


def time_gradient(og, torch, ctx, stream, dev, flush, X, Y, R, S, args):
    """Velocity + velocity gradient of the headline patch (VELANDGRAD, generic kernel):
    one timed call per accumulation mode after one warm-up, CUDA events, L2 flushed."""
    n = X.numel()
    U, V = torch.zeros(n, device=dev), torch.zeros(n, device=dev)
    G = [torch.zeros(n, device=dev) for _ in range(4)]
    out = {"kernel": "p2p_packed_res_kernel<thick, compensated, GRAD> (Morton-ordered; far blocks d^2/s^2 > 25 "
                     "without the exponential)", "flops_per_interaction": 41}
    for name, accum in (("compensated", og.COMPENSATED), ("plain", og.PLAIN_F32)):
        def call():
            for t in (U, V, *G):
                t.zero_()
            og.points_affect_points_dev(ctx, og.CORE_GAUSSIAN, og.VELANDGRAD, accum, X, Y, R, S, X, Y, R, U, V,
                                        extra=G)
        ms = _event_time(torch, stream, flush, call, 1, 1)
        out[name] = {"ms": ms, "ginter_s": float(n) * n / (ms * 1e-3) / 1e9}
        out["_grad_" + name] = [t.cpu().numpy() for t in G]
    return out


def time_tree(og, torch, ctx, stream, flush, X, Y, R, S, args):
    """The same N x N velocity evaluation by treecode (obs_points_affect_points_tree: theta 0.5,
    24 terms), CUDA events on the launching stream, L2 flushed; its error against the FP64 direct
    sum is filled in with the headline's precision check."""
    n = X.numel()
    U, V = torch.zeros(n, device=X.device), torch.zeros(n, device=X.device)

    def call():
        U.zero_()
        V.zero_()
        og.points_affect_points_tree_dev(ctx, og.CORE_GAUSSIAN, X, Y, R, S, X, Y, R, U, V)
    ms = _event_time(torch, stream, flush, call, max(1, args.steps // 2), 2)
    return {"kernel": "tree_eval_kernel (Morton-ordered tree of 32-source leaves, 4-way nodes, 24-term "
                      "multipole expansions; theta 0.5)", "ms": ms,
            "effective_ginter_s": float(n) * n / (ms * 1e-3) / 1e9,
            "_uv": (U, V)}


def workload_config() -> dict:
    """The headline workload, named the same way by both arms."""
    return {"workload": f"gaussian_patch_{N}", "n": N, "core": "gaussian", "sigma": SIGMA,
            "targets": "thick (the particles)", "seed": SEED, "l2": "flushed between steps (256 MB write)"}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        # samples go to a temporary file, or to $OBS_CLOCKS_DIR when the caller wants to keep them
        keep = os.environ.get("OBS_CLOCKS_DIR")
        self.path = (os.path.join(keep, f"clocks_gpu{gpu_index}.csv") if keep else
                     os.path.join(tempfile.gettempdir(), f"omega2d_clocks_{os.getpid()}_gpu{gpu_index}.csv"))

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [q.strip() for q in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if p[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


def profiled_traffic():
    """Per-launch DRAM traffic of the main kernel from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("p2p_gauss_comp_1M_bytes_per_launch"):
            return float(line.split("=")[1])
    return None


def rel_errs(ref64, got):
    e = np.abs(np.asarray(got, np.float64) - ref64)
    return float(e.max() / np.abs(ref64).max()), float(np.sqrt((e ** 2).sum() / (ref64 ** 2).sum()))


def cpu_sample(kind_pref, x, y, r, s, sample, threads):
    """Time the reference CPU path on `sample` targets against all sources; returns (sec, kind)."""
    from oracle import pyoracle as po
    idx = np.random.default_rng(99).choice(x.size, sample, replace=False)
    tx, ty, tr = x[idx], y[idx], r[idx]
    os.environ["OMP_NUM_THREADS"] = str(threads)
    if kind_pref == "reference" and po.Reference.available(po.GAUSS):
        ref = po.Reference(po.GAUSS)
        t0 = time.perf_counter()
        ref.points_affect_points(po.VELONLY, x, y, r, s, tx, ty, tr)
        return time.perf_counter() - t0, "reference"
    orc = po.Restatement(native=True)
    t0 = time.perf_counter()
    orc.points_affect_points(po.GAUSS, po.VELONLY, x, y, r, s, tx, ty, tr)
    return time.perf_counter() - t0, "port"


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    x, y, r, s = make_workload()
    threads = os.cpu_count() or 1
    sample = args.cpu_sample
    for _ in range(args.warmup if args.warmup < 1 else 1):
        cpu_sample("reference", x, y, r, s, 256, threads)
    tot, kind = 0.0, "port"
    for _ in range(args.steps):
        dt, kind = cpu_sample("reference", x, y, r, s, sample, threads)
        tot += dt
    v = args.steps * sample * x.size / tot / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 pairs, f64 accum",
            "data": "synthetic", "config": workload_config(),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": kind,
                             "sample": f"{sample} seeded targets x {N} sources per step"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_engine(args):
    import torch
    import omega2d_gb300 as og

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    x, y, r, s = make_workload(SEED + rank)      # each rank: its own 1M-target shard problem
    ctx = og.Context(local)
    stream = torch.cuda.Stream(dev)            # kernels and CUDA events share this stream
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    X, Y, R, S = [torch.from_numpy(a).to(dev) for a in (x, y, r, s)]
    TU = torch.zeros(N, device=dev)
    TV = torch.zeros(N, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)   # > L2 (129 MB)
    pairs = float(N) * float(N)

    def step(accum):
        TU.zero_()
        TV.zero_()
        og.points_affect_points_dev(ctx, og.CORE_GAUSSIAN, og.VELONLY, accum, X, Y, R, S, X, Y, R, TU, TV)

    def timed(accum, steps, warmup):
        ctx.enable_timing(True)
        for _ in range(warmup):
            step(accum)
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        tot, main = 0.0, 0.0
        launches0 = ctx.launches
        for _ in range(steps):
            flush.fill_(1.0)                     # evict L2 between timed steps
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step(accum)
            e1.record(stream)
            e1.synchronize()
            tot += e0.elapsed_time(e1)
            main += ctx.last_timing()[0]
        torch.cuda.synchronize()
        ctx.synchronize()
        launches = ctx.launches - launches0
        if ws > 1:
            tot = max_over_ranks(tot, dev)
            torch.distributed.barrier()
        return tot / steps, main / steps, launches

    with ClockSampler(local) as clk:
        ms_comp, main_comp, launches = timed(og.COMPENSATED, args.steps, args.warmup)
        ms_plain, main_plain, _ = timed(og.PLAIN_F32, max(1, args.steps // 2), 1)
        adjoint, adj_launches, adj_host = time_adjoint(og, torch, ctx, stream, dev, flush, args.steps, args.warmup)
        gradient = time_gradient(og, torch, ctx, stream, dev, flush, X, Y, R, S, args)
        tree = time_tree(og, torch, ctx, stream, flush, X, Y, R, S, args)
    clocks = clk.summary()

    # end to end through the host-pointer C ABI call (copies in the timed region), the host
    # arrays in pinned memory
    keep = []

    def pinned(a):
        t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).pin_memory()
        keep.append(t)
        return t.numpy()

    e2e_ms = []
    hp_src = og.Points(x, y, r, s)
    hp_src.x, hp_src.y, hp_src.r, hp_src.s = (pinned(a) for a in (x, y, r, s))
    tx_p, ty_p, tr_p = (pinned(a) for a in (x, y, r))
    for k in range(1 + max(1, args.steps // 2)):
        hp_t = og.Points(x, y, r, None)
        hp_t.x, hp_t.y, hp_t.r = tx_p, ty_p, tr_p
        hp_t.u, hp_t.v = pinned(np.zeros(N, np.float32)), pinned(np.zeros(N, np.float32))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        og.points_affect_points(hp_src, hp_t, og.VELONLY, og.ExecEnv(og.CORE_GAUSSIAN, og.COMPENSATED, ctx))
        t1 = time.perf_counter()
        if k > 0:
            e2e_ms.append(1e3 * (t1 - t0))
    h2d = 4 * N * 4 + 3 * N * 4 + 2 * N * 4
    d2h = 2 * N * 4

    value = aggregate_rate(pairs, ws, ms_comp)
    plain_value = aggregate_rate(pairs, ws, ms_plain)
    e2e_value = aggregate_rate(pairs, ws, max_over_ranks(float(np.mean(e2e_ms)), dev))

    if rank != 0:
        if ws > 1:
            torch.distributed.destroy_process_group()
        return

    # precision vs the FP64 oracle on a seeded target subset (outside the timed region)
    from oracle import pyoracle as po
    orc = po.Restatement()
    sub = np.random.default_rng(1234).choice(N, 1024, replace=False)
    u64, v64, _ = orc.points_affect_points(po.GAUSS, po.VELONLY, x, y, r, s, x[sub], y[sub], r[sub], fp64=True)
    ref64 = np.concatenate([u64, v64])
    prec = {"subset_targets": 1024}
    for name, accum in (("compensated", og.COMPENSATED), ("plain", og.PLAIN_F32)):
        step(accum)
        torch.cuda.synchronize()
        got = np.concatenate([TU.cpu().numpy()[sub], TV.cpu().numpy()[sub]])
        mx, rms = rel_errs(ref64, got)
        prec[name] = {"max_rel": mx, "rms_rel": rms}
    # velocity-gradient precision on the same 1024 targets (du/dx, dv/dx, du/dy, dv/dy)
    _, _, g64 = orc.points_affect_points(po.GAUSS, po.VELANDGRAD, x, y, r, s, x[sub], y[sub], r[sub], fp64=True)
    U_t, V_t = tree.pop("_uv")
    mx, rms = rel_errs(ref64, np.concatenate([U_t.cpu().numpy()[sub], V_t.cpu().numpy()[sub]]))
    tree.update(max_rel=mx, rms_rel=rms, speedup_over_direct=ms_comp / tree["ms"])
    ref_g = np.concatenate(g64)
    for name in ("compensated", "plain"):
        got = np.concatenate([a[sub] for a in gradient.pop("_grad_" + name)])
        mx, rms = rel_errs(ref_g, got)
        gradient[name]["max_rel"], gradient[name]["rms_rel"] = mx, rms
    # backward precision: the FP64 reference adjoint for 1024 seeded sources, with the same
    # cotangents (twice the engine's probe velocities)
    asx, asy, asr, ass, apx, apy, apu, apv, agx, agy, ags = adj_host
    asub = np.random.default_rng(4321).choice(ADJ_NS, 1024, replace=False)
    rx, ry, rs = orc.probe_vjp(po.GAUSS, asx[asub], asy[asub], asr[asub], ass[asub], apx, apy, 2.0 * apu, 2.0 * apv)
    adjoint["precision"] = {"subset_sources": 1024}
    for nm, ref, got in (("dL/dx", rx, agx[asub]), ("dL/dy", ry, agy[asub]), ("dL/dG", rs, ags[asub])):
        mx, rms = rel_errs(ref, got)
        adjoint["precision"][nm] = {"max_rel": mx, "rms_rel": rms}

    # CPU baseline: the reference's CPU path on a bounded sample, all host cores
    threads = os.cpu_count() or 1
    cpu_s, kind = cpu_sample("reference", x, y, r, s, args.cpu_sample, threads)
    cpu_v = args.cpu_sample * N / cpu_s / 1e9

    peaks = measured_peaks()
    sm_max = peaks.get("sm_max_mhz") or clocks.get("sm_max_mhz") or 2070.0
    nsm = torch.cuda.get_device_properties(dev).multi_processor_count
    fp32_peak = 2.0 * FMA_PER_CLK_PER_SM * nsm * sm_max * 1e6 / 1e12     # TFLOP/s
    achieved = pairs * FLOPS_PER_PAIR / (main_comp * 1e-3) / 1e12
    traffic = profiled_traffic()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_comp, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 pairs, compensated f32 + f64 reduce", "data": "synthetic",
        "config": workload_config(),
        "plain_fp32": {"value": plain_value, "unit": UNIT, "ms_per_step": ms_plain,
                       "compensated_over_plain": value / plain_value},
        "precision": prec,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": float(np.mean(e2e_ms))},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak, "traffic": traffic,
                     "kernel": "p2p_packed_kernel<GAUSS,thick,compensated,4> (Morton-ordered targets and sources)",
                     "flops_per_interaction": FLOPS_PER_PAIR,
                     "flops_note": "the reference's count for the Gaussian thick-target velocity kernel; far "
                                   "(warp, block) pairs execute 7 FP32 lane-ops + 1 MUFU.RCP per interaction",
                     "peak_note": f"2 x {FMA_PER_CLK_PER_SM} FP32 lanes x {nsm} SMs x {sm_max:.0f} MHz (max SM clock of measured)",
                     "frac_at_median_clock": (achieved / (fp32_peak * clocks["sm_mhz"] / sm_max)) if clocks.get("sm_mhz") else None,
                     "main_kernel_ms": main_comp},
        "cpu_baseline": {"value": cpu_v, "unit": UNIT, "cores": threads, "kind": kind,
                         "sample": f"{args.cpu_sample} seeded targets x {N} sources"},
        "adjoint": adjoint,
        "gradient": gradient,
        "treecode": tree,
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if not args.no_configs:
        # the other configurations, each with its own timings, precision and CPU baseline
        line["euler20k"] = run_euler20k(args)
        line["bem2048"] = run_bem2048(args)
        line["rk2adjoint"] = run_rk2adjoint2M(args, K=args.line_rk_steps, every=8)
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


# ---------------------------------------------------------------- the other configurations
# `--workload` runs one of them instead of the headline line; each prints one JSON line with
# its own metric, CUDA-event timings on the launching stream (L2 flushed between timed
# calls), a precision check against the FP64 oracle where one fits in seconds, and the CPU
# restatement timed on the host cores.

def _engine_setup():
    import torch
    import omega2d_gb300 as og
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    ctx = og.Context(0)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    return torch, og, dev, ctx, stream, flush


def _event_time(torch, stream, flush, fn, steps, warmup, prep=None):
    """Mean milliseconds of fn() over `steps` timed calls after `warmup` untimed ones; prep()
    (untimed) runs before every call."""
    for _ in range(warmup):
        if prep:
            prep()
        fn()
    torch.cuda.synchronize()
    tot = 0.0
    for _ in range(steps):
        if prep:
            prep()
        flush.fill_(1.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        tot += e0.elapsed_time(e1)
    return tot / steps


def run_euler20k(args):
    """20,000 vortex blobs U[-1,1]^2, G ~ N(0, 1/N), core 0.01, Rosenhead-Moore, freestream
    (1, 0): one velocity evaluation, then 10 first-order Euler steps with dt = 0.01.  Returns
    the result object."""
    torch, og, dev, ctx, stream, flush = _engine_setup()
    n, K, dt, fs = 20_000, 10, 0.01, (1.0, 0.0)
    rng = np.random.default_rng(1)
    x, y = rng.uniform(-1.0, 1.0, (2, n)).astype(np.float32)
    s = rng.normal(0.0, 1.0 / np.sqrt(n), n).astype(np.float32)
    r = np.full(n, 0.01, np.float32)
    X0, Y0, R, S = [torch.from_numpy(a).to(dev) for a in (x, y, r, s)]
    X, Y = X0.clone(), Y0.clone()
    U, V = torch.zeros(n, device=dev), torch.zeros(n, device=dev)
    out = {"workload": "euler20k", "metric": "Ginteractions/s, RM core, 20k particles, 10 Euler steps",
           "unit": UNIT, "data": "synthetic (seed 1)", "n": n, "steps_per_run": K}
    with ClockSampler(0) as clk:
        for name, accum in (("compensated", og.COMPENSATED), ("plain", og.PLAIN_F32)):
            def vel():
                U.zero_()
                V.zero_()
                og.points_affect_points_dev(ctx, og.CORE_RM, og.VELONLY, accum, X0, Y0, R, S, X0, Y0, R, U, V,
                                            finalize=True, fs=fs)

            def reset():
                X.copy_(X0)
                Y.copy_(Y0)

            def euler():
                og.advect_dev(ctx, og.CORE_RM, accum, 1, X, Y, R, S, fs, dt, K)
            tv = _event_time(torch, stream, flush, vel, args.steps, args.warmup)
            te = _event_time(torch, stream, flush, euler, args.steps, args.warmup, prep=reset)
            ctx.synchronize()
            out[name] = {"velocity_ms": tv, "velocity_ginter_s": n * n / (tv * 1e-3) / 1e9,
                         "euler10_ms": te, "value": K * n * n / (te * 1e-3) / 1e9,
                         "final_x": X.cpu().numpy().astype(np.float64), "final_y": Y.cpu().numpy().astype(np.float64)}
    out["clocks"] = clk.summary()
    out["value"] = out["compensated"]["value"]
    # FP64 oracle trajectories and the CPU restatement (float pairs, double sums, all cores)
    from oracle import pyoracle as po
    orc = po.Restatement()
    x64, y64 = orc.advect(1, po.RM, x, y, r, s, fs, dt, K, fp64=True)
    disp = float(np.max(np.hypot(x64 - x, y64 - y)))
    for name in ("compensated", "plain"):
        ex = np.hypot(out[name].pop("final_x") - x64, out[name].pop("final_y") - y64)
        out[name]["position_error_max_over_displacement"] = float(ex.max() / disp)
    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    nat = po.Restatement(native=True)
    t0 = time.perf_counter()
    nat.advect(1, po.RM, x, y, r, s, fs, dt, K)
    tc = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": K * n * n / tc / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
                           "sample": "the full workload (10 Euler steps of 20k particles)"}
    return out


def run_bem2048(args):
    """Unit-diameter circle of 2048 panels and 200,000 particles uniform in the annulus
    0.55 < r < 3 (G ~ N(0, 1e-4)): particles-on-panels (RHS), the 4096 x 4096 panels-on-panels
    matrix in FP64, its FP64 GMRES solve (the FP64 LU timed beside it), and panels-on-particles
    velocity, all on the device.  Returns the result object."""
    torch, og, dev, ctx, stream, flush = _engine_setup()
    npan, npart = 2048, 200_000
    rng = np.random.default_rng(3)
    rad = np.sqrt(rng.uniform(0.55 ** 2, 3.0 ** 2, npart))
    th = rng.uniform(0.0, 2.0 * np.pi, npart)
    px, py = (rad * np.cos(th)).astype(np.float32), (rad * np.sin(th)).astype(np.float32)
    ps = rng.normal(0.0, 1e-2, npart).astype(np.float32)
    bd = og.circle_panels(npan)
    NX, NY = torch.from_numpy(bd.nx).to(dev), torch.from_numpy(bd.ny).to(dev)
    IDX = torch.from_numpy(bd.idx.astype(np.int32)).to(dev)
    PX, PY, PS = [torch.from_numpy(a).to(dev) for a in (px, py, ps)]
    nunk, m = 2, 2 * npan
    # velocities of each (u, v) pair in one array, zeroed by one fill per step
    PUV = torch.zeros(2, npan, device=dev)
    PU, PV = PUV[0], PUV[1]
    RHS = torch.zeros(m, dtype=torch.float64, device=dev)
    A = torch.zeros(m * m, dtype=torch.float64, device=dev)
    SOL = torch.zeros(m, dtype=torch.float64, device=dev)
    TUV = torch.zeros(2, npart, device=dev)
    TU, TV = TUV[0], TUV[1]
    # the solution's (vortex, source) strength pairs as two FP32 rows, one conversion per step
    STR = torch.zeros(2, npan, device=dev)
    acc = og.COMPENSATED
    box = {}

    def d3():
        PUV.zero_()
        og.points_affect_panels_dev(ctx, acc, PX, PY, PS, NX, NY, IDX, PU, PV, finalize=True)

    def b2():
        og.vels_to_rhs_panels_dev(ctx, nunk, NX, NY, IDX, PU, PV, None, None, RHS)

    def b1():
        og.panels_on_panels_coeff_dev(ctx, nunk, NX, NY, IDX, None, A)

    def solve():
        SOL.zero_()
        box["it"], box["rel"] = og.solve_gmres_f64_dev(ctx, A, RHS, SOL)

    def solve_lu():
        box["rel_lu"] = og.solve_dense_f64_dev(ctx, A, RHS, SOL)

    def d2():
        TUV.zero_()
        STR.copy_(SOL.view(npan, 2).t())
        og.panels_affect_points_dev(ctx, acc, NX, NY, IDX, STR[0], STR[1], PX, PY, TU, TV)

    def pipeline():
        d3(); b2(); b1(); solve(); d2()

    # clear_inner_layer of the same particles against the body (src/Reflect.h:491-760): every
    # particle is tested against every panel; those inside the layer are cropped
    CX, CY, CS = PX.clone(), PY.clone(), PS.clone()
    CR = torch.full((npart,), 0.01, device=dev)

    def clear_reset():
        CX.copy_(PX); CY.copy_(PY); CS.copy_(PS)

    def clear():
        box["clear"] = og.clear_inner_layer_dev(ctx, 0, og.CLEAR_CUTOFF, 0.01, NX, NY, IDX, CX, CY, CS, CR)

    # the literal 2048 x 2048 system: vortex strengths only (the nunk == 1 branch,
    # src/Coefficients.h:366-385)
    RHS1 = torch.zeros(npan, dtype=torch.float64, device=dev)
    A1 = torch.zeros(npan * npan, dtype=torch.float64, device=dev)
    SOL1 = torch.zeros(npan, dtype=torch.float64, device=dev)

    def solve1():
        SOL1.zero_()
        box["it1"], box["rel1"] = og.solve_gmres_f64_dev(ctx, A1, RHS1, SOL1)

    def pipeline1():
        d3()
        og.vels_to_rhs_panels_dev(ctx, 1, NX, NY, IDX, PU, PV, None, None, RHS1)
        og.panels_on_panels_coeff_dev(ctx, 1, NX, NY, IDX, None, A1)
        solve1()
        TUV.zero_()
        og.panels_affect_points_dev(ctx, acc, NX, NY, IDX, SOL1.float(), None, PX, PY, TU, TV)
    out = {"workload": "bem2048", "metric": "ms per BEM coupling step (2048 panels, 200k particles)",
           "unit": "ms", "higher_is_better": False, "data": "synthetic (seed 3)", "unknowns": m}
    with ClockSampler(0) as clk:
        times = {k: _event_time(torch, stream, flush, f, args.steps, args.warmup)
                 # the vortex-only system first: the checks below read the full system's outputs
                 for k, f in (("vortex_only_pipeline", pipeline1), ("vortex_only_gmres_f64", solve1),
                              ("points_affect_panels", d3), ("vels_to_rhs", b2), ("panels_on_panels_coeff_f64", b1),
                              ("lu_solve_f64", solve_lu), ("gmres_solve_f64", solve), ("panels_affect_points", d2),
                              ("pipeline", pipeline))}
        times["clear_inner_layer"] = _event_time(torch, stream, flush, clear, args.steps, args.warmup, prep=clear_reset)
    ctx.synchronize()
    out["clocks"] = clk.summary()
    out["ms"] = times
    out["value"] = times["pipeline"]
    out["ginter_s"] = {"points_affect_panels": npart * npan / (times["points_affect_panels"] * 1e-3) / 1e9,
                       "panels_affect_points": npart * npan / (times["panels_affect_points"] * 1e-3) / 1e9,
                       "clear_inner_layer_pairs": npart * npan / (times["clear_inner_layer"] * 1e-3) / 1e9,
                       "lu_tflops_f64": (2.0 / 3.0) * m ** 3 / (times["lu_solve_f64"] * 1e-3) / 1e12}
    # GMRES: one FP64 matrix-vector product per iteration reads the 4096^2 matrix from HBM
    out["gmres"] = {"iterations": box.get("it"), "relative_residual": box.get("rel"),
                    "matrix_gbs_per_iteration": (m * m * 8) * (box.get("it") or 1) / (times["gmres_solve_f64"] * 1e-3) / 1e9}
    out["vortex_only_2048"] = {"unknowns": npan, "pipeline_ms": times["vortex_only_pipeline"],
                               "gmres_ms": times["vortex_only_gmres_f64"], "iterations": box.get("it1"),
                               "relative_residual": box.get("rel1")}
    out["relative_residual"] = box.get("rel")
    out["lu_relative_residual"] = box.get("rel_lu")
    sol = SOL.cpu().numpy()
    tu, tv = TU.cpu().numpy(), TV.cpu().numpy()
    # FP64 oracle: the same five steps in FP64 (D2 on a 4096-particle subset)
    from oracle import pyoracle as po
    orc = po.Restatement()
    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    t0 = time.perf_counter()
    pu, pv = orc.points_affect_panels(px, py, ps, bd.nx, bd.ny, bd.idx, fp64=True)
    t_d3 = time.perf_counter() - t0
    pu, pv = pu / (2 * np.pi), pv / (2 * np.pi)
    rhs = orc.vels_to_rhs_panels(nunk, bd.nx, bd.ny, bd.idx, pu, pv, fp64=True)
    t0 = time.perf_counter()
    A64 = orc.panels_on_panels_coeff(nunk, bd.nx, bd.ny, bd.idx, fp64=True)
    t_b1 = time.perf_counter() - t0
    x64 = np.linalg.solve(A64, rhs)
    sub = np.random.default_rng(33).choice(npart, 4096, replace=False)
    u64, v64 = orc.panels_affect_points(bd.nx, bd.ny, bd.idx, x64[0::2], x64[1::2], px[sub], py[sub], fp64=True)
    vel = np.concatenate([u64, v64])
    out["precision"] = {"strengths_max_rel": float(np.max(np.abs(sol - x64)) / np.max(np.abs(x64))),
                        "panels_affect_points_subset_max_rel":
                            float(np.max(np.abs(np.concatenate([tu[sub], tv[sub]]) - vel)) / np.max(np.abs(vel)))}
    # clear_inner_layer: parity with the oracle on a 4096-particle sample, and its CPU time
    cres = box.get("clear")
    cx_, cy_, cs_ = CX.cpu().numpy(), CY.cpu().numpy(), CS.cpu().numpy()
    rs = np.full(sub.size, 0.01, np.float32)
    ox, oy, os_, _, _ = orc.clear_inner(0, og.CLEAR_CUTOFF, 0.01, bd.nx, bd.ny, bd.idx, px[sub], py[sub], ps[sub], rs)
    out["clear_inner_layer"] = {"particles": npart, "panels": npan, "ms": times["clear_inner_layer"],
                                "circulation_removed_and_modifications": cres,
                                "particles_moved": int(((cx_ != px) | (cy_ != py)).sum()),
                                "sample_equal_to_oracle": bool((ox == cx_[sub]).all() and (oy == cy_[sub]).all()
                                                               and (os_ == cs_[sub]).all())}
    nat = po.Restatement(native=True)
    t0 = time.perf_counter()
    nat.clear_inner(0, og.CLEAR_CUTOFF, 0.01, bd.nx, bd.ny, bd.idx, px[sub], py[sub], ps[sub], rs)
    t_cl = time.perf_counter() - t0
    out["cpu_baseline"] = {"kind": "port", "cores": threads,
                           "points_affect_panels_ginter_s": npart * npan / t_d3 / 1e9,
                           "panels_on_panels_coeff_ms": 1e3 * t_b1,
                           "clear_inner_layer_pairs_per_s": sub.size * npan / t_cl,
                           "sample": "FP64 restatement of the full particles-on-panels sum and matrix; "
                                     "clear_inner_layer on 4096 of the particles"}
    out["bodies4"] = run_bem_bodies(torch, og, dev, ctx, stream, flush, args, npan)
    return out


def run_bem_bodies(torch, og, dev, ctx, stream, flush, args, npan):
    """Four circles of `npan` panels, centres (+-1.5, +-1.5), joined into one system of
    8 npan unknowns: the joined matrix rebuilt in full (the engine's choice where the reference
    rebuilds only the blocks of bodies in relative motion, src/BEMHelper.h:147-221) against
    the FP64 GMRES solve of the same system, right-hand side A x for a seeded x."""
    bodies = [og.circle_panels(npan, center=c) for c in ((-1.5, -1.5), (1.5, -1.5), (-1.5, 1.5), (1.5, 1.5))]
    J, _ = og.join_surfaces(bodies)
    NX, NY = torch.from_numpy(J.nx).to(dev), torch.from_numpy(J.ny).to(dev)
    IDX = torch.from_numpy(J.idx.astype(np.int32)).to(dev)
    m = 2 * J.npan
    A = torch.zeros(m * m, dtype=torch.float64, device=dev)
    og.panels_on_panels_coeff_dev(ctx, 2, NX, NY, IDX, None, A)
    ctx.synchronize()
    xt = torch.from_numpy(np.random.default_rng(41).normal(size=m)).to(dev)
    rhs = A.view(m, m).t() @ xt            # A is column-major
    X = torch.zeros(m, dtype=torch.float64, device=dev)
    box = {}

    def build():
        og.panels_on_panels_coeff_dev(ctx, 2, NX, NY, IDX, None, A)

    def solve():
        X.zero_()
        box["it"], box["rel"] = og.solve_gmres_f64_dev(ctx, A, rhs, X)

    t_build = _event_time(torch, stream, flush, build, args.steps, args.warmup)
    t_solve = _event_time(torch, stream, flush, solve, args.steps, args.warmup)
    err = float((X - xt).abs().max() / xt.abs().max())
    return {"bodies": 4, "panels": J.npan, "unknowns": m, "matrix_gb": m * m * 8 / 1e9,
            "matrix_ms": t_build, "gmres_ms": t_solve, "gmres_iterations": box.get("it"),
            "relative_residual": box.get("rel"), "solution_max_rel_error": err,
            "matrix_share": t_build / (t_build + t_solve)}


def two_patches(n, seed=5):
    """Two co-rotating Gaussian patches (sigma 0.1, centres (+-0.3, 0), total circulation 1
    each; particles alternate between the patches), core 0.004."""
    rng = np.random.default_rng(seed)
    lab = (np.arange(n) % 2).astype(np.int64)
    cx = np.where(lab == 0, -0.3, 0.3)
    x = cx + rng.normal(0.0, 0.1, n)
    y = rng.normal(0.0, 0.1, n)
    w = np.exp(-((x - cx) ** 2 + y ** 2) / (2 * 0.1 ** 2))
    s = np.where(lab == 0, w / w[lab == 0].sum(), w / w[lab == 1].sum())
    x, y, s = x.astype(np.float32), y.astype(np.float32), s.astype(np.float32)
    return x, y, np.full(n, 0.004, np.float32), s, lab


def centroid_loss_seed(xT, yT, s, lab):
    """L = |X_A - X_B|^2 with X_P = sum_P G^2 x / sum_P G^2, in FP64 on the host; returns L,
    dL/d(final x), dL/d(final y) and the direct part of dL/dG (through the weights)."""
    n = xT.size
    s64 = s.astype(np.float64)
    gxT, gyT, gs_direct = np.zeros(n), np.zeros(n), np.zeros(n)
    cen = []
    for P in (0, 1):
        m = lab == P
        w2 = s64[m] ** 2
        cen.append((np.sum(w2 * xT[m]) / w2.sum(), np.sum(w2 * yT[m]) / w2.sum(), w2.sum()))
    dX, dY = cen[0][0] - cen[1][0], cen[0][1] - cen[1][1]
    for P, sg in ((0, 1.0), (1, -1.0)):
        m = lab == P
        W = cen[P][2]
        gxT[m] = sg * 2 * dX * s64[m] ** 2 / W
        gyT[m] = sg * 2 * dY * s64[m] ** 2 / W
        gs_direct[m] = sg * 2 * (dX * (xT[m] - cen[P][0]) + dY * (yT[m] - cen[P][1])) * 2 * s64[m] / W
    return dX * dX + dY * dY, gxT, gyT, gs_direct


def rk2_adjoint(og, torch, dev, ctx, stream, x, y, r, s, lab, K, every, dt=0.005):
    """Forward: K Ralston RK2 steps recording checkpoints every `every` steps; backward: the
    gradient of the centroid loss with respect to the initial strengths through the trajectory
    from those checkpoints.  CUDA events on the launching stream; returns (forward ms, backward
    ms, L, dL/dG, engine buffer bytes)."""
    X, Y, R, S = [torch.from_numpy(a).to(dev) for a in (x, y, r, s)]
    GS = torch.zeros(x.size, device=dev)
    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    torch.cuda.synchronize()
    e[0].record(stream)
    og.advect_record_dev(ctx, og.CORE_GAUSSIAN, og.COMPENSATED, 2, X, Y, R, S, (0.0, 0.0), dt, K, every)
    e[1].record(stream)
    e[1].synchronize()
    # loss and its seed on the host in FP64 (the loss is not part of the engine)
    L, gxT, gyT, gs_direct = centroid_loss_seed(X.cpu().numpy().astype(np.float64),
                                                Y.cpu().numpy().astype(np.float64), s, lab)
    LX = torch.from_numpy(gxT.astype(np.float32)).to(dev)
    LY = torch.from_numpy(gyT.astype(np.float32)).to(dev)
    torch.cuda.synchronize()
    e[2].record(stream)
    peak = og.advect_vjp_tape_dev(ctx, LX, LY, GS, None, None)
    e[3].record(stream)
    e[3].synchronize()
    ctx.synchronize()
    gs = GS.cpu().numpy().astype(np.float64) + gs_direct
    return e[0].elapsed_time(e[1]), e[2].elapsed_time(e[3]), L, gs, peak


def run_rk2adjoint2M(args, K=None, every=None):
    """Two co-rotating Gaussian patches of 1M particles each (sigma 0.1, centres (+-0.3, 0),
    total circulation 1 each), core 0.004, Gaussian; K Ralston RK2 steps with dt = 0.005; loss
    L = |X_A - X_B|^2 with X_P = sum_P G^2 x / sum_P G^2; gradient of L with respect to the
    initial strengths through the trajectory, checkpoints every 8 steps (`every` -1: every
    step's positions and stage positions kept in HBM, so the backward recomputes nothing).
    Beside it: the same engine path on a 4096-particle draw of the same patches against the FP64
    oracle's trajectory gradient, and the CPU port's velocity sum and FP64 self-VJP.  Returns
    the result object."""
    torch, og, dev, ctx, stream, flush = _engine_setup()
    n, dt = 2_000_000, 0.005
    K = args.rk_steps if K is None else K
    every = args.checkpoint_every if every is None else every
    x, y, r, s, lab = two_patches(n)
    torch.cuda.reset_peak_memory_stats(dev)
    with ClockSampler(0) as clk:
        rk2_adjoint(og, torch, dev, ctx, stream, x, y, r, s, lab, 1, every, dt)      # warm-up
        f_ms, b_ms, L, gs, peak = rk2_adjoint(og, torch, dev, ctx, stream, x, y, r, s, lab, K, every, dt)
    clocks = clk.summary()
    evals = 2.0 * K * float(n) * float(n)
    nck = 1 if every == og.TAPE_ALL else -(-K // max(1, every))
    recomputed = 0 if every == og.TAPE_ALL else (nck - 1) * (2 * min(every, K) - 1)
    out = {"workload": "rk2adjoint2M", "metric": "Ginteractions/s forward and adjoint, 2M particles, RK2",
           "unit": UNIT, "data": "synthetic (seed 5)", "n": n, "rk2_steps": K, "dt": dt, "checkpoint_every": every,
           "forward_ms": f_ms, "forward_ginter_s": evals / (f_ms * 1e-3) / 1e9,
           "adjoint_ms": b_ms, "adjoint_ginter_s": evals / (b_ms * 1e-3) / 1e9, "adjoint_over_forward": b_ms / f_ms,
           "adjoint_work": {"self_vjp_gathers": 2 * K, "recomputed_velocity_sums": recomputed,
                            "forward_velocity_sums": 2 * K,
                            "note": "the recorded forward keeps the last segment's stage positions; every other "
                                    "segment is recomputed from its checkpoint (its last step needs one sum)"},
           "value": evals / (f_ms * 1e-3) / 1e9, "loss": L, "grad_strength_norm": float(np.linalg.norm(gs)),
           "grad_strength_finite": bool(np.isfinite(gs).all()),
           "peak_hbm_bytes": {"engine": int(peak), "caller_tensors": int(torch.cuda.max_memory_allocated(dev))},
           "clocks": clocks}
    # precision: the same engine path on a 4096-particle draw of the patches vs the FP64 oracle
    from oracle import pyoracle as po
    orc = po.Restatement()
    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    m = 4096
    xs, ys, rs, ss, ls = two_patches(m, seed=55)
    _, _, Ls, gss, _ = rk2_adjoint(og, torch, dev, ctx, stream, xs, ys, rs, ss, ls, K, every, dt)
    Lr, gs_ref, _, _ = orc.rk2_centroid_grad(po.GAUSS, xs, ys, rs, ss, ls, (0.0, 0.0), dt, K)
    mx, rms = rel_errs(gs_ref, gss)
    out["precision"] = {"sample": f"{m} particles of the same two patches, {K} steps, checkpoints every {every}",
                        "loss_rel": abs(Ls - Lr) / abs(Lr), "dL/dG_max_rel": mx, "dL/dG_rms_rel": rms}
    # CPU: the port's velocity sum on a target sample of the 2M set, the FP64 self VJP on 4096
    sub = np.random.default_rng(97).choice(n, 512, replace=False)
    nat = po.Restatement(native=True)
    t0 = time.perf_counter()
    nat.points_affect_points(po.GAUSS, po.VELONLY, x, y, r, s, x[sub], y[sub], r[sub])
    tf = time.perf_counter() - t0
    lu, lv = np.random.default_rng(98).normal(size=(2, m))
    t0 = time.perf_counter()
    orc.self_vjp(po.GAUSS, xs, ys, rs, ss, lu, lv)
    tb = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": 512.0 * n / tf / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
                           "sample": f"velocity sum, 512 seeded targets x {n} sources (float pairs, double sums)",
                           "adjoint_value": float(m) * m / tb / 1e9,
                           "adjoint_sample": f"FP64 self-interaction VJP of {m} particles"}
    return out


def run_rows(args):
    """Every row of the hot-path scope on its own: device time (CUDA events, L2 flushed), the
    interactions per second, the achieved FLOP/s at the reference's flop count per interaction
    and its fraction of the FP32 peak (HBM peak for the GMRES matrix-vector products), and the
    C restatement (float pairs, double sums, all host cores) on a target sample beside it."""
    torch, og, dev, ctx, stream, flush = _engine_setup()
    from oracle import pyoracle as po
    orc = po.Restatement(native=True)          # timed only: the Release-flag build
    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    peaks = measured_peaks()
    sm_max = peaks.get("sm_max_mhz") or 2070.0
    nsm = torch.cuda.get_device_properties(dev).multi_processor_count
    fp32_peak = 2.0 * FMA_PER_CLK_PER_SM * nsm * sm_max * 1e6
    hbm_peak = float(peaks.get("hbm_gbs") or 6800.0) * 1e9
    n = 131072
    x, y, r, s = make_workload(7, n)
    T = {k: torch.from_numpy(v).to(dev) for k, v in dict(x=x, y=y, r=r, s=s).items()}
    U, V = torch.zeros(n, device=dev), torch.zeros(n, device=dev)
    E = [torch.zeros(n, device=dev) for _ in range(4)]
    rows = []

    def cpu_rate(fn, pairs):
        t0 = time.perf_counter()
        fn()
        return pairs / (time.perf_counter() - t0) / 1e9

    def row(name, ref, fn, pairs, flops_per, cpu=None, bound="fp32", bytes_per_call=None):
        ms = _event_time(torch, stream, flush, fn, args.steps, 1)
        d = {"row": name, "reference": ref, "ms": round(ms, 4), "ginter_s": round(pairs / (ms * 1e-3) / 1e9, 1)}
        if flops_per:
            tf = pairs * flops_per / (ms * 1e-3)
            d.update(flops_per_interaction=flops_per, tflops=round(tf / 1e12, 2), frac_fp32=round(tf / fp32_peak, 3))
        if bytes_per_call:
            bw = bytes_per_call / (ms * 1e-3)
            d.update(gb_s=round(bw / 1e9, 1), frac_hbm=round(bw / hbm_peak, 3))
        if cpu:
            d["cpu_ginter_s"] = round(cpu, 3)
        rows.append(d)

    sub = np.random.default_rng(8).choice(n, 256, replace=False)
    acc = og.COMPENSATED
    cores = {"K1/C1 RM": og.CORE_RM, "K1/C2 Gaussian": og.CORE_GAUSSIAN, "K1/C3 Vatistas-2": og.CORE_V2,
             "K1/C4 Winckelmans-Leonard": og.CORE_WL, "K1/C4 Vatistas-3": og.CORE_V3,
             "K1/C5 singular": og.CORE_SINGULAR, "K1/C6 compact exponential": og.CORE_COMPACT_EXP}
    for name, core in cores.items():
        def f(core=core):
            U.zero_(); V.zero_()
            og.points_affect_points_dev(ctx, core, og.VELONLY, acc, T["x"], T["y"], T["r"], T["s"], T["x"], T["y"],
                                        T["r"], U, V)
        cpu = cpu_rate(lambda core=core: orc.points_affect_points(core, 1, x, y, r, s, x[sub], y[sub], r[sub]),
                       256 * n)
        fp = og.flops_per_pair(core, og.VELONLY, True)
        row(name + " (0v_0b velocity)", "src/Kernels.h:81-92, src/CoreFunc.h", f, float(n) * n, fp if fp > 0 else None,
            cpu)

    def fp_(g=og.CORE_GAUSSIAN, res=og.VELONLY, thick=True):
        v = og.flops_per_pair(g, res, thick)
        return v if v > 0 else None

    def p2p(res, thick, extra):
        def f():
            U.zero_(); V.zero_()
            for e in E:
                e.zero_()
            og.points_affect_points_dev(ctx, og.CORE_GAUSSIAN, res, acc, T["x"], T["y"], T["r"], T["s"], T["x"],
                                        T["y"], T["r"] if thick else None, U, V, extra=E[:extra])
        return f
    for name, ref, res, thick, extra in (
            ("K2 Gaussian field points (0v_0p)", "src/Kernels.h:95-106", og.VELONLY, False, 0),
            ("K3 velocity + gradient", "src/Kernels.h:112-133", og.VELANDGRAD, True, 4),
            ("K4 velocity + vorticity", "src/Kernels.h:139-179", og.VELANDVORT, True, 1),
            ("K4 velocity + shear rate", "src/Kernels.h:185-231", og.VELANDSHEAR, True, 1),
            ("K5 streamfunction", "src/Kernels.h:52-74", og.PSIONLY, True, 1)):
        cpu = cpu_rate(lambda res=res, thick=thick: orc.points_affect_points(
            og.CORE_GAUSSIAN, res, x, y, r, s, x[sub], y[sub], r[sub] if thick else None), 256 * n)
        row(name, ref, p2p(res, thick, extra), float(n) * n, fp_(res=res, thick=thick), cpu)

    def vort():
        E[0].zero_()
        og.points_affect_points_vorticity_dev(ctx, acc, T["x"], T["y"], T["r"], T["s"], T["x"], T["y"], E[0])
    row("D5 blob vorticity", "src/InfluenceVort.h:47-126", vort, float(n) * n, 13,
        cpu_rate(lambda: orc.points_affect_points_vorticity(x, y, r, s, x[sub], y[sub]), 256 * n))

    # panels: unit circle of 2048 panels, 200,000 points in the annulus
    npan, npt = 2048, 200_000
    rng = np.random.default_rng(3)
    rad = np.sqrt(rng.uniform(0.55 ** 2, 9.0, npt))
    th = rng.uniform(0, 2 * np.pi, npt)
    px, py = (rad * np.cos(th)).astype(np.float32), (rad * np.sin(th)).astype(np.float32)
    pg = rng.normal(0, 1e-2, npt).astype(np.float32)
    bd = og.circle_panels(npan)
    vsh = rng.normal(0, 1, npan).astype(np.float32)
    ssh = rng.normal(0, 1, npan).astype(np.float32)
    P = {k: torch.from_numpy(v).to(dev) for k, v in dict(px=px, py=py, pg=pg, nx=bd.nx, ny=bd.ny, vs=vsh, ss=ssh).items()}
    IDX = torch.from_numpy(bd.idx.astype(np.int32)).to(dev)
    PU, PV = torch.zeros(npt, device=dev), torch.zeros(npt, device=dev)
    QU, QV = torch.zeros(npan, device=dev), torch.zeros(npan, device=dev)
    psub = np.random.default_rng(9).choice(npt, 4096, replace=False)

    def d2():
        PU.zero_(); PV.zero_()
        og.panels_affect_points_dev(ctx, acc, P["nx"], P["ny"], IDX, P["vs"], P["ss"], P["px"], P["py"], PU, PV)
    row("D2 panels on points (1vs)", "src/Influence.h:422-614", d2, float(npan) * npt, 47,
        cpu_rate(lambda: orc.panels_affect_points(bd.nx, bd.ny, bd.idx, vsh, ssh, px[psub], py[psub]), npan * 4096.0))

    def d3():
        QU.zero_(); QV.zero_()
        og.points_affect_panels_dev(ctx, acc, P["px"], P["py"], P["pg"], P["nx"], P["ny"], IDX, QU, QV)
    row("D3 points on panels (reversed 1v)", "src/Influence.h:633-771", d3, float(npan) * npt, 39,
        cpu_rate(lambda: orc.points_affect_panels(px[psub], py[psub], pg[psub], bd.nx, bd.ny, bd.idx), npan * 4096.0))

    def d4():
        QU.zero_(); QV.zero_()
        og.panels_affect_panels_dev(ctx, acc, P["nx"], P["ny"], IDX, P["vs"], P["ss"], P["nx"], P["ny"], IDX, QU, QV)
    row("D4 panels on panels", "src/Influence.h:774-795", d4, float(npan) * npan, 47,
        cpu_rate(lambda: orc.panels_affect_panels(bd.nx, bd.ny, bd.idx, vsh, ssh, bd.nx, bd.ny, bd.idx),
                 float(npan) * npan))
    m = 2 * npan
    A = torch.zeros(m * m, dtype=torch.float64, device=dev)

    def b1():
        og.panels_on_panels_coeff_dev(ctx, 2, P["nx"], P["ny"], IDX, None, A)
    row("B1 panels-on-panels matrix (two-way, 1vos)", "src/Coefficients.h:155-427", b1, 2.0 * npan * npan, 45,
        cpu_rate(lambda: orc.panels_on_panels_coeff(2, bd.nx, bd.ny, bd.idx), 2.0 * npan * npan))
    RHS = torch.from_numpy(np.random.default_rng(10).normal(size=m)).to(dev)
    SOL = torch.zeros(m, dtype=torch.float64, device=dev)
    it_box = {}

    def b3():
        SOL.zero_()
        it_box["it"], it_box["rel"] = og.solve_gmres_f64_dev(ctx, A, RHS, SOL)
    b1()
    _event_time(torch, stream, flush, b3, 1, 1)
    row("B3 FP64 GMRES solve (4096 unknowns)", "src/BEM.h:169-234", b3, float(m) * m * (it_box["it"] or 1), None,
        None, bytes_per_call=8.0 * m * m * (it_box["it"] or 1))
    rows[-1]["iterations"] = it_box["it"]
    rows[-1]["relative_residual"] = it_box["rel"]

    # clear_inner_layer over the same points and panels: the annulus starts outside the layer,
    # so each point is tested once against every panel (the usual case in a run)
    PRc = torch.full((npt,), 0.01, device=dev)
    PXc, PYc, PSc = P["px"].clone(), P["py"].clone(), P["pg"].clone()
    rsub = np.full(psub.size, 0.01, np.float32)

    def clr():
        PXc.copy_(P["px"]); PYc.copy_(P["py"]); PSc.copy_(P["pg"])
        og.clear_inner_layer_dev(ctx, 0, og.CLEAR_CUTOFF, 0.01, P["nx"], P["ny"], IDX, PXc, PYc, PSc, PRc)
    row("clear_inner_layer (crop test of every point)", "src/Reflect.h:491-760", clr, float(npan) * npt, None,
        cpu_rate(lambda: orc.clear_inner(0, og.CLEAR_CUTOFF, 0.01, bd.nx, bd.ny, bd.idx, px[psub], py[psub],
                                         pg[psub], rsub), npan * float(psub.size)))

    # time stepping: one step of each scheme on the 131072-particle patch
    for order, name in ((1, "E3 Euler step"), (2, "E3 Ralston RK2 step"), (3, "E3 RK3 step"), (4, "E3 Heun RK2 step")):
        X2, Y2 = T["x"].clone(), T["y"].clone()

        def stepf(order=order, X2=X2, Y2=Y2):
            og.advect_dev(ctx, og.CORE_GAUSSIAN, acc, order, X2, Y2, T["r"], T["s"], (0.0, 0.0), 1e-4, 1)
        stages = {1: 1, 2: 2, 3: 3, 4: 2}[order]
        row(name, "src/Convection.h:274-598", stepf, stages * float(n) * n, fp_())

    # reverse mode
    LU, LV = [torch.from_numpy(a).to(dev) for a in np.random.default_rng(11).normal(size=(2, n)).astype(np.float32)]
    G = [torch.zeros(n, device=dev) for _ in range(3)]

    def vjp_self():
        for g in G:
            g.zero_()
        og.points_affect_points_vjp_self_dev(ctx, og.CORE_GAUSSIAN, acc, T["x"], T["y"], T["r"], T["s"], LU, LV, *G)
    row("adjoint: self-interaction VJP", "(no reference counterpart)", vjp_self, float(n) * n, None,
        cpu_rate(lambda: orc.self_vjp(po.GAUSS, x[:4096], y[:4096], r[:4096], s[:4096], LU.cpu().numpy()[:4096],
                                      LV.cpu().numpy()[:4096]), 4096.0 * 4096))
    rows[-1]["cpu_note"] = "FP64 reference adjoint, 4096 particles"

    def vjp_src():
        for g in G:
            g.zero_()
        og.points_affect_points_vjp_dev(ctx, og.CORE_GAUSSIAN, acc, T["x"], T["y"], T["r"], T["s"], T["x"][:16384],
                                        T["y"][:16384], None, LU[:16384], LV[:16384], *G)
    row("adjoint: source-side VJP (16384 probes)", "(no reference counterpart)", vjp_src, float(n) * 16384, None)
    ctx.synchronize()
    out = {"workload": "rows", "metric": "per-row device throughput", "n_particles": n, "panels": npan,
           "panel_points": npt, "fp32_peak_tflops": fp32_peak / 1e12, "hbm_peak_gbs": hbm_peak / 1e9,
           "cpu_cores": threads, "rows": rows}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--cpu-sample", type=int, default=2048)
    ap.add_argument("--n", type=int, default=N, help="particles (the headline workload is 1,000,000)")
    ap.add_argument("--workload", default="patch1M", choices=["patch1M", "euler20k", "bem2048", "rk2adjoint2M", "rows"],
                    help="patch1M is the headline line; the others measure the remaining configurations")
    ap.add_argument("--rk-steps", type=int, default=64, help="RK2 steps of --workload rk2adjoint2M")
    ap.add_argument("--line-rk-steps", type=int, default=16,
                    help="RK2 steps of the rk2adjoint object in the default line (two checkpoint segments)")
    ap.add_argument("--no-configs", action="store_true",
                    help="the headline line only, without the euler20k, bem2048 and rk2adjoint objects")
    ap.add_argument("--checkpoint-every", type=int, default=8,
                    help="rk2adjoint2M checkpoint interval; -1 keeps the whole trajectory (no recompute)")
    args = ap.parse_args()
    globals()["N"] = args.n
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "euler20k":
        print(json.dumps(run_euler20k(args)), flush=True)
    elif args.workload == "bem2048":
        print(json.dumps(run_bem2048(args)), flush=True)
    elif args.workload == "rk2adjoint2M":
        print(json.dumps(run_rk2adjoint2M(args)), flush=True)
    elif args.workload == "rows":
        run_rows(args)
    else:
        run_engine(args)


if __name__ == "__main__":
    main()
