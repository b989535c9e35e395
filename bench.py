"""Benchmark of the GB300 hybrid dealiased convolution.

Default workload (the configuration the headline metric is quoted on):
2D centred-Hermitian binary convolution, input 1023 x 512 complex128 modes
(Lx = Ly = 1023, Hermitian y storing ceil(Ly/2) = 512 modes), 3/2-rule
padding Mx = My = 1534, FP64 -- the reference's
HybridConvolutionHermitian2 / fftwpp_hconv2d path
(wrappers/HybridConvolution.h:80-111).  Inputs iid U[-1,1] from a seed, then
Hermitian-symmetrised (HermitianSymmetrizeX) with a real origin.

A step is one convolution.  `value` = device-timed convolutions/s with
inputs resident in HBM (L2 flushed before every timed step, the flush
outside the timed events); `e2e` = the same metric through the reference's
C ABI (fftwpp_hconv2d_convolve) on page-locked host buffers, host<->device
copies inside the timed call.  Multi-GPU: independent replicas, one per
rank (the single convolution does not shard without an all-to-all, which is
out of scope); value = all ranks' convolutions / max-over-ranks time.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload hconv2d|conv1d|real3d|batched1d|jacobian2d]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("dealiased convs/s + % of HBM roofline; FP32-comp vs FP64 at "
          "≤2e-6 rel L2 err")

PAD, CENTERED, HERMITIAN, REAL = 0, 1, 2, 3

WORKLOADS = {
    "hconv2d": dict(
        kinds=[CENTERED, HERMITIAN], L=[1023, 1023], M=[1534, 1534],
        mult="realbinary", A=2, B=1,
        desc="2D centred-Hermitian binary convolution, 1023x512 complex128 "
             "modes (Lx=Ly=1023), Mx=My=1534 (3/2 rule)"),
    "conv1d": dict(
        kinds=[PAD], L=[1024], M=[2047], mult="binary", A=2, B=1, batch=4096,
        desc="1D complex binary convolution L=1024, M=2047, 4096 independent "
             "pairs per step"),
    "real3d": dict(
        kinds=[REAL, PAD, PAD], L=[256, 256, 256], M=[511, 511, 511],
        mult="binary", A=2, B=1,
        desc="3D real convolution 256^3 float64, M=511 per axis"),
    "jacobian2d": dict(
        kinds=[CENTERED, HERMITIAN], L=[1023, 1023], M=[1534, 1534],
        mult="realjacobian", A=4, B=1,
        desc="2D advection Jacobian, 4 centred-Hermitian inputs 1023x512, "
             "2/3 rule (M=1534)"),
}


def algorithmic_bytes(w, elem):
    """Compulsory HBM traffic of one convolution: A inputs read + B outputs
    written at their stored size."""
    n = 1
    for k, l in zip(w["kinds"], w["L"]):
        n *= (l + 1) // 2 if k == HERMITIAN else l
    n *= w.get("batch", 1)
    return (w["A"] + w["B"]) * elem * n


def spot_check(fs, got, w, n=12, seed=9):
    """Relative L2 error of `got` at n sampled output points against FP64
    direct sums h[i,j,k] = sum f[a,b,c] g[i-a,j-b,k-c] (tests/direct.h:
    118-133), for the real/complex 3D workloads whose full oracle would not
    fit a CPU time budget."""
    rng = np.random.default_rng(seed)
    f, g = fs[0], fs[1]
    num = den = 0.0
    for _ in range(n):
        idx = tuple(int(rng.integers(s // 2, s)) for s in f.shape)
        sl = tuple(slice(0, i + 1) for i in idx)
        rev = tuple(slice(i, None, -1) if i > 0 else slice(0, 1) for i in idx)
        val = np.sum(f[sl] * g[rev])
        num += abs(got[idx] - val) ** 2
        den += abs(val) ** 2
    return float(np.sqrt(num / den))


def synth_inputs(w, seed=1):
    """Seeded inputs with the workload's shapes and distributions."""
    rng = np.random.default_rng(seed)
    kinds, L = w["kinds"], w["L"]
    shape = [(l + 1) // 2 if k == HERMITIAN else l for k, l in zip(kinds, L)]
    if w.get("batch", 1) > 1:
        shape = [w["batch"]] + shape
    out = []
    for _ in range(w["A"]):
        if kinds[0] == REAL:
            f = rng.normal(size=shape)
        else:
            f = rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)
        if kinds[-1] == HERMITIAN and len(kinds) == 2:
            Lx, Hy = L[0], shape[-1]
            Hx, x0 = (Lx + 1) // 2, Lx // 2
            for i in range(1, Hx):
                f[x0 - i, 0] = np.conj(f[x0 + i, 0])
            f[x0, 0] = f[x0, 0].real
            if x0 == Hx:
                f[0, :] = 0
        out.append(np.ascontiguousarray(f))
    return out


# ---------------------------------------------------------------------------
# Clock sampling during the timed region.

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,"
              "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}",
                 f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------

def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_oracle_rate(w, budget_s, max_convs, workers):
    """Time the CPU restatement (oracle/hybrid.py, scipy.fft with `workers`
    threads) on a bounded sample of the workload; returns (convs/s, n)."""
    from oracle import hybrid as H
    fs = synth_inputs(w, seed=7)
    batch = w.get("batch", 1)
    if batch > 1:
        fs = [f[0] for f in fs]
    n, t0 = 0, time.perf_counter()
    while n < max_convs:
        H.convolve(fs, w["kinds"], w["L"], w["M"], mult=w["mult"],
                   workers=workers)
        n += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return n * 1.0 / dt, n, dt


def profile_figure(tag, workload, kernel, precision):
    """A per-launch figure from a committed ncu summary line
    `<tag> <workload> <precision> <kernel> <value>` under profiles/
    (TRAFFIC: DRAM bytes; DPINST: FP64 instructions)."""
    pdir = os.path.join(ROOT, "profiles")
    if not os.path.isdir(pdir):
        return None
    for fn in sorted(os.listdir(pdir)):
        if not fn.endswith((".md", ".txt")):
            continue
        for line in open(os.path.join(pdir, fn)):
            parts = line.strip().strip("`").split()
            if (len(parts) == 5 and parts[0] == tag and
                    parts[1] == workload and parts[2] == precision and
                    parts[3] == kernel):
                return float(parts[4])
    return None


def traffic_from_profiles(workload, kernel, precision):
    return profile_figure("TRAFFIC", workload, kernel, precision)


def measured_fma_rates():
    """(DFMA/s, FFMA/s) measured on this GPU by the library's probes."""
    import ctypes
    from fftwpp_gb300 import _native
    d, f = ctypes.c_double(), ctypes.c_double()
    if _native.load().fgb_measure_fma_rate(ctypes.byref(d), ctypes.byref(f)):
        return None, None
    return d.value, f.value


def run_reference(args, w):
    """--impl reference: the reference's CPU algorithm (the oracle port;
    the compiled reference cannot travel to the GPU host) on the host cores."""
    world, rank, _ = dist_setup()
    if rank != 0:
        return 0
    workers = os.cpu_count() or 1
    from oracle import hybrid as H
    fs = synth_inputs(w, seed=7)
    if w.get("batch", 1) > 1:
        fs = [f[0] for f in fs]
    for _ in range(args.warmup):
        H.convolve(fs, w["kinds"], w["L"], w["M"], mult=w["mult"],
                   workers=workers)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        H.convolve(fs, w["kinds"], w["L"], w["M"], mult=w["mult"],
                   workers=workers)
    dt = time.perf_counter() - t0
    value = args.steps / dt
    sample = (f"{args.steps} timed single convolutions of the workload "
              f"(numpy/scipy.fft restatement of FFTW++'s hybrid convolution, "
              f"scipy workers={workers})")
    line = {
        "impl": "reference", "metric": METRIC, "value": value,
        "unit": "convs/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": w["desc"], "parallelism": "cpu"},
        "cpu_baseline": {"value": value, "unit": "convs/s", "cores": workers,
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "convs/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def time_device(conv, ts, steps, warmup, flush, timing=True):
    """Per-step CUDA-event timing on the current stream; returns total ms."""
    import torch
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        conv.convolve(*ts)
    torch.cuda.synchronize()
    if timing:
        conv.enable_timing(True)
    total = 0.0
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    outs = [torch.empty_like(ts[0]) for _ in range(conv.B)]
    for _ in range(steps):
        flush.zero_()
        start.record(stream)
        conv.convolve(*ts, out=outs)
        stop.record(stream)
        stop.synchronize()
        total += start.elapsed_time(stop)
        if timing:
            conv.collect_timing()
    if timing:
        conv.enable_timing(False)
    return total, outs


def run_ours(args, w):
    import torch
    world, rank, local = dist_setup()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    from fftwpp_gb300 import _native
    from fftwpp_gb300.gpu import HybridConvolution

    prec = args.precision
    fs = synth_inputs(w, seed=1)
    conv = HybridConvolution(w["kinds"], w["L"], w["M"], A=w["A"], B=w["B"],
                             mult=w["mult"], precision=prec,
                             batch=w.get("batch", 1))
    ts = [torch.from_numpy(f).to(conv.dtype).cuda() for f in fs]
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")

    clocks = ClockSampler(local) if rank == 0 else None
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    if clocks:
        clocks.start()
    total_ms, outs = time_device(conv, ts, args.steps, args.warmup, flush)
    clk = clocks.stop() if clocks else None
    if world > 1:
        t = torch.tensor([total_ms], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
        torch.distributed.barrier()
    value = world * args.steps / (total_ms * 1e-3)

    names = conv.launch_names()
    kms = conv.kernel_ms()
    per_launch = [k / args.steps for k in kms]
    dom = int(np.argmax(per_launch))
    elem = (8 if conv.real else 16) if prec == "f64" else (4 if conv.real else 8)
    abytes = algorithmic_bytes(w, elem)

    if rank != 0:
        torch.distributed.destroy_process_group()
        return 0

    peaks = {}
    pfile = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pfile):
        peaks = json.load(open(pfile))
    peak = peaks.get("hbm_gbs")
    peak_src = "measured"
    if not peak:
        peak, peak_src = 6800.0, "fallback"
    if per_launch[dom] <= 0:
        raise RuntimeError("per-kernel timing recorded nothing")
    achieved = abytes / (per_launch[dom] * 1e-3) / 1e9
    traffic = traffic_from_profiles(args.workload, names[dom], prec)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                "kernel": names[dom], "peak_source": peak_src,
                "algorithmic_bytes_per_launch": abytes,
                "whole_step_frac": abytes / (total_ms / args.steps * 1e-3)
                / 1e9 / peak}

    # Compute roofline of the FP64 kernels: FP64 instructions per launch
    # (ncu, committed under profiles/) over the live launch time, against
    # the DFMA issue rate measured on this GPU.
    compute = None
    dfma, ffma = measured_fma_rates()
    if prec == "f64" and dfma:
        dp = [profile_figure("DPINST", args.workload, n, prec) for n in names]
        if dp[dom]:
            total_dp = sum(x for x in dp if x) if all(dp) else None
            compute = {
                "bound": "fp64_issue", "kernel": names[dom],
                "achieved": dp[dom] / (per_launch[dom] * 1e-3),
                "peak": dfma, "unit": "FP64 inst/s",
                "frac": dp[dom] / (per_launch[dom] * 1e-3) / dfma,
                "whole_step_frac": (total_dp / (total_ms / args.steps * 1e-3)
                                    / dfma) if total_dp else None,
                "fp64_tflops_peak_measured": 2 * dfma / 1e12,
                "fp32_tflops_peak_measured": 2 * ffma / 1e12,
                "source": "DP instructions per launch from ncu "
                          "(profiles/), peak from fgb_measure_fma_rate"}
    elif dfma:
        compute = {"fp64_tflops_peak_measured": 2 * dfma / 1e12,
                   "fp32_tflops_peak_measured": 2 * ffma / 1e12}

    # Accuracy at full size against the CPU oracle (FP64 restatement), or,
    # for the 256^3 workload, against FP64 direct sums at sampled outputs.
    from oracle import hybrid as H
    from oracle.direct import rel_l2
    big = np.prod([l for l in w["L"]]) > 5e6
    want = None
    if w.get("batch", 1) == 1 and not big:
        want = H.convolve(fs, w["kinds"], w["L"], w["M"], mult=w["mult"],
                          workers=os.cpu_count() or 1)[0]
    got0 = outs[0].cpu().numpy()
    if want is not None:
        err = rel_l2(got0, want)
    elif big:
        err = spot_check(fs, got0, w, n=12)
    else:
        err = None

    extra = {}
    if not args.quick and prec == "f64":
        # FP32 compensated mode on the same workload.
        c32 = HybridConvolution(w["kinds"], w["L"], w["M"], A=w["A"], B=w["B"],
                                mult=w["mult"], precision="f32",
                                batch=w.get("batch", 1))
        t32 = [torch.from_numpy(f).to(c32.dtype).cuda() for f in fs]
        ms32, o32 = time_device(c32, t32, args.steps, args.warmup, flush,
                                timing=False)
        if want is not None:
            e32 = rel_l2(o32[0].cpu().numpy(), want)
        elif big:
            e32 = spot_check(fs, o32[0].cpu().numpy().astype(got0.dtype), w,
                             n=12)
        else:
            e32 = None
        extra["fp32_compensated"] = {"value": args.steps / (ms32 * 1e-3),
                                     "unit": "convs/s",
                                     "rel_l2_vs_fp64_oracle": e32,
                                     "speedup_vs_fp64": (args.steps / ms32) /
                                     (args.steps / total_ms)}

    # End to end through the reference-facing C ABI on host buffers.
    e2e = None
    if args.workload == "hconv2d" and prec == "f64":
        lib = _native.load()
        import ctypes
        h = lib.fftwpp_create_hconv2d(w["L"][0], w["L"][1])
        n = fs[0].size
        pa = lib.create_complexAlign(n)
        pb = lib.create_complexAlign(n)
        A_ = np.ctypeslib.as_array((ctypes.c_double * (2 * n)).from_address(pa))
        B_ = np.ctypeslib.as_array((ctypes.c_double * (2 * n)).from_address(pb))
        src0 = fs[0].view(np.float64).ravel()
        B_[:] = fs[1].view(np.float64).ravel()
        for _ in range(args.warmup):
            A_[:] = src0
            lib.fftwpp_hconv2d_convolve(h, pa, pb)
        tot = 0.0
        for _ in range(args.steps):
            A_[:] = src0
            t0 = time.perf_counter()
            lib.fftwpp_hconv2d_convolve(h, pa, pb)
            tot += time.perf_counter() - t0
        e2e_err = rel_l2(A_.view(np.complex128).reshape(fs[0].shape), want)
        e2e = {"value": args.steps / tot, "unit": "convs/s",
               "h2d_bytes_per_step": 2 * n * 16, "d2h_bytes_per_step": n * 16,
               "api": "fftwpp_hconv2d_convolve (host pointers)",
               "rel_l2_vs_oracle": e2e_err}
        lib.fftwpp_hconv2d_delete(h)
        lib.delete_complexAlign(pa)
        lib.delete_complexAlign(pb)
    else:
        # Host-pointer entry of the device-API plan.
        host = [f.astype(np.complex128 if not conv.real else np.float64)
                if prec == "f64" else f.astype(np.complex64 if not conv.real
                                               else np.float32) for f in fs]
        tot = 0.0
        for _ in range(args.steps):
            hs = [x.copy() for x in host]
            t0 = time.perf_counter()
            conv.convolve_host(*hs)
            tot += time.perf_counter() - t0
        nb = host[0].nbytes
        e2e = {"value": args.steps / tot, "unit": "convs/s",
               "h2d_bytes_per_step": w["A"] * nb,
               "d2h_bytes_per_step": w["B"] * nb,
               "api": "fgb_convolve_host (host pointers)"}

    if big:
        cpu_rate, cpu_n, cpu_dt = None, 0, 0.0
    else:
        cpu_rate, cpu_n, cpu_dt = cpu_oracle_rate(w, args.cpu_budget, 64,
                                                  os.cpu_count() or 1)
    line = {
        "metric": METRIC, "value": value, "unit": "convs/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": prec,
        "data": "synthetic (seeded)",
        "config": {"workload": w["desc"], "precision": prec,
                   "parallelism": f"replicas x{world}",
                   "l2": "flushed (256 MB write) before every timed step",
                   "plan": conv.axes},
        "roofline": roofline,
        "compute_roofline": compute,
        "kernels_ms_per_step": dict(zip(names, per_launch)),
        "rel_l2_vs_fp64_oracle": err,
        "cpu_baseline": {"value": cpu_rate, "unit": "convs/s",
                         "cores": os.cpu_count() or 1, "kind": "port",
                         "sample": f"{cpu_n} single convolutions of the same "
                                   f"workload in {cpu_dt:.1f} s (numpy/scipy.fft "
                                   f"restatement of FFTW++'s hybrid convolution)"},
        "e2e": e2e,
        "gpu_launches": conv.launches * args.steps,
        "clocks": clk,
    }
    line.update(extra)
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def batched_lengths(n=512, lo=64, hi=65536, seed=2024):
    """512 lengths drawn log-uniformly in [64, 65536] from a seed."""
    rng = np.random.default_rng(seed)
    return [int(round(np.exp(u))) for u in
            rng.uniform(np.log(lo), np.log(hi), n)]


def run_batched(args):
    """Batched uneven 1D complex binary convolutions: one persistent launch
    replayed from a CUDA graph, against the same problems launched one plain
    convolution at a time."""
    import torch
    torch.cuda.set_device(0)
    from fftwpp_gb300.gpu import BatchedConvolution, HybridConvolution
    Ls = batched_lengths()
    prec = args.precision
    conv = BatchedConvolution(Ls, precision=prec, tune=True)
    rng = np.random.default_rng(3)
    f = rng.uniform(-1, 1, conv.total) + 1j * rng.uniform(-1, 1, conv.total)
    g = rng.uniform(-1, 1, conv.total) + 1j * rng.uniform(-1, 1, conv.total)
    tf = torch.from_numpy(f).to(conv.dtype).cuda()
    tg = torch.from_numpy(g).to(conv.dtype).cuda()
    out = [torch.empty_like(tf)]
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        conv.convolve(tf, tg, out=out, graph=True)
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(0)
    clocks.start()
    total = 0.0
    for _ in range(args.steps):
        flush.zero_()
        start.record(stream)
        conv.convolve(tf, tg, out=out, graph=True)
        stop.record(stream)
        stop.synchronize()
        total += start.elapsed_time(stop)
    clk = clocks.stop()
    assert conv.error() == 0
    value = len(Ls) * args.steps / (total * 1e-3)

    # Accuracy on a sample of problems against the FP64 oracle.
    from oracle import hybrid as H
    from oracle.direct import rel_l2
    h = out[0].cpu().numpy()
    errs = []
    for i in range(0, len(Ls), 37):
        o, L = conv.offsets[i], Ls[i]
        want = H.convolve([f[o:o + L], g[o:o + L]], [H.PAD], [L], [2 * L - 1])[0]
        errs.append(rel_l2(h[o:o + L], want))

    # The same problems as separate plain launches (one plan per problem).
    def separate(precision):
        plans = [HybridConvolution([PAD], [L], [2 * L - 1], precision=precision)
                 for L in Ls]
        dt = plans[0].dtype
        ins = [(torch.from_numpy(f[o:o + L].copy()).to(dt).cuda(),
                torch.from_numpy(g[o:o + L].copy()).to(dt).cuda())
               for o, L in zip(conv.offsets, Ls)]
        outs = [torch.empty_like(a) for a, _ in ins]
        for p, (a, b), c in zip(plans, ins, outs):
            p.convolve(a, b, out=[c])
        torch.cuda.synchronize()
        t = 0.0
        reps = max(1, args.steps // 5)
        for _ in range(reps):
            flush.zero_()
            start.record(stream)
            for p, (a, b), c in zip(plans, ins, outs):
                p.convolve(a, b, out=[c])
            stop.record(stream)
            stop.synchronize()
            t += start.elapsed_time(stop)
        return len(Ls) * reps / (t * 1e-3), sum(p.launches for p in plans)

    sep_same, sep_launches = separate(prec)
    sep_f64, _ = separate("f64") if prec != "f64" else (sep_same, None)
    elem = 16 if prec == "f64" else 8
    abytes = 3 * elem * conv.total
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) \
        if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = abytes / (total / args.steps * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "convs/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": prec,
        "data": "synthetic (seeded)",
        "config": {"workload": "512 independent 1D complex binary convolutions,"
                               " L log-uniform in [64, 65536] (seed 2024), "
                               "M=2L-1, one persistent launch per step "
                               "replayed from a CUDA graph, autotuned plans",
                   "l2": "flushed (256 MB write) before every timed step",
                   "total_length": conv.total, "tasks": conv.tasks,
                   "grid": conv.grid, "short_problems": conv.short_problems,
                   "long_problems": conv.long_problems},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                     "kernel": "batchKernel",
                     "algorithmic_bytes_per_launch": abytes},
        "rel_l2_vs_fp64_oracle_max_sample": max(errs),
        "separate_plain_launches": {"value": sep_same, "unit": "convs/s",
                                    "launches_per_step": sep_launches,
                                    "batched_speedup": value / sep_same},
        "plain_fp64_separate_launches": {"value": sep_f64, "unit": "convs/s",
                                         "batched_speedup": value / sep_f64},
        "gpu_launches": args.steps,
        "clocks": clk,
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="hconv2d",
                    choices=sorted(WORKLOADS) + ["batched1d"])
    ap.add_argument("--precision", default="f64", choices=["f64", "f32"])
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    ap.add_argument("--quick", action="store_true",
                    help="skip the FP32 comparison leg")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.workload == "batched1d":
        if args.impl == "reference":
            return run_reference(args, dict(
                kinds=[PAD], L=[4096], M=[8191], mult="binary", A=2, B=1,
                desc="one 1D complex binary convolution L=4096 (a sample of "
                     "the batched workload)"))
        return run_batched(args)
    w = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, w)
    return run_ours(args, w)


if __name__ == "__main__":
    sys.exit(main())
