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
import datetime
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
    """nvidia-smi clock/throttle samples every 20 ms; only samples stamped
    inside the timed window (begin() .. end()) are summarised.  start()
    returns once the first sample has arrived, so the sampler is running
    before the window opens."""
    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,"
              "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")
    STAMP = "%Y/%m/%d %H:%M:%S.%f"

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}",
                 f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True, bufsize=1)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        deadline = time.time() + 5.0
        while not self.lines and time.time() < deadline:
            time.sleep(0.01)

    def begin(self):
        self.t0 = datetime.datetime.now()

    def end(self):
        self.t1 = datetime.datetime.now()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def _parse(self):
        out = []
        for ln in list(self.lines):
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 10:
                continue
            try:
                ts = datetime.datetime.strptime(parts[0], self.STAMP)
                out.append((ts, float(parts[2]), float(parts[3]), parts[6:10]))
            except ValueError:
                continue
        return out

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        # Let the sample that follows the window arrive, then stop.
        deadline = time.time() + 1.0
        while time.time() < deadline and self.t1 is not None:
            s = self._parse()
            if s and s[-1][0] >= self.t1:
                break
            time.sleep(0.02)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        samples = self._parse()
        t0 = self.t0 or datetime.datetime.min
        t1 = self.t1 or datetime.datetime.max
        inside = [x for x in samples if t0 <= x[0] <= t1]
        window = "timed region"
        if not inside:
            # Window shorter than the sampling period: the first sample after
            # it opened.
            after = [x for x in samples if x[0] >= t0]
            inside, window = after[:1], "first sample after the timed region opened"
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        reasons = set()
        for _, _, _, flags in inside:
            for name, val in zip(names, flags):
                if val.lower().startswith("active"):
                    reasons.add(name)
        sm = [x[1] for x in inside]
        smax = [x[2] for x in inside]
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm),
                "window": window,
                "window_ms": ((t1 - t0).total_seconds() * 1e3
                              if self.t0 and self.t1 else None)}


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
        H.convolve(fs, w["kinds"], w["L"], w["M"], ms=w.get("m"), mult=w["mult"],
                   workers=workers)
        n += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return n * 1.0 / dt, n, dt


def scipy_explicit(fs, w, workers):
    """Explicit zero-padded convolution with scipy.fft (the textbook method
    the hybrid scheme replaces): every input goes to a physical grid of at
    least the padded size, the multiplier is applied pointwise, the product
    is transformed back and the stored modes are kept.  Unnormalised like
    the reference's convolve (h_k = sum_p f_p g_{k-p})."""
    import scipy.fft as sf
    kinds, L, M = w["kinds"], w["L"], w["M"]

    def combine(us):
        if w["mult"] in ("binary", "realbinary"):
            return us[0] * us[1]
        if w["mult"] == "realjacobian":
            return us[0] * us[3] - us[1] * us[2]
        raise ValueError(w["mult"])

    if kinds == [PAD]:
        n = sf.next_fast_len(M[0])
        us = [sf.ifft(f, n=n, axis=-1, workers=workers) for f in fs]
        return sf.fft(combine(us), axis=-1, workers=workers)[..., :L[0]] * n
    if kinds == [REAL, PAD, PAD]:
        s = [sf.next_fast_len(m, real=True) for m in M]
        Fs = [sf.rfftn(f, s=s, workers=workers) for f in fs]
        h = sf.irfftn(Fs[0] * Fs[1], s=s, workers=workers)
        return h[:L[0], :L[1], :L[2]]
    if kinds == [CENTERED, HERMITIAN]:
        nx = sf.next_fast_len(M[0])
        ny = sf.next_fast_len(M[1], real=True)
        ny += ny % 2
        x0 = L[0] // 2
        kx = np.arange(L[0]) - x0
        Hy = fs[0].shape[1]
        us = []
        for f in fs:
            F = np.zeros((nx, ny // 2 + 1), dtype=np.complex128)
            F[kx % nx, :Hy] = f
            us.append(sf.irfft2(F, s=(nx, ny), workers=workers))
        H = sf.rfft2(combine(us), workers=workers) * (nx * ny)
        return H[kx % nx, :Hy]
    raise ValueError("no explicit-padding baseline for this workload")


def cpu_scipy_rate(w, budget_s, workers, fs, max_convs=64):
    """Time scipy_explicit on the workload's inputs fs (bounded like the
    oracle leg); returns (convs/s, n, seconds, result of the last call)."""
    n, t0, h = 0, time.perf_counter(), None
    while n < max_convs:
        h = scipy_explicit(fs, w, workers)
        n += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    batch = w.get("batch", 1)
    return n * batch / dt, n, dt, h


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
    # Bound the run: about 15 s of warm-up and 60 s of timed work at most.
    t0 = time.perf_counter()
    H.convolve(fs, w["kinds"], w["L"], w["M"], ms=w.get("m"), mult=w["mult"],
               workers=workers)
    est = time.perf_counter() - t0
    nwarm = min(args.warmup, max(1, int(15.0 / est))) - 1
    ntimed = min(args.steps, max(1, int(60.0 / est)))
    for _ in range(nwarm):
        H.convolve(fs, w["kinds"], w["L"], w["M"], ms=w.get("m"), mult=w["mult"],
                   workers=workers)
    t0 = time.perf_counter()
    for _ in range(ntimed):
        H.convolve(fs, w["kinds"], w["L"], w["M"], ms=w.get("m"), mult=w["mult"],
                   workers=workers)
    dt = time.perf_counter() - t0
    value = ntimed / dt
    sample = (f"{ntimed} timed single convolutions of the workload "
              f"(numpy/scipy.fft restatement of FFTW++'s hybrid convolution, "
              f"scipy workers={workers})")
    line = {
        "impl": "reference", "metric": METRIC, "value": value,
        "unit": "convs/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt / ntimed * 1e3,
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


def barrier_sync(world):
    """Barrier across ranks (when there are several) and a device sync."""
    import torch
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
        torch.cuda.synchronize()


def time_device(conv, ts, steps, warmup, flush, timing=True, clocks=None,
                world=1):
    """Per-step CUDA-event timing on the current stream; returns total ms.
    The timed loop is bracketed by a barrier and a device sync on both
    sides; `clocks` (a started ClockSampler) is told when it opens and
    closes."""
    import torch
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        conv.convolve(*ts)
    barrier_sync(world)
    if clocks:
        clocks.begin()
    # NVTX range "timed": lets a profiler capture only the timed launches
    # (plan-time autotuning launches come before it).
    torch.cuda.nvtx.range_push("timed")
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
    torch.cuda.nvtx.range_pop()
    barrier_sync(world)
    if clocks:
        clocks.end()
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
    line = measure(args, w, args.workload, args.steps, args.warmup, world,
                   rank, local)
    if (args.workload == "hconv2d" and args.precision == "f64" and
            not args.quick and not args.no_real3d):
        # The largest single-GPU configuration, the 3D real convolution,
        # measured in the same run with its own roofline, CPU baseline and
        # end-to-end rate (fewer steps: one FP64 convolution is ~20 ms).
        w3 = WORKLOADS["real3d"]
        sub = measure(args, w3, "real3d", min(args.steps, 40),
                      max(3, min(args.warmup, 5)), world, rank, local)
        if line is not None:
            line["real3d"] = sub
    if line is not None:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def measure(args, w, workload, steps, warmup, world, rank, local):
    """One workload on this rank's GPU: device-timed rate, per-kernel times,
    roofline, accuracy against the oracle, the other precisions, end to
    end through the host entry and the CPU baselines.  Returns the JSON
    line on rank 0, None elsewhere."""
    import torch
    from fftwpp_gb300 import _native
    from fftwpp_gb300.gpu import HybridConvolution

    prec = args.precision
    fs = synth_inputs(w, seed=1)
    conv = HybridConvolution(w["kinds"], w["L"], w["M"], m=w.get("m"), A=w["A"], B=w["B"],
                             mult=w["mult"], precision=prec,
                             batch=w.get("batch", 1))
    ts = [torch.from_numpy(f).to(conv.dtype).cuda() for f in fs]
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")

    clocks = ClockSampler(local) if rank == 0 else None
    if clocks:
        clocks.start()
    total_ms, outs = time_device(conv, ts, steps, warmup, flush,
                                 clocks=clocks, world=world)
    clk = clocks.stop() if clocks else None
    if world > 1:
        t = torch.tensor([total_ms], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
        torch.distributed.barrier()
    nb = w.get("batch", 1)          # convolutions per step
    value = world * nb * steps / (total_ms * 1e-3)

    names = conv.launch_names()
    kms = conv.kernel_ms()
    per_launch = [k / steps for k in kms]
    dom = int(np.argmax(per_launch))
    elem = (8 if conv.real else 16) if prec != "f32" else (4 if conv.real else 8)
    abytes = algorithmic_bytes(w, elem)

    if rank != 0:
        return None

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
    traffic = (None if w.get("custom") else
               traffic_from_profiles(workload, names[dom], prec))
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                "kernel": names[dom], "peak_source": peak_src,
                "algorithmic_bytes_per_launch": abytes,
                "whole_step_frac": abytes / (total_ms / steps * 1e-3)
                / 1e9 / peak}

    # Compute roofline of the FP64 kernels: FP64 instructions per launch
    # (ncu, committed under profiles/) over the live launch time, against
    # the DFMA issue rate measured on this GPU.
    # The FP64 kernels against the DFMA issue rate (FP64 instructions per
    # launch, DPINST); the float-float and FP32 kernels against the FFMA
    # issue rate (FP32 instructions per launch, SPINST).  Both counts come
    # from the committed ncu summaries, the rates from fgb_measure_fma_rate.
    compute = None
    dfma, ffma = measured_fma_rates()
    tag, rate, bound = (("DPINST", dfma, "fp64_issue") if prec == "f64" else
                        ("SPINST", ffma, "fp32_issue"))
    if rate:
        cnt = [None if w.get("custom") else
               profile_figure(tag, workload, n, prec) for n in names]
        compute = {"fp64_tflops_peak_measured": 2 * dfma / 1e12,
                   "fp32_tflops_peak_measured": 2 * ffma / 1e12}
        if cnt[dom]:
            total = sum(cnt) if all(cnt) else None
            compute.update({
                "bound": bound, "kernel": names[dom],
                "achieved": cnt[dom] / (per_launch[dom] * 1e-3),
                "peak": rate,
                "unit": ("FP64" if tag == "DPINST" else "FP32") + " inst/s",
                "frac": cnt[dom] / (per_launch[dom] * 1e-3) / rate,
                "whole_step_frac": (total / (total_ms / steps * 1e-3)
                                    / rate) if total else None,
                "source": f"{tag} lines (instructions per launch, ncu) "
                          "under profiles/, peak from fgb_measure_fma_rate"})

    # Accuracy at full size against the CPU oracle (FP64 restatement), or,
    # for the 256^3 workload, against FP64 direct sums at sampled outputs.
    from oracle import hybrid as H
    from oracle.direct import rel_l2
    big = np.prod([l for l in w["L"]]) > 5e6
    want = None
    if w.get("batch", 1) == 1 and not big:
        want = H.convolve(fs, w["kinds"], w["L"], w["M"], ms=w.get("m"), mult=w["mult"],
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
        # The FP32-compensated and float-float modes on the same workload.
        for other, key in (("f32", "fp32_compensated"), ("ff", "float_float")):
            co = HybridConvolution(w["kinds"], w["L"], w["M"], m=w.get("m"), A=w["A"],
                                   B=w["B"], mult=w["mult"], precision=other,
                                   batch=w.get("batch", 1))
            to = [torch.from_numpy(f).to(co.dtype).cuda() for f in fs]
            mso, oo = time_device(co, to, steps, warmup, flush,
                                  timing=False)
            if want is not None:
                eo = rel_l2(oo[0].cpu().numpy(), want)
            elif big:
                eo = spot_check(fs, oo[0].cpu().numpy().astype(got0.dtype), w,
                                n=12)
            else:
                eo = None
            extra[key] = {"value": nb * steps / (mso * 1e-3),
                          "unit": "convs/s", "rel_l2_vs_fp64_oracle": eo,
                          "speedup_vs_fp64": total_ms / mso}
            del co, to, oo

    # End to end through the reference-facing C ABI on host buffers.
    e2e = None
    if workload == "hconv2d" and prec == "f64":
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
        for _ in range(warmup):
            A_[:] = src0
            lib.fftwpp_hconv2d_convolve(h, pa, pb)
        tot = 0.0
        for _ in range(steps):
            A_[:] = src0
            t0 = time.perf_counter()
            lib.fftwpp_hconv2d_convolve(h, pa, pb)
            tot += time.perf_counter() - t0
        e2e_err = rel_l2(A_.view(np.complex128).reshape(fs[0].shape), want)
        e2e = {"value": nb * steps / tot, "unit": "convs/s",
               "h2d_bytes_per_step": 2 * n * 16, "d2h_bytes_per_step": n * 16,
               "api": "fftwpp_hconv2d_convolve (create_complexAlign "
                      "page-locked buffers, zero copy over the host link)",
               "rel_l2_vs_oracle": e2e_err}
        lib.fftwpp_hconv2d_delete(h)
        lib.delete_complexAlign(pa)
        lib.delete_complexAlign(pb)
    else:
        # Host-pointer entry of the device-API plan, on page-locked arrays
        # (the kernels read and write them over the host link).
        host = [torch.from_numpy(np.ascontiguousarray(f)).to(conv.dtype)
                .pin_memory().numpy() for f in fs]
        src0 = host[0].copy()
        for _ in range(warmup):
            host[0][...] = src0
            conv.convolve_host(*host)
        tot = 0.0
        for _ in range(steps):
            host[0][...] = src0
            t0 = time.perf_counter()
            conv.convolve_host(*host)
            tot += time.perf_counter() - t0
        nbytes = host[0].nbytes
        e2e = {"value": nb * steps / tot, "unit": "convs/s",
               "h2d_bytes_per_step": w["A"] * nbytes,
               "d2h_bytes_per_step": w["B"] * nbytes,
               "api": "fgb_convolve_host (page-locked host arrays, "
                      "zero copy over the host link)",
               "host_path": list(conv.host_path())}

    cpu_rate, cpu_n, cpu_dt = cpu_oracle_rate(w, args.cpu_budget, 64,
                                              os.cpu_count() or 1)
    sp_rate, sp_n, sp_dt, sp_h = cpu_scipy_rate(w, args.cpu_budget,
                                                os.cpu_count() or 1, fs)
    sp_first = sp_h[0] if w.get("batch", 1) > 1 else sp_h
    ours_first = (outs[0][0] if w.get("batch", 1) > 1 else outs[0])
    scipy_point = {
        "value": sp_rate, "unit": "convs/s", "cores": os.cpu_count() or 1,
        "label": "scipy explicit-padding CPU",
        "sample": f"{sp_n} calls in {sp_dt:.1f} s (scipy.fft, zero-padded "
                  f"physical grids, workers={os.cpu_count() or 1})",
        "rel_l2_gpu_vs_scipy": rel_l2(
            ours_first.cpu().numpy().astype(np.result_type(sp_first)),
            sp_first)}
    line = {
        "metric": METRIC, "value": value, "unit": "convs/s", "n_gpus": world,
        "steps": steps, "warmup": warmup,
        "ms_per_step": total_ms / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": prec,
        "data": "synthetic (seeded)",
        "config": {"workload": w["desc"], "precision": prec,
                   "parallelism": f"replicas x{world}",
                   "l2": "flushed (256 MB write) before every timed step",
                   "plan": conv.axes, "rows_per_cta": conv.rows_per_cta,
                   "threads_per_cta": conv.threads_per_cta},
        "roofline": roofline,
        "compute_roofline": compute,
        "kernels_ms_per_step": dict(zip(names, per_launch)),
        "rel_l2_vs_fp64_oracle": err,
        "cpu_baseline": {"value": cpu_rate, "unit": "convs/s",
                         "cores": os.cpu_count() or 1, "kind": "port",
                         "sample": f"{cpu_n} single convolutions of the same "
                                   f"workload in {cpu_dt:.1f} s (numpy/scipy.fft "
                                   f"restatement of FFTW++'s hybrid convolution)"},
        "cpu_scipy_explicit": scipy_point,
        "e2e": e2e,
        "gpu_launches": conv.launches * steps,
        "clocks": clk,
    }
    line.update(extra)
    return line


def batched_lengths(n=512, lo=64, hi=65536, seed=2024):
    """512 lengths drawn log-uniformly in [64, 65536] from a seed."""
    rng = np.random.default_rng(seed)
    return [int(round(np.exp(u))) for u in
            rng.uniform(np.log(lo), np.log(hi), n)]


def batched_job(world):
    """The whole batched job at `world` ranks: one 512-problem batch per rank
    (seeds 2024, 2025, ...), so per-rank work stays fixed as ranks are added.
    Returns the lengths and the packed inputs f, g (iid U[-1,1])."""
    Ls = []
    for s in range(world):
        Ls += batched_lengths(seed=2024 + s)
    rng = np.random.default_rng(3)
    tot = sum(Ls)
    f = rng.uniform(-1, 1, tot) + 1j * rng.uniform(-1, 1, tot)
    g = rng.uniform(-1, 1, tot) + 1j * rng.uniform(-1, 1, tot)
    return Ls, f, g


BATCHED_DESC = ("512 independent 1D complex binary convolutions per GPU, L "
                "log-uniform in [64, 65536] (seed 2024 + shard), M=2L-1, "
                "sharded across ranks by cost (L log L), one persistent launch "
                "per step replayed from a CUDA graph, autotuned plans")


def oracle_batch_rate(Ls, f, g, budget_s, workers, stride=None):
    """Time the CPU restatement over a bounded, evenly strided sample of the
    batch's problems; returns (convs/s, problems timed, seconds, stride).
    Without a stride, one is chosen from a calibration pass over every 16th
    problem so that the sample takes about budget_s."""
    from oracle import hybrid as H
    from fftwpp_gb300.sharding import offsets
    off = offsets(Ls)
    if stride is None:
        t0 = time.perf_counter()
        for i in range(0, len(Ls), 16):
            o, L = off[i], Ls[i]
            H.convolve([f[o:o + L], g[o:o + L]], [H.PAD], [L], [2 * L - 1],
                       workers=workers)
        per = (time.perf_counter() - t0) / len(range(0, len(Ls), 16))
        stride = max(1, int(np.ceil(per * len(Ls) / max(budget_s, 1e-3))))
    idx = list(range(0, len(Ls), stride))
    t0 = time.perf_counter()
    for i in idx:
        o, L = off[i], Ls[i]
        H.convolve([f[o:o + L], g[o:o + L]], [H.PAD], [L], [2 * L - 1],
                   workers=workers)
    dt = time.perf_counter() - t0
    return len(idx) / dt, len(idx), dt, stride


GRAD_DESC = ("differentiable 2D advection Jacobian on 1023x512 "
             "centred-Hermitian modes (Lx=Ly=1023), 2/3 rule (M=1534): one "
             "step = J(psi, omega) from the four derivative fields, loss = "
             "sum |J|^2, backward through the adjoint convolution (A=5, B=4); "
             "2 dealiased convolutions per step; psi, omega with amplitude "
             "|k|^-2 and seeded random phases")


def grad_spectra(Lx, Ly, seed):
    """psi, omega with amplitude |k|^-2 (0 at k=0) and uniform random
    phases, Hermitian-symmetrised on the k_y = 0 column."""
    from oracle import hybrid as H
    Hy = (Ly + 1) // 2
    rng = np.random.default_rng(seed)
    kx = (np.arange(Lx) - Lx // 2)[:, None]
    ky = np.arange(Hy)[None, :]
    k2 = (kx ** 2 + ky ** 2).astype(float)
    amp = np.where(k2 > 0, 1.0 / np.where(k2 > 0, k2, 1.0), 0.0)
    out = []
    for _ in range(2):
        f = amp * np.exp(2j * np.pi * rng.uniform(size=(Lx, Hy)))
        H.hermitian_symmetrize_x(f, (Lx + 1) // 2, Hy, Lx // 2)
        out.append(np.ascontiguousarray(f))
    return out


def oracle_grad_step(psi, omega, Lx, Ly, workers):
    """One gradient step of loss = sum |J|^2 on the CPU restatement: the
    forward Jacobian convolution and the adjoint convolution (the same
    algebra as fftwpp_gb300.autograd), numpy elsewhere."""
    from oracle import hybrid as H
    kinds = [H.CENTERED, H.HERMITIAN]
    M = [H.default_M(k, l) for k, l in zip(kinds, [Lx, Ly])]
    Hy = (Ly + 1) // 2
    kx = (np.arange(Lx) - Lx // 2)[:, None]
    ky = np.arange(Hy)[None, :]
    a = [1j * kx * psi, 1j * ky * psi, 1j * kx * omega, 1j * ky * omega]
    J = H.convolve(a, kinds, [Lx, Ly], M, mult="realjacobian",
                   workers=workers)[0]
    w = np.ones((1, Hy))
    w[0, 1:] = 2.0
    G = 2 * J / w
    g = H.convolve(a + [G], kinds, [Lx, Ly], M, mult="realjacadj", B=4,
                   workers=workers)
    g = [w * x for x in g]
    # Chain rule through a = (i kx psi, i ky psi, i kx omega, i ky omega).
    gp = np.conj(1j * kx) * g[0] + np.conj(1j * ky) * g[1]
    go = np.conj(1j * kx) * g[2] + np.conj(1j * ky) * g[3]
    return float(np.sum(np.abs(J) ** 2)), gp, go


def run_jacobian_grad(args):
    """C5: forward + loss + adjoint backward of the differentiable 2D
    advection Jacobian through torch.autograd, timed per step on the
    device; the adjoint checked at full size against central differences
    (FP64, float-float) or against the FP64 gradient (FP32)."""
    import torch
    world, rank, local = dist_setup()
    if world > 1:
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    from fftwpp_gb300.autograd import AdvectionJacobian, GraphedLossStep
    prec = args.precision
    Lx = Ly = 1023
    op = AdvectionJacobian(Lx, Ly, precision=prec)
    cdt = op.dtype
    p0, o0 = grad_spectra(Lx, Ly, seed=11)
    psi = torch.from_numpy(p0).to(cdt).cuda().requires_grad_(True)
    omega = torch.from_numpy(o0).to(cdt).cuda().requires_grad_(True)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    def step(p, o):
        J = op(p, o)
        loss = (J.real ** 2 + J.imag ** 2).sum()
        loss.backward()
        return loss

    for _ in range(args.warmup):
        psi.grad = omega.grad = None
        step(psi, omega)
    clocks = ClockSampler(local) if rank == 0 else None
    if clocks:
        clocks.start()
    barrier_sync(world)
    torch.cuda.nvtx.range_push("timed")
    # The backward pass runs on autograd's device thread, outside this
    # thread's NVTX range: profiler start/stop (process-wide) brackets the
    # timed steps for a profiler run with profiling off at start.
    torch.cuda.profiler.start()
    op.fwd.enable_timing(True)
    op.adj.enable_timing(True)
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    total = 0.0
    for _ in range(args.steps):
        psi.grad = omega.grad = None
        flush.zero_()
        start.record(stream)
        step(psi, omega)
        stop.record(stream)
        stop.synchronize()
        total += start.elapsed_time(stop)
        op.fwd.collect_timing()
        op.adj.collect_timing()
    torch.cuda.profiler.stop()
    torch.cuda.nvtx.range_pop()
    barrier_sync(world)
    kf = [t / args.steps for t in op.fwd.kernel_ms()]
    ka = [t / args.steps for t in op.adj.kernel_ms()]
    op.fwd.enable_timing(False)
    op.adj.enable_timing(False)
    eager_total = total

    # The same step captured once in a CUDA graph and replayed: the value.
    graphed = GraphedLossStep(op, psi.detach(), omega.detach())
    for _ in range(args.warmup):
        graphed()
    barrier_sync(world)
    if clocks:
        clocks.begin()
    torch.cuda.nvtx.range_push("timed")
    total = 0.0
    for _ in range(args.steps):
        flush.zero_()
        start.record(stream)
        graphed()
        stop.record(stream)
        stop.synchronize()
        total += start.elapsed_time(stop)
    torch.cuda.nvtx.range_pop()
    barrier_sync(world)
    if clocks:
        clocks.end()
    clk = clocks.stop() if clocks else None
    if world > 1:
        t = torch.tensor([total], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total = float(t.item())
    ms = total / args.steps
    value = world * 2 * args.steps / (total * 1e-3)
    if rank != 0:
        torch.distributed.destroy_process_group()
        return 0

    # Roofline of the dominant kernel: its convolution's compulsory bytes
    # (inputs read + outputs written at the stored size) over its launch.
    names = [f"fwd/{n}" for n in op.fwd.launch_names()] + \
        [f"adj/{n}" for n in op.adj.launch_names()]
    per = kf + ka
    dom = int(np.argmax(per))
    nmodes = Lx * ((Ly + 1) // 2)
    elem = 8 if prec == "f32" else 16
    conv_bytes = ((4 + 1) if dom < len(kf) else (5 + 4)) * elem * nmodes
    peaks = {}
    pfile = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pfile):
        peaks = json.load(open(pfile))
    peak = peaks.get("hbm_gbs")
    peak_src = "measured"
    if not peak:
        peak, peak_src = 6800.0, "fallback"
    achieved = conv_bytes / (per[dom] * 1e-3) / 1e9
    step_bytes = (5 + 9) * elem * nmodes
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic_from_profiles("jacobian2d_grad",
                                                 names[dom], prec),
                "kernel": names[dom], "peak_source": peak_src,
                "algorithmic_bytes_per_launch": conv_bytes,
                "whole_step_frac": step_bytes / (ms * 1e-3) / 1e9 / peak}
    compute = None
    dfma, ffma = measured_fma_rates()
    tag, rate, bound = (("DPINST", dfma, "fp64_issue") if prec == "f64" else
                        ("SPINST", ffma, "fp32_issue"))
    if rate:
        compute = {"fp64_tflops_peak_measured": 2 * dfma / 1e12,
                   "fp32_tflops_peak_measured": 2 * ffma / 1e12}
        cnt = profile_figure(tag, "jacobian2d_grad", names[dom], prec)
        if cnt:
            compute.update({
                "bound": bound, "kernel": names[dom],
                "achieved": cnt / (per[dom] * 1e-3), "peak": rate,
                "unit": ("FP64" if tag == "DPINST" else "FP32") + " inst/s",
                "frac": cnt / (per[dom] * 1e-3) / rate,
                "source": f"{tag} line (instructions per launch, ncu) "
                          "under profiles/, peak from fgb_measure_fma_rate"})

    # The adjoint at full size: central differences along random directions
    # (FP64 and float-float), or the FP32 gradient against the FP64 one.
    def loss_of(p, o):
        J = op(p, o)
        return (J.real ** 2 + J.imag ** 2).sum()
    psi.grad = omega.grad = None
    loss = loss_of(psi, omega)
    gp, go = torch.autograd.grad(loss, (psi, omega))
    check = {}
    if prec == "f32":
        ref = AdvectionJacobian(Lx, Ly, precision="f64")
        p64 = psi.detach().to(torch.complex128).requires_grad_(True)
        o64 = omega.detach().to(torch.complex128).requires_grad_(True)
        l64 = (lambda J: (J.real ** 2 + J.imag ** 2).sum())(ref(p64, o64))
        gp64, go64 = torch.autograd.grad(l64, (p64, o64))
        num = float((gp.to(torch.complex128) - gp64).abs().pow(2).sum() +
                    (go.to(torch.complex128) - go64).abs().pow(2).sum())
        den = float(gp64.abs().pow(2).sum() + go64.abs().pow(2).sum())
        check = {"fp32_gradient_rel_l2_vs_fp64": (num / den) ** 0.5}
        del ref
    else:
        # Directions with the spectra's |k|^-2 amplitude, so that h v is a
        # relative perturbation of every mode (white-noise directions would
        # swamp the ~1e-6 high-k modes and measure the h^2 term instead).
        rng = np.random.default_rng(17)
        h, worst, ndir = 1e-6, 0.0, 16
        kx = (np.arange(Lx) - Lx // 2)[:, None]
        ky = np.arange((Ly + 1) // 2)[None, :]
        k2 = (kx ** 2 + ky ** 2).astype(float)
        amp = np.where(k2 > 0, 1.0 / np.where(k2 > 0, k2, 1.0), 0.0)
        with torch.no_grad():
            for _ in range(ndir):
                vp = torch.from_numpy(amp * (rng.normal(size=p0.shape) + 1j *
                                             rng.normal(size=p0.shape))
                                      ).to(cdt).cuda()
                vo = torch.from_numpy(amp * (rng.normal(size=p0.shape) + 1j *
                                             rng.normal(size=p0.shape))
                                      ).to(cdt).cuda()
                lp = loss_of(psi + h * vp, omega + h * vo)
                lm = loss_of(psi - h * vp, omega - h * vo)
                fd = float((lp - lm) / (2 * h))
                an = float((torch.conj(gp) * vp).real.sum() +
                           (torch.conj(go) * vo).real.sum())
                worst = max(worst, abs(fd - an) / max(abs(an), 1e-300))
        check = {"adjoint_vs_central_differences": {
            "directions": ndir, "h": h, "max_rel_err": worst}}

    # End to end: page-locked spectra copied into the graph's inputs, the
    # graphed step, the loss read back, every step.
    hp = torch.from_numpy(p0).to(cdt).pin_memory()
    ho = torch.from_numpy(o0).to(cdt).pin_memory()

    def e2e_step():
        with torch.no_grad():
            graphed.psi.copy_(hp, non_blocking=True)
            graphed.omega.copy_(ho, non_blocking=True)
        return float(graphed()[0])
    for _ in range(args.warmup):
        e2e_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_dt = time.perf_counter() - t0
    e2e = {"value": 2 * args.steps / e2e_dt, "unit": "convs/s",
           "grad_steps_per_s": args.steps / e2e_dt,
           "h2d_bytes_per_step": hp.nbytes + ho.nbytes,
           "d2h_bytes_per_step": 8 if prec != "f32" else 4,
           "api": "fftwpp_gb300.autograd.GraphedLossStep over "
                  "AdvectionJacobian (page-locked spectra copied in, the "
                  "loss read back)"}

    # CPU: the same step on the restatement, a bounded sample.
    workers = os.cpu_count() or 1
    n, t0 = 0, time.perf_counter()
    while True:
        oracle_grad_step(p0, o0, Lx, Ly, workers)
        n += 1
        if time.perf_counter() - t0 > args.cpu_budget:
            break
    cdt_s = time.perf_counter() - t0
    cpu = {"value": 2 * n / cdt_s, "unit": "convs/s", "cores": workers,
           "kind": "port",
           "sample": f"{n} gradient steps ({2 * n} convolutions) in "
                     f"{cdt_s:.1f} s (numpy/scipy.fft restatement of "
                     "FFTW++'s hybrid convolution, forward and adjoint)"}
    line = {
        "metric": METRIC, "value": value, "unit": "convs/s",
        "grad_steps_per_s": value / 2, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": prec,
        "data": "synthetic (seeded)",
        "config": {"workload": GRAD_DESC,
                   "parallelism": f"replicas x{world}",
                   "l2": "flushed (256 MB write) before every timed step"},
        "roofline": roofline, "compute_roofline": compute,
        "kernels_ms_per_step": dict(zip(names, per)),
        "eager_autograd": {"value": world * 2 * args.steps /
                           (eager_total * 1e-3), "unit": "convs/s",
                           "ms_per_step": eager_total / args.steps,
                           "note": "the same step launched op by op; "
                                   "kernel times above are from it"},
        "graph": "the step is one CUDA graph replay (GraphedLossStep)",
        **check,
        "cpu_baseline": cpu, "e2e": e2e,
        "gpu_launches": args.steps * (op.fwd.launches + op.adj.launches + 5),
        "clocks": clk,
    }
    print(json.dumps(line))
    return 0


def run_reference_grad(args):
    """--impl reference for the gradient step: the CPU restatement's
    forward and adjoint convolutions on every host core."""
    world, rank, _ = dist_setup()
    if rank != 0:
        return 0
    workers = os.cpu_count() or 1
    Lx = Ly = 1023
    p0, o0 = grad_spectra(Lx, Ly, seed=11)
    t0 = time.perf_counter()
    oracle_grad_step(p0, o0, Lx, Ly, workers)
    est = time.perf_counter() - t0
    nwarm = min(args.warmup, max(1, int(15.0 / est))) - 1
    ntimed = min(args.steps, max(1, int(60.0 / est)))
    for _ in range(nwarm):
        oracle_grad_step(p0, o0, Lx, Ly, workers)
    t0 = time.perf_counter()
    for _ in range(ntimed):
        oracle_grad_step(p0, o0, Lx, Ly, workers)
    dt = time.perf_counter() - t0
    value = 2 * ntimed / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value,
        "unit": "convs/s", "grad_steps_per_s": value / 2,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt / ntimed * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": GRAD_DESC, "parallelism": "cpu"},
        "cpu_baseline": {"value": value, "unit": "convs/s", "cores": workers,
                         "kind": "port",
                         "sample": f"{ntimed} timed gradient steps"},
        "e2e": {"value": value, "unit": "convs/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_reference_batched(args):
    """--impl reference for the batched workload: the CPU restatement over
    the same problem distribution, one bounded strided sample per step."""
    world, rank, _ = dist_setup()
    if rank != 0:
        return 0
    workers = os.cpu_count() or 1
    Ls, f, g = batched_job(1)
    budget = max(1.0, 120.0 / max(args.steps + args.warmup, 1))
    n = 0
    dt = 0.0
    stride = None
    for it in range(args.warmup + args.steps):
        rate, k, t, stride = oracle_batch_rate(Ls, f, g, budget, workers,
                                               stride)
        if it >= args.warmup:
            n += k
            dt += t
    value = n / dt
    sample = (f"a stride-{stride} sample of the 512 problems per step "
              f"(numpy/scipy.fft restatement of FFTW++'s hybrid convolution, "
              f"scipy workers={workers})")
    line = {
        "impl": "reference", "metric": METRIC, "value": value,
        "unit": "convs/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": BATCHED_DESC, "parallelism": "cpu"},
        "cpu_baseline": {"value": value, "unit": "convs/s", "cores": workers,
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "convs/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_batched(args):
    """Batched uneven 1D complex binary convolutions: one persistent launch
    per rank replayed from a CUDA graph, against the same problems launched
    one plain convolution at a time."""
    import torch
    world, rank, local = dist_setup()
    if world > 1:
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    from fftwpp_gb300.gpu import HybridConvolution
    from fftwpp_gb300.sharding import ShardedBatch
    Lall, fall, gall = batched_job(world)
    prec = args.precision
    shard = ShardedBatch(Lall, rank, world, precision=prec, tune=True)
    conv = shard.conv
    Ls = shard.local_lengths
    f, g = shard.local(fall), shard.local(gall)
    tf = torch.from_numpy(f).to(conv.dtype).cuda()
    tg = torch.from_numpy(g).to(conv.dtype).cuda()
    out = [torch.empty_like(tf)]
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    clocks = ClockSampler(local) if rank == 0 else None
    if clocks:
        clocks.start()
    for _ in range(args.warmup):
        conv.convolve(tf, tg, out=out, graph=True)
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    barrier_sync(world)
    if clocks:
        clocks.begin()
    total = 0.0
    torch.cuda.nvtx.range_push("timed")
    for _ in range(args.steps):
        flush.zero_()
        start.record(stream)
        conv.convolve(tf, tg, out=out, graph=True)
        stop.record(stream)
        stop.synchronize()
        total += start.elapsed_time(stop)
    torch.cuda.nvtx.range_pop()
    barrier_sync(world)
    if clocks:
        clocks.end()
    clk = clocks.stop() if clocks else None
    if conv.error() != 0:
        raise RuntimeError("a wait of the persistent kernel gave up")
    if world > 1:
        t = torch.tensor([total], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total = float(t.item())
    value = len(Lall) * args.steps / (total * 1e-3)

    # End to end through the public API: page-locked host inputs copied in,
    # one graph-replayed launch, the outputs copied back, every step.
    hf = torch.from_numpy(f).to(conv.dtype).pin_memory()
    hg = torch.from_numpy(g).to(conv.dtype).pin_memory()
    ho = torch.empty_like(hf).pin_memory()
    barrier_sync(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        tf.copy_(hf, non_blocking=True)
        tg.copy_(hg, non_blocking=True)
        conv.convolve(tf, tg, out=out, graph=True)
        ho.copy_(out[0], non_blocking=True)
    torch.cuda.synchronize()
    e2e_dt = time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([e2e_dt], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_dt = float(t.item())
    elem = 16 if prec == "f64" else 8
    e2e = {"value": len(Lall) * args.steps / e2e_dt, "unit": "convs/s",
           "h2d_bytes_per_step": 2 * elem * shard.local_total,
           "d2h_bytes_per_step": elem * shard.local_total,
           "api": "fftwpp_gb300.sharding.ShardedBatch / BatchedConvolution "
                  "on page-locked host tensors (copies inside the timed loop)"}

    if rank != 0:
        torch.distributed.destroy_process_group()
        return 0

    # Accuracy on a sample of this rank's problems against the FP64 oracle.
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
        reps = max(1, min(args.steps // 5, 20))
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
    abytes = 3 * elem * shard.local_total
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) \
        if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    peak = peaks.get("hbm_gbs")
    peak_src = "measured"
    if not peak:
        peak, peak_src = 6800.0, "fallback"
    achieved = abytes / (total / args.steps * 1e-3) / 1e9
    cpu = None
    if world == 1:
        rate, k, dt, stride = oracle_batch_rate(Ls, f, g, args.cpu_budget,
                                                os.cpu_count() or 1)
        cpu = {"value": rate, "unit": "convs/s", "cores": os.cpu_count() or 1,
               "kind": "port",
               "sample": f"a stride-{stride} sample of the 512 problems ({k} "
                         f"convolutions, {dt:.1f} s; numpy/scipy.fft "
                         f"restatement of FFTW++'s hybrid convolution)"}
    # Compute roofline of the persistent launch: its FP64 (FP32)
    # instructions per launch from the committed ncu summary over the live
    # step, against the issue rate measured on this GPU.
    compute = None
    dfma, ffma = measured_fma_rates()
    tag, rate, bound = (("DPINST", dfma, "fp64_issue") if prec == "f64" else
                        ("SPINST", ffma, "fp32_issue"))
    if rate:
        compute = {"fp64_tflops_peak_measured": 2 * dfma / 1e12,
                   "fp32_tflops_peak_measured": 2 * ffma / 1e12}
        cnt = profile_figure(tag, "batched1d", "batch", prec)
        if cnt:
            per = total / args.steps * 1e-3
            compute.update({
                "bound": bound, "kernel": "batchKernel",
                "achieved": cnt / per, "peak": rate,
                "unit": ("FP64" if tag == "DPINST" else "FP32") + " inst/s",
                "frac": cnt / per / rate,
                "source": f"{tag} line (instructions per launch, ncu) "
                          "under profiles/, peak from fgb_measure_fma_rate"})
    line = {
        "metric": METRIC, "value": value, "unit": "convs/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": prec,
        "data": "synthetic (seeded)",
        "config": {"workload": BATCHED_DESC,
                   "parallelism": f"shards x{world} (no data-path collective)",
                   "l2": "flushed (256 MB write) before every timed step",
                   "problems": len(Lall), "rank0_problems": len(Ls),
                   "rank0_total_length": shard.local_total,
                   "tasks": conv.tasks, "grid": conv.grid,
                   "short_problems": conv.short_problems,
                   "long_problems": conv.long_problems},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic_from_profiles("batched1d", "batch",
                                                      prec),
                     "kernel": "batchKernel", "peak_source": peak_src,
                     "algorithmic_bytes_per_launch": abytes},
        "compute_roofline": compute,
        "rel_l2_vs_fp64_oracle_max_sample": max(errs),
        "separate_plain_launches": {"value": sep_same, "unit": "convs/s",
                                    "launches_per_step": sep_launches,
                                    "batched_speedup": value / world / sep_same},
        "plain_fp64_separate_launches": {"value": sep_f64, "unit": "convs/s",
                                         "batched_speedup":
                                         value / world / sep_f64},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": args.steps,
        "clocks": clk,
    }
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def override(w, args):
    """The workload with -L/-M/-m applied (the reference and GPU arms take
    the same parameters, as the reference's test programs do)."""
    if not (args.L or args.M or args.m):
        return w
    w = dict(w)
    dim = len(w["kinds"])

    def ints(text):
        v = [int(x) for x in text.split(",")]
        if len(v) != dim:
            raise SystemExit(f"expected {dim} comma-separated values")
        return v
    if args.L:
        w["L"] = ints(args.L)
        w["M"] = [3 * ((l + 1) // 2) - 2 * (l % 2)
                  if k in (CENTERED, HERMITIAN) else 2 * l - 1
                  for k, l in zip(w["kinds"], w["L"])]
    if args.M:
        w["M"] = ints(args.M)
    if args.m:
        w["m"] = ints(args.m)
    w["custom"] = True         # the committed ncu figures do not apply
    w["desc"] = (w["desc"] + f" [overridden: L={w['L']}, M={w['M']}"
                 + (f", m={w['m']}" if args.m else "") + "]")
    return w


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="hconv2d",
                    choices=sorted(WORKLOADS) + ["batched1d",
                                                 "jacobian2d_grad"])
    ap.add_argument("--precision", default="f64", choices=["f64", "f32", "ff"])
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    ap.add_argument("--L", help="comma-separated data lengths per axis, "
                    "outermost first (the reference tests' -L)")
    ap.add_argument("--M", help="comma-separated minimum padded lengths "
                    "(-M; default: the workload's dealiasing rule)")
    ap.add_argument("--m", help="comma-separated forced residue block "
                    "lengths (-m; 0 = planner's choice)")
    ap.add_argument("--no-real3d", action="store_true",
                    help="skip the 3D real block of the default line")
    ap.add_argument("--quick", action="store_true",
                    help="skip the FP32 comparison leg")
    ap.add_argument("--wisdom", help="plan wisdom file: loaded before the "
                    "plans are made and saved after the run, so that a "
                    "profiled run rebuilds the plans a plain run tuned")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        if args.workload == "batched1d":
            return run_reference_batched(args)
        if args.workload == "jacobian2d_grad":
            return run_reference_grad(args)
        return run_reference(args, override(WORKLOADS[args.workload], args))
    if args.wisdom:
        from fftwpp_gb300 import gpu
        gpu.load_wisdom(args.wisdom)
    if args.workload == "batched1d":
        rc = run_batched(args)
    elif args.workload == "jacobian2d_grad":
        rc = run_jacobian_grad(args)
    else:
        rc = run_ours(args, override(WORKLOADS[args.workload], args))
    if args.wisdom:
        gpu.save_wisdom(args.wisdom)
    return rc


if __name__ == "__main__":
    sys.exit(main())
