#!/usr/bin/env python
"""FLCT velocity vectors/s on one GB300: the headline workload and the
other benchmark configurations.

Headline (one "step" = the whole flct computation on one frame pair):
1024 x 1024 float64 k^-2 random field, image2 = image1 advected by five
Gaussian vortices through the spectral warp (warp_frac2d semantics, run on
the GPU by this library), sigma = 8 (box 32), -s 4i (every 4th pixel
correlated, the rest cubic-convolution interpolated), thresh = 0.  That is
65,536 correlation windows and 1,048,576 output pixels per step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--form auto|fp32|tc_fp16|tc_bf16]
    python bench.py --impl reference ...   # the CPU implementation arm

value  = correlation windows per second with inputs resident in HBM
         (flct_gpu_velocity_device, CUDA events per step on the launch
         stream, L2 flushed with a 256 MiB write between steps).
e2e    = the same metric through flct_gpu_velocity with pinned host
         buffers: both input frames copied in and vx, vy, vm copied out
         every step.
Beside the headline line's keys: measured peaks (FP32 pipe, pinned copies),
`configs` with one record per other benchmark configuration (128^2 blobs,
the 512^2 precision study, the 64-pair heterogeneous batch, the 4096^2
sigma-15 stress case with its GPU warp), each with every window form, the
accuracy against the FP64 oracle and the oracle on one host core, and the
warp entry points at 512^2.  --no-batch skips the batch, the 4096^2 case
and the warp timing; --no-cpu skips the oracle runs.
"""
from __future__ import annotations

import argparse
import ctypes as C
import functools
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

WORKLOAD = "1024x1024 k^-2 field, 5-vortex spectral warp, sigma=8 (box 32), -s 4i, thresh 0"
METRIC = "FLCT velocity vectors/s (correlation windows/s) at 1024^2 sigma=8"
NSIDE, SIGMA, SKIP = 1024, 8.0, "4i"
FORMS = ("fp32", "tc_fp16", "tc_bf16")
CPU_SAMPLE = ("the oracle (C restatement of flct.c over the project double FFT; FFTW unavailable), "
              "1 thread")


# algorithmic flops of one n x n window: 3 real transforms at 2.5 M log2 M,
# M = n^2, plus means (2n^2), windowing (4n^2), conj product (4n^2), |c| and
# argmax (2n^2); 4 n (n/2+1) more with -k.
def window_flops(n: int, kr: bool = False) -> float:
    m = n * n
    f = 7.5 * m * np.log2(m) + 12 * m
    return f + (4 * n * (n // 2 + 1) if kr else 0)


def tc_flops_per_window(n: int) -> float:
    """Tensor flops the split tensor-core form executes per n x n window:
    four M = 128 GEMM stages per CTA iteration (the geometry of TcCfg<n> in
    window_tc.cuh), each product as hi*hi + hi*lo + lo*hi."""
    r8 = lambda x: (x + 7) // 8 * 8  # noqa: E731
    r16 = lambda x: (x + 15) // 16 * 16  # noqa: E731
    h = n // 2
    pack = h % 8 == 0
    r2 = h if pack else r8(h + 1)
    wit = 128 // r2
    n8, k1 = r8(n), r16(n)
    k2 = 2 * n8
    t1 = (2 * wit * n8 + 127) // 128
    t4 = (wit * n8 + 127) // 128
    macs = 3 * (t1 * 128 * k1 * k1 + 2 * 128 * k2 * k2 + 128 * k2 * k2 + t4 * 128 * k1 * k1)
    return 2.0 * macs / wit


def box_of(sigma: float) -> int:
    """n = 2 nsize, nsize = even part of (int)((int)sigma sqrt(ln 100))."""
    return 2 * (int(int(sigma) * np.sqrt(np.log(100.0))) // 2 * 2)


def workload(device=0):
    from pyflct_gb300 import synth
    rng = np.random.default_rng(20263)
    f1 = synth.kfield((NSIDE, NSIDE), rng)
    dfast, dslow = synth.vortex_shift(f1.shape, rng)
    f2 = synth.spectral_warp(f1, dfast, dslow, device)
    return np.ascontiguousarray(f1), np.ascontiguousarray(f2)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            return json.load(fh), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
            "sm_max_mhz": 2070.0}, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region: every 20 ms, started
    before the region and entered only once the first sample has arrived
    (nvidia-smi takes ~0.1 s to start), so the samples cover the region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        cmd = ["nvidia-smi", "-i", str(self.index),
               "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
               "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
               "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "20"]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.perf_counter()
            while not self.lines and time.perf_counter() - t0 < 3.0:
                time.sleep(0.005)
            self.lines = []  # samples from here on belong to the timed region
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax = max(smax, float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax or None,
                "samples": len(sm), "reasons": sorted(reasons)}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def reduce_max(value: float, device=None) -> float:
    """Max of a per-rank number over all ranks (the job's time is its
    slowest rank's); the identity without a process group."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


@functools.lru_cache(maxsize=1)
def cpu_model() -> str:
    """The host CPU's model name and core count (lscpu, else /proc/cpuinfo)."""
    name = ""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.lower().startswith("model name"):
                name = ln.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    if not name:
        try:
            with open("/proc/cpuinfo") as fh:
                for ln in fh:
                    if ln.lower().startswith(("model name", "cpu part")):
                        name = ln.split(":", 1)[1].strip()
                        break
        except OSError:
            pass
    return f"{name or 'unknown'}, {os.cpu_count()} cores"


def oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    po.build()
    return po


def run_reference(a):
    """The reference arm: the CPU implementation of the path (the oracle's
    C restatement of flct.c; the reference itself cannot be compiled on the
    GPU host because its sources do not travel there) on all host threads,
    with the same run on one thread reported beside it.  image2 is made by
    the same GPU spectral warp as in the GPU arm (input generation, outside
    the timed region)."""
    ws, rank, _ = dist_init()
    if rank != 0:
        return
    po = oracle()
    f1, f2 = workload()
    kw = dict(sigma=SIGMA, skip=4, interpolate=True)
    threads = os.cpu_count() or 1
    for _ in range(a.warmup):
        po.velocity(f1, f2, nthreads=threads, **kw)
    t0 = time.perf_counter()
    for _ in range(a.steps):
        po.velocity(f1, f2, nthreads=threads, **kw)
    dt = time.perf_counter() - t0
    windows = 256 * 256
    v = windows * a.steps / dt
    t1 = time.perf_counter()
    po.velocity(f1, f2, nthreads=1, **kw)
    one = windows / (time.perf_counter() - t1)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "windows/s", "n_gpus": ws,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * dt / a.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": WORKLOAD, "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": v, "unit": "windows/s", "cores": threads, "cpu": cpu_model(), "kind": "port",
                         "sample": "full frame per step (65,536 windows + interpolation), "
                                   f"{threads} threads, C restatement of flct.c over the "
                                   "project double FFT (FFTW unavailable)"},
        "cpu_1core": {"value": one, "unit": "windows/s", "cores": 1, "cpu": cpu_model(), "kind": "port",
                      "sample": "one full frame, 1 thread (the reference program is single-threaded)"},
        "e2e": {"value": v, "unit": "windows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU side


def measured_fp32_peak():
    """FP32-pipe throughput measured here (libflctprobe.so: independent FMA
    chains, scalar and packed, CUDA events); TFLOP/s, or None."""
    from pyflct_gb300 import build
    try:
        lib = C.CDLL(build.build_probe())
        s, p = C.c_double(), C.c_double()
        if lib.flct_probe_fp32_peak(5, C.byref(s), C.byref(p)) != 0:
            return None
        return {"scalar_tflops": s.value, "packed_tflops": p.value, "tflops": max(s.value, p.value)}
    except Exception:
        return None


def measured_copy_peaks(dev, h2d_bytes, d2h_bytes):
    """Pinned host <-> device copy bandwidth: one 256 MiB cudaMemcpyAsync
    each way (torch copy_), best of 5, CUDA events; and one step's copies
    (h2d_bytes in, d2h_bytes out) issued at the same time on two streams,
    best of 5, host clock.  On this machine the two directions share the
    host link (together they move about as much per second as one alone),
    so the step's copy time is the latter, not the longer direction."""
    import torch
    nbytes = 256 << 20
    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    out = {}
    hi = torch.empty(h2d_bytes, dtype=torch.uint8, pin_memory=True)
    ho = torch.empty(d2h_bytes, dtype=torch.uint8, pin_memory=True)
    di = torch.empty(h2d_bytes, dtype=torch.uint8, device=dev)
    do = torch.empty(d2h_bytes, dtype=torch.uint8, device=dev)
    s1, s2 = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    best = float("inf")
    for _ in range(6):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with torch.cuda.stream(s1):
            di.copy_(hi, non_blocking=True)
        with torch.cuda.stream(s2):
            ho.copy_(do, non_blocking=True)
        torch.cuda.synchronize()
        best = min(best, time.perf_counter() - t0)
    out["step_copies_ms"] = best * 1e3
    out["step_copies_gbs"] = (h2d_bytes + d2h_bytes) / best / 1e9
    for name, fn in (("h2d_gbs", lambda: d.copy_(h, non_blocking=True)),
                     ("d2h_gbs", lambda: h.copy_(d, non_blocking=True))):
        best = 0.0
        for _ in range(6):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            best = max(best, nbytes / (e0.elapsed_time(e1) / 1e3) / 1e9)
        out[name] = best
    return out


class DeviceRunner:
    """Timed device-buffer calls (flct_gpu_velocity_device) of one frame
    pair with one parameter set, L2 flushed between steps."""

    def __init__(self, ctx, dev, flush, f1, f2):
        import torch
        self.ctx, self.dev, self.flush = ctx, dev, flush
        self.nx, self.ny = f1.shape
        self.d1 = torch.from_numpy(np.ascontiguousarray(f1)).to(dev)
        self.d2 = torch.from_numpy(np.ascontiguousarray(f2)).to(dev)
        self.stream = torch.cuda.current_stream(dev)

    def run(self, p, steps, warmup, clocks=None):
        import torch
        from pyflct_gb300 import _lib
        lib, ctx = self.ctx.lib, self.ctx
        out = [torch.empty(self.nx, self.ny, dtype=torch.float64, device=self.dev) for _ in range(3)]
        sh = C.c_void_p(self.stream.cuda_stream)

        def step():
            ctx.check(lib.flct_gpu_velocity_device(
                ctx.h, C.byref(p), C.c_void_p(self.d1.data_ptr()), C.c_void_p(self.d2.data_ptr()),
                self.nx, self.ny, *[C.c_void_p(o.data_ptr()) for o in out], sh))

        for _ in range(max(3, warmup)):
            step()
        torch.cuda.synchronize()
        t = ctx.timing()
        names = {v: k for k, v in _lib.FORMS.items()}
        res = dict(windows=int(t.windows), launches=int(t.launches), box=int(t.box), used=names[int(t.form)])
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        win_ms = []
        torch.cuda.synchronize()
        if clocks:
            clocks.__enter__()
        wall0 = time.perf_counter()
        for k in range(steps):
            self.flush.zero_()
            evs[k][0].record(self.stream)
            step()
            evs[k][1].record(self.stream)
            win_ms.append(ctx.timing().ms_window)
        torch.cuda.synchronize()
        if clocks:
            clocks.__exit__()
        res["wall_s"] = time.perf_counter() - wall0
        res["total_ms"] = sum(e0.elapsed_time(e1) for e0, e1 in evs)
        res["ms_per_step"] = res["total_ms"] / steps
        res["window_ms"] = statistics.mean(win_ms)
        res["value"] = res["windows"] * steps / (res["total_ms"] / 1e3)
        res["out"] = out
        return res


def accuracy(got, ref, tol=1e-3):
    """max / rms |dv| on computed (vm = 1) and interpolated (vm = 0.5)
    pixels against the oracle, and mask equality."""
    vx, vy, vm = got
    ox, oy, om = ref
    comp = om == 1.0
    finite = np.isfinite(ox) & np.isfinite(oy)
    dv = np.where(finite, np.maximum(np.abs(vx - ox), np.abs(vy - oy)), 0.0)
    r = {"mask_equal": bool(np.array_equal(vm, om)),
         "max_dv_computed": float(dv[comp].max(initial=0.0)),
         "rms_dv_computed": float(np.sqrt(np.mean(dv[comp] ** 2))) if comp.any() else 0.0,
         "n_over_tol": int((dv[comp] > tol).sum())}
    if (om == 0.5).any():
        r["max_dv_interp"] = float(dv[om == 0.5].max())
    return r


def config_record(name, desc, f1, f2, kw_gpu, kw_oracle, a, runner_args, po):
    """Every window form on one frame pair: windows/s with inputs resident,
    accuracy against the FP64 oracle, and the oracle on one core."""
    from pyflct_gb300.flct import make_params
    ctx, dev, flush = runner_args
    r = DeviceRunner(ctx, dev, flush, f1, f2)
    steps = max(3, min(a.steps, 10))
    rec = {"workload": desc, "shape": list(f1.shape), "forms": {}}
    ref = po.velocity(f1, f2, nthreads=os.cpu_count(), **kw_oracle) if po else None
    for form in FORMS:
        p = make_params(1.0, 1.0, form=form, **kw_gpu)
        x = r.run(p, steps, 3)
        rec["windows_per_step"] = x["windows"]
        rec["box"] = x["box"]
        f = {"windows_s": x["value"], "ms_per_step": x["ms_per_step"], "window_ms": x["window_ms"]}
        if ref is not None:
            f["accuracy_vs_fp64_oracle"] = accuracy([o.cpu().numpy() for o in x["out"]], ref)
        rec["forms"][form] = f
    if po:
        t0 = time.perf_counter()
        po.velocity(f1, f2, nthreads=1, **kw_oracle)
        dt = time.perf_counter() - t0
        rec["cpu_1core"] = {"windows_s": rec["windows_per_step"] / dt, "cores": 1, "cpu": cpu_model(), "kind": "port",
                            "sample": "one full frame, " + CPU_SAMPLE}
    rec["tc_fp16_speedup_over_fp32_form"] = rec["forms"]["tc_fp16"]["windows_s"] / rec["forms"]["fp32"]["windows_s"]
    return rec


def run_config1(a, runner_args, po):
    from pyflct_gb300 import synth
    f1, f2, kw = synth.config1()
    return config_record("config1", "128x128 Gaussian blobs + noise, exact shift (0.3, -0.2), sigma=4 (box 16)",
                         f1, f2, dict(sigma=4.0), dict(sigma=4.0), a, runner_args, po)


def run_config2(a, runner_args, po):
    from pyflct_gb300 import synth
    rng = np.random.default_rng(20262)
    f1 = synth.config2_image1(rng)
    f2 = synth.spectral_warp(f1, *synth.rotation_shift(f1.shape, 0.01), runner_args[1].index or 0)
    return config_record("config2", "512x512 k^-2 field with 20% near-zero pixels, 0.01 deg rotation by the "
                         "spectral warp, sigma=8 (box 32), -t 0.1a -k 0.5", f1, f2,
                         dict(sigma=8.0, thresh="0.1a", kr=0.5),
                         dict(sigma=8.0, thresh=0.1, thresh_abs=True, kr=0.5), a, runner_args, po)


def run_batch(a, dev, flush, po):
    """The 64-pair heterogeneous workload (sides from {128..768}, sigma from
    {3, 5, 8, 12}, uniform sub-pixel shifts) as one batched call per step
    (a captured CUDA graph): windows/s with the inputs resident in HBM per
    window form, accuracy of 8 pairs against the oracle, and the oracle on
    one core and on every host core over a sample of pairs."""
    import torch
    from pyflct_gb300 import synth
    from pyflct_gb300.flct import FlctBatch, make_params
    pairs = synth.config4_pairs()
    stream = torch.cuda.current_stream(dev)
    boxes = sorted({box_of(kw["sigma"]) for _, _, kw, _ in pairs})
    flops = sum(window_flops(box_of(kw["sigma"])) * f1.size for f1, _, kw, _ in pairs)
    res = {"pairs": len(pairs), "boxes": boxes, "forms": {},
           "note": "inputs resident in HBM (179 MB > L2), L2 flushed between steps"}
    check = list(range(0, len(pairs), 8))
    refs = {k: po.velocity(pairs[k][0], pairs[k][1], nthreads=os.cpu_count(), sigma=pairs[k][2]["sigma"])
            for k in check} if po else {}
    for form in ("auto",) + FORMS:
        params = [make_params(1.0, 1.0, kw["sigma"], form=form) for _, _, kw, _ in pairs]
        b = FlctBatch([f1.shape for f1, _, _, _ in pairs], params, device=dev.index or 0)
        b.load([(f1, f2) for f1, f2, _, _ in pairs])
        for _ in range(3):
            b.run(stream)
        torch.cuda.synchronize()
        t = b.timing()
        windows, launches = int(t.windows), int(t.launches)
        steps = max(3, min(a.steps, 10))
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for k in range(steps):
            flush.zero_()
            evs[k][0].record(stream)
            b.run(stream)
            evs[k][1].record(stream)
        torch.cuda.synchronize()
        ms = sum(e0.elapsed_time(e1) for e0, e1 in evs) / steps
        f = {"windows_s": windows / (ms / 1e3), "ms_per_step": ms, "kernels_per_graph": launches,
             "algorithmic_tflops": flops / (ms / 1e3) / 1e12}
        if refs:
            worst = {"max_dv_computed": 0.0, "mask_equal": True}
            for k in check:
                got = (b.vx[k].cpu().numpy(), b.vy[k].cpu().numpy(), b.vm[k].cpu().numpy())
                acc = accuracy(got, refs[k])
                worst["max_dv_computed"] = max(worst["max_dv_computed"], acc["max_dv_computed"])
                worst["mask_equal"] &= acc["mask_equal"]
            worst["pairs_checked"] = len(check)
            f["accuracy_vs_fp64_oracle"] = worst
        res["forms"][form] = f
        res["windows_per_step"] = windows
        del b
        torch.cuda.empty_cache()
    # headline keys of this record: the autotuned form
    res.update({"value": res["forms"]["auto"]["windows_s"], "unit": "windows/s",
                "ms_per_step": res["forms"]["auto"]["ms_per_step"],
                "kernels_per_graph": res["forms"]["auto"]["kernels_per_graph"],
                "algorithmic_tflops": res["forms"]["auto"]["algorithmic_tflops"]})
    if po:
        sample = list(range(0, len(pairs), 4))
        nwin = 0
        t0 = time.perf_counter()
        for k in sample[:4]:
            o = po.velocity(pairs[k][0], pairs[k][1], nthreads=1, sigma=pairs[k][2]["sigma"])
            nwin += int((o[2] == 1).sum())
        one = nwin / (time.perf_counter() - t0)
        nwin = 0
        t0 = time.perf_counter()
        for k in sample:
            o = po.velocity(pairs[k][0], pairs[k][1], nthreads=os.cpu_count(), sigma=pairs[k][2]["sigma"])
            nwin += int((o[2] == 1).sum())
        allc = nwin / (time.perf_counter() - t0)
        res["cpu_1core"] = {"windows_s": one, "cores": 1, "cpu": cpu_model(), "kind": "port",
                            "sample": f"pairs {sample[:4]}, " + CPU_SAMPLE}
        res["cpu_nproc"] = {"windows_s": allc, "cores": os.cpu_count(), "cpu": cpu_model(), "kind": "port",
                            "sample": f"{len(sample)} of the 64 pairs, the oracle's windows on every host thread"}
    return res


def run_config5(a, runner_args, po):
    """4096^2 float32 k^-2 field, image2 by the GPU spectral warp along a
    k^-3 displacement field of RMS 0.3 px (its time is the warp's Mpixel/s),
    sigma 15 (box 64), every pixel a window (16.7M): windows/s per form,
    accuracy against the FP64 oracle's per-window correlation on a random
    1% of the pixels, the oracle's windows/s on one core over a sample."""
    import torch
    from pyflct_gb300 import synth
    from pyflct_gb300.flct import make_params
    ctx, dev, flush = runner_args
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    f1, f2, kw, _ = synth.config5(device=dev.index or 0)
    warp_s = time.perf_counter() - t0  # dominated by warp_frac2d (field synthesis on the host is ~2 s)
    rec = {"workload": "4096x4096 float32 k^-2 field, k^-3 displacement RMS 0.3 px by the GPU spectral "
                       "warp, sigma=15 (box 64), every pixel", "shape": list(f1.shape), "forms": {}}
    rec["warp_4096"] = {"seconds": warp_s, "mpix_s": f1.size / warp_s / 1e6,
                        "note": "synth.config5 wall time: warp_frac2d through the host-buffer C ABI plus "
                                "the field synthesis"}
    r = DeviceRunner(ctx, dev, flush, f1, f2)
    steps = max(2, min(a.steps, 3))
    pts = None
    if po:
        rng = np.random.default_rng(5)
        flat = rng.choice(f1.size, size=f1.size // 100, replace=False)
        pts = np.stack([flat // f1.shape[1], flat % f1.shape[1]], axis=1)
        sx, sy = np.empty(len(pts)), np.empty(len(pts))
        for b0 in range(0, len(pts), 4096):
            part = pts[b0:b0 + 4096]
            w = [po.extract_window(f1, f2, i, j, sigma=15.0) for i, j in part]
            sx[b0:b0 + len(part)], sy[b0:b0 + len(part)] = po.cross_cor_batch(
                np.stack([x for x, _ in w]), np.stack([y for _, y in w]))
        t0 = time.perf_counter()
        w = [po.extract_window(f1, f2, i, j, sigma=15.0) for i, j in pts[:400]]
        po.cross_cor_batch(np.stack([x for x, _ in w]), np.stack([y for _, y in w]), nthreads=1)
        rec["cpu_1core"] = {"windows_s": 400 / (time.perf_counter() - t0), "cores": 1, "cpu": cpu_model(), "kind": "port",
                            "sample": "400 of the sampled windows (extraction + cross_cor), " + CPU_SAMPLE}
    for form in ("fp32", "tc_fp16"):
        p = make_params(1.0, 1.0, 15.0, form=form)
        x = r.run(p, steps, 1)
        rec["windows_per_step"] = x["windows"]
        f = {"windows_s": x["value"], "ms_per_step": x["ms_per_step"], "window_ms": x["window_ms"]}
        if form == "tc_fp16":
            tf = tc_flops_per_window(64) * x["windows"] / (x["window_ms"] / 1e3) / 1e12
            pk, src = peaks()
            f["tensor_tflops_executed"] = tf
            f["tensor_pipe_frac_of_bf16_peak"] = tf / pk["bf16_tflops"]
        if pts is not None:
            vx, vy = x["out"][0].cpu().numpy(), x["out"][1].cpu().numpy()
            dv = np.maximum(np.abs(vx[pts[:, 0], pts[:, 1]] - sy), np.abs(vy[pts[:, 0], pts[:, 1]] - sx))
            f["accuracy_vs_fp64_oracle_1pct"] = {"pixels": int(len(pts)), "max_dv": float(dv.max()),
                                                 "rms_dv": float(np.sqrt(np.mean(dv ** 2))),
                                                 "n_over_1e-3": int((dv > 1e-3).sum())}
        rec["forms"][form] = f
        del x
    rec["tc_fp16_speedup_over_fp32_form"] = rec["forms"]["tc_fp16"]["windows_s"] / rec["forms"]["fp32"]["windows_s"]
    del r
    torch.cuda.empty_cache()
    return rec


def run_warp(a, dev):
    """The warp entry points on a 512^2 k^-2 field (the crop size the
    large-frame configuration checks the warp on): shift_frac2d with one
    uniform shift and warp_frac2d with a smooth per-pixel displacement
    (RMS 0.3 px), Mpixel/s per call through the host-buffer C ABI (copies
    included; the spectral warp is O(N^2) per pixel, so it dominates)."""
    from pyflct_gb300 import _lib, synth
    from pyflct_gb300.flct import shift_frac2d, warp_frac2d
    rng = np.random.default_rng(20265)
    img = synth.kfield((512, 512), rng)
    dfast, dslow = synth.smooth_shift(img.shape, rng, rms=0.3)
    out = {}
    for name, fn in (("shift_frac2d", lambda: shift_frac2d(img, 0.37, -2.6, device=dev.index or 0)),
                     ("warp_frac2d", lambda: warp_frac2d(img, dfast, dslow, device=dev.index or 0))):
        fn()
        reps = 3
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        dt = (time.perf_counter() - t0) / reps
        out[name] = {"mpix_s": img.size / dt / 1e6, "ms_per_call": dt * 1e3}
        if name == "warp_frac2d":
            # the spectral sum on the tensor cores: the half-spectrum GEMM's
            # executed flops (3 split products, 2 nx x 32 ceil((ny/2+1)/16)
            # real K per pixel) and the reference loop's 8 nx ny flops per pixel
            tm = _lib.context(dev.index or 0).timing()
            nx, ny = img.shape
            gemm = 6.0 * (2 * nx) * (32 * ((ny // 2 + 1 + 15) // 16)) * img.size
            pk, src = peaks()
            out[name].update({
                "sum_ms": tm.ms_window, "dft_ms": tm.ms_prepass,
                "tensor_tflops": gemm / (tm.ms_window * 1e-3) / 1e12,
                "tensor_frac_of_bf16_peak": gemm / (tm.ms_window * 1e-3) / 1e12 / pk["bf16_tflops"],
                "peak_source": f"{src} bf16_tflops (dense 16-bit rate)",
                "reference_equivalent_tflops": 8.0 * nx * ny * img.size / (tm.ms_window * 1e-3) / 1e12})
    out["size"] = list(img.shape)
    out["note"] = "host buffers in and out, wall clock per call"
    # a 4096^2 uniform shift: power-of-two axes take the transform path
    big = synth.kfield((4096, 4096), rng)
    shift_frac2d(big, 0.37, -2.6, device=dev.index or 0)
    walls, devs = [], []
    for _ in range(3):
        t0 = time.perf_counter()
        shift_frac2d(big, 0.37, -2.6, device=dev.index or 0)
        walls.append(time.perf_counter() - t0)
        devs.append(_lib.context(dev.index or 0).timing().ms_total)
    out["shift_frac2d_4096"] = {"ms_per_call": min(walls) * 1e3, "device_ms": min(devs),
                                "mpix_s_device": big.size / (min(devs) / 1e3) / 1e6,
                                "note": "wall clock with 134 MB copied each way; device_ms = the kernels alone"}
    return out


def run_ours(a):
    import torch
    from pyflct_gb300 import _lib
    from pyflct_gb300.flct import make_params

    ws, rank, local = dist_init()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    ctx = _lib.context(local)
    lib = ctx.lib
    dev = torch.device("cuda", local)
    f1, f2 = workload(local)
    npx = f1.size
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    runner = DeviceRunner(ctx, dev, flush, f1, f2)
    forms = [a.form] + [f for f in FORMS if f != a.form and not a.only]
    res = {}
    clk = None
    for form in forms:
        p = make_params(1.0, 1.0, SIGMA, skip=SKIP, form=form)
        barrier()
        clocks = Clocks(local) if form == a.form else None
        r = runner.run(p, a.steps, a.warmup, clocks)
        if clocks:
            clk = clocks
        r["total_ms"] = reduce_max(r["total_ms"], dev)
        r["value"] = r["windows"] * a.steps * ws / (r["total_ms"] / 1e3)
        r["ms_per_step"] = r["total_ms"] / a.steps
        res[form] = r

    head = res[a.form]
    windows, launches, box = head["windows"], head["launches"], head["box"]
    p = make_params(1.0, 1.0, SIGMA, skip=SKIP, form=a.form)

    # end to end through the host-buffer entry point with pinned buffers
    pin = [torch.empty(NSIDE, NSIDE, dtype=torch.float64, pin_memory=True) for _ in range(5)]
    pin[0].copy_(torch.from_numpy(f1))
    pin[1].copy_(torch.from_numpy(f2))
    ptr = [C.cast(C.c_void_p(x.data_ptr()), C.POINTER(C.c_double)) for x in pin]

    def e2e_step():
        ctx.check(lib.flct_gpu_velocity(ctx.h, C.byref(p), ptr[0], ptr[1], NSIDE, NSIDE,
                                        ptr[2], ptr[3], ptr[4]))

    for _ in range(3):
        e2e_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(a.steps):
        flush.zero_()
        torch.cuda.synchronize()
        e2e_step()
    barrier()
    e2e_s = time.perf_counter() - t0
    t1 = time.perf_counter()
    for _ in range(a.steps):
        flush.zero_()
        torch.cuda.synchronize()
    flush_s = time.perf_counter() - t1
    e2e_val = windows * a.steps * ws / max(1e-9, reduce_max(e2e_s - flush_s, dev))

    if rank != 0:
        if ws > 1:
            torch.distributed.destroy_process_group()
        return

    po = None if a.no_cpu else oracle()
    runner_args = (ctx, dev, flush)
    configs = {}
    if not a.no_configs:
        configs["config1"] = run_config1(a, runner_args, po)
        configs["config2"] = run_config2(a, runner_args, po)
    batch = None if a.no_batch else run_batch(a, dev, flush, po)
    if batch is not None:
        configs["config4"] = batch
    if not (a.no_batch or a.no_configs):
        configs["config5"] = run_config5(a, runner_args, po)
    warp = None if a.no_batch else run_warp(a, dev)

    pk, src = peaks()
    fl = window_flops(box)
    nsm = torch.cuda.get_device_properties(dev).multi_processor_count
    fp32pk = measured_fp32_peak()
    copies = measured_copy_peaks(dev, 2 * NSIDE * NSIDE * 8, 3 * NSIDE * NSIDE * 8)

    def roofline(form):
        r = res[form]
        form = r["used"]
        achieved = r["windows"] * fl / (r["window_ms"] / 1e3) / 1e12
        if form == "fp32":
            if fp32pk:
                peak = fp32pk["tflops"]
                psrc = ("measured here: libflctprobe.so FMA chains (best of scalar and packed f32x2), "
                        "CUDA events")
            else:
                peak = nsm * 128 * 2 * pk.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
                psrc = f"derived: {nsm} SMs x 128 FP32 lanes x 2 x {pk.get('sm_max_mhz')} MHz"
            return {"bound": "fp32", "kernel": f"k_window_fp32<{box}>", "achieved": achieved, "peak": peak,
                    "unit": "TFLOP/s", "frac": achieved / peak, "flops_per_window": fl,
                    "window_ms": r["window_ms"], "peak_source": psrc}
        peak = pk["bf16_tflops"]
        tfl = tc_flops_per_window(box)
        tensor = r["windows"] * tfl / (r["window_ms"] / 1e3) / 1e12
        return {"bound": "tensor", "kernel": f"k_window_tc<{box}, {'half' if form == 'tc_fp16' else 'bf16'}>",
                "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "flops_per_window": fl, "window_ms": r["window_ms"],
                "tensor_flops_per_window": tfl, "tensor_achieved": tensor,
                "tensor_frac": tensor / peak, "peak_source": f"{src} bf16_tflops (dense 16-bit rate)"}

    rl = roofline(a.form)
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    rl["traffic"] = None
    if os.path.exists(tp):
        with open(tp) as fh:
            rl["traffic"] = json.load(fh).get(f"window_{head['used']}_n{box}")

    # accuracy against the FP64 oracle on the same frame, and the CPU baseline
    acc, cpu = {}, None
    if po:
        kw = dict(sigma=SIGMA, skip=4, interpolate=True)
        ref = po.velocity(f1, f2, nthreads=os.cpu_count(), **kw)
        for form, r in res.items():
            acc[form] = accuracy([x.cpu().numpy() for x in r["out"]], ref)
        t0 = time.perf_counter()
        po.velocity(f1, f2, nthreads=1, **kw)
        cdt = time.perf_counter() - t0
        cpu = {"value": windows / cdt, "unit": "windows/s", "cores": 1, "cpu": cpu_model(), "kind": "port",
               "sample": "one full frame (65,536 windows + interpolation), 1 thread, C restatement "
                         "of flct.c over the project double FFT (FFTW unavailable)"}

    # e2e against its bound: the step's copies (both directions at once, as
    # measured) or the device step, whichever is longer
    h2d, d2h = 2 * npx * 8, 3 * npx * 8
    copy_ms = copies["step_copies_ms"]
    bound_ms = max(copy_ms, head["ms_per_step"])
    e2e_ms = windows / e2e_val * 1e3

    line = {
        "metric": METRIC, "value": head["value"], "unit": "windows/s", "n_gpus": ws, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp32": "f32", "tc_fp16": "f16x2 split (f32 accumulate)",
                  "tc_bf16": "bf16x2 split (f32 accumulate)"}[head["used"]],
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "form": a.form, "form_used": head["used"], "box": box,
                   "windows_per_step": windows,
                   "output_pixels_per_step": npx, "l2": "flushed (256 MiB write) between steps",
                   "parallelism": f"replicas x{ws}"},
        "e2e": {"value": e2e_val, "unit": "windows/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_ms, "bound_ms": bound_ms, "copy_bound_ms": copy_ms,
                "frac_of_bound": bound_ms / e2e_ms},
        "roofline": rl,
        "measured_peaks": {"fp32": fp32pk, "pinned_copies": copies},
        "forms": {f: {"value": r["value"], "ms_per_step": r["ms_per_step"], "window_ms": r["window_ms"],
                      "used": r["used"]} for f, r in res.items()},
        "configs": configs,
        "batch_64_pairs": batch,
        "warp_512": warp,
        "cpu_baseline": cpu,
        "accuracy_vs_fp64_oracle": acc,
        "gpu_launches": launches * a.steps,
        "clocks": clk.summary() if clk else None,
        "wall_s_timed": head["wall_s"],
        "output_pixels_per_s": head["value"] / windows * npx,
    }
    if "fp32" in res and "tc_fp16" in res:
        line["tc_fp16_speedup_over_fp32_form"] = res["tc_fp16"]["value"] / res["fp32"]["value"]
        line["tc_fp16_window_kernel_speedup_over_fp32"] = res["fp32"]["window_ms"] / res["tc_fp16"]["window_ms"]
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="auto", choices=["auto", "fp32", "tc_fp16", "tc_bf16"])
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the 64-pair batch, the 4096^2 configuration and the warp timing")
    ap.add_argument("--no-configs", action="store_true", help="skip configurations 1, 2 and 5")
    ap.add_argument("--only", action="store_true", help="time only --form (skip the other forms)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the oracle accuracy and CPU baselines")
    a = ap.parse_args()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
