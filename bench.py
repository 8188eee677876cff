#!/usr/bin/env python
"""FLCT velocity vectors/s on one GB300: the headline workload.

Workload (one "step" = the whole flct computation on one frame pair):
1024 x 1024 float64 k^-2 random field, image2 = image1 advected by five
Gaussian vortices, sigma = 8 (box 32), -s 4i (every 4th pixel correlated,
the rest cubic-convolution interpolated), thresh = 0.  That is 65,536
correlation windows and 1,048,576 output pixels per step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--form auto|fp32|tc_fp16|tc_bf16]
    python bench.py --impl reference ...   # the CPU implementation arm

value  = correlation windows per second with inputs resident in HBM
         (flct_gpu_velocity_device, CUDA events per step on the launch
         stream, L2 flushed with a 256 MiB write between steps).
e2e    = the same metric through flct_gpu_velocity with pinned host
         buffers: both input frames copied in and vx, vy, vm copied out
         every step.
Beside the headline line's keys: the 64-pair heterogeneous batch
(batch_64_pairs) and the warp entry points' Mpixel/s at 512^2 (warp_512);
--no-batch skips both.
"""
from __future__ import annotations

import argparse
import ctypes as C
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

WORKLOAD = "1024x1024 k^-2 field, 5-vortex warp, sigma=8 (box 32), -s 4i, thresh 0"
METRIC = "FLCT velocity vectors/s (correlation windows/s) at 1024^2 sigma=8"
NSIDE, SIGMA, SKIP = 1024, 8.0, "4i"
# algorithmic flops of one n x n window: 3 real transforms at 2.5 M log2 M,
# M = n^2, plus means (2n^2), windowing (4n^2), conj product (4n^2), |c| and
# argmax (2n^2); 4 n (n/2+1) more with -k.
def window_flops(n: int, kr: bool = False) -> float:
    m = n * n
    f = 7.5 * m * np.log2(m) + 12 * m
    return f + (4 * n * (n // 2 + 1) if kr else 0)


def workload():
    from pyflct_gb300 import synth
    rng = np.random.default_rng(20263)
    f1 = synth.kfield((NSIDE, NSIDE), rng)
    dfast, dslow = synth.vortex_shift(f1.shape, rng)
    f2 = synth.spline_warp(f1, dfast, dslow)
    return np.ascontiguousarray(f1), np.ascontiguousarray(f2)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            return json.load(fh), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
            "sm_max_mhz": 2070.0}, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        cmd = ["nvidia-smi", "-i", str(self.index),
               "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
               "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
               "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "100"]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
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


def oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    po.build()
    return po


def run_reference(a):
    """The reference arm: the CPU implementation of the path (the oracle's
    C restatement of flct.c; the reference itself cannot be compiled on the
    GPU host because its sources do not travel there) on all host threads."""
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
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "windows/s", "n_gpus": ws,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * dt / a.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": WORKLOAD, "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": v, "unit": "windows/s", "cores": threads, "kind": "port",
                         "sample": "full frame per step (65,536 windows + interpolation), "
                                   f"{threads} threads, C restatement of flct.c over the "
                                   "project double FFT (FFTW unavailable)"},
        "e2e": {"value": v, "unit": "windows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# MMA work the tensor-core form executes per 32x32 window: four M=128 GEMM
# stages over 8 windows, each product as hi*hi + hi*lo + lo*hi.
TC_MACS_PER_8 = 3 * (4 * 128 * 32 * 32 + 2 * 128 * 64 * 64 + 128 * 64 * 64 + 2 * 128 * 32 * 32)
TC_FLOPS_PER_WINDOW = 2 * TC_MACS_PER_8 / 8


def run_batch(a, dev, flush):
    """The 64-pair heterogeneous workload (sides from {128..768}, sigma from
    {3, 5, 8, 12}, uniform sub-pixel shifts) as one batched call: windows/s
    with the inputs resident in HBM, one captured CUDA graph per step."""
    import torch
    from pyflct_gb300 import synth
    from pyflct_gb300.flct import FlctBatch, make_params
    pairs = synth.config4_pairs()
    params = [make_params(1.0, 1.0, kw["sigma"], form="auto") for _, _, kw, _ in pairs]
    b = FlctBatch([f1.shape for f1, _, _, _ in pairs], params, device=dev.index or 0)
    b.load([(f1, f2) for f1, f2, _, _ in pairs])
    stream = torch.cuda.current_stream(dev)
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
    def box(sigma):  # n = 2 nsize, nsize = even part of (int)((int)sigma sqrt(ln 100))
        return 2 * (int(int(sigma) * np.sqrt(np.log(100.0))) // 2 * 2)

    boxes = sorted({box(kw["sigma"]) for _, _, kw, _ in pairs})
    flops = sum(window_flops(box(kw["sigma"])) * f1.size for f1, _, kw, _ in pairs)
    return {"pairs": len(pairs), "windows_per_step": windows, "value": windows / (ms / 1e3),
            "unit": "windows/s", "ms_per_step": ms, "steps": steps, "kernels_per_graph": launches,
            "boxes": boxes, "algorithmic_tflops": flops / (ms / 1e3) / 1e12,
            "note": "inputs resident in HBM (179 MB > L2), L2 flushed between steps, form auto"}


def run_warp(a, dev):
    """The warp entry points on a 512^2 k^-2 field (the crop size the
    large-frame configuration checks the warp on): shift_frac2d with one
    uniform shift and warp_frac2d with a smooth per-pixel displacement
    (RMS 0.3 px), Mpixel/s per call through the host-buffer C ABI (copies
    included; the spectral warp is O(N^2) per pixel, so it dominates)."""
    from pyflct_gb300 import synth
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
    out["size"] = list(img.shape)
    out["note"] = "host buffers in and out, wall clock per call"
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
    f1, f2 = workload()
    npx = f1.size
    dev = torch.device("cuda", local)
    d_f1 = torch.from_numpy(f1).to(dev)
    d_f2 = torch.from_numpy(f2).to(dev)
    outs = {}
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    sh = C.c_void_p(stream.cuda_stream)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    forms = [a.form] + [f for f in ("fp32", "tc_fp16", "tc_bf16") if f != a.form and not a.only]
    names = {v: k for k, v in _lib.FORMS.items()}
    res = {}
    clk = None
    for form in forms:
        p = make_params(1.0, 1.0, SIGMA, skip=SKIP, form=form)
        d_out = [torch.empty(NSIDE, NSIDE, dtype=torch.float64, device=dev) for _ in range(3)]
        outs[form] = d_out

        def step():
            ctx.check(lib.flct_gpu_velocity_device(
                ctx.h, C.byref(p), C.c_void_p(d_f1.data_ptr()), C.c_void_p(d_f2.data_ptr()), NSIDE, NSIDE,
                C.c_void_p(d_out[0].data_ptr()), C.c_void_p(d_out[1].data_ptr()),
                C.c_void_p(d_out[2].data_ptr()), sh))

        for _ in range(max(3, a.warmup)):
            step()
        torch.cuda.synchronize()
        t = ctx.timing()
        windows, launches, box = int(t.windows), int(t.launches), int(t.box)
        used = names[int(t.form)]  # the autotuner's choice for "auto"
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(a.steps)]
        win_ms = []
        barrier()
        wall0 = time.perf_counter()
        clocks = Clocks(local) if form == a.form else None
        if clocks:
            clocks.__enter__()
        for k in range(a.steps):
            flush.zero_()  # L2 flush between steps (outside the step's events)
            evs[k][0].record(stream)
            step()
            evs[k][1].record(stream)
            win_ms.append(ctx.timing().ms_window)
        barrier()
        if clocks:
            clocks.__exit__()
            clk = clocks
        wall = time.perf_counter() - wall0
        total_ms = sum(e0.elapsed_time(e1) for e0, e1 in evs)
        total_ms = reduce_max(total_ms, dev)
        res[form] = dict(value=windows * a.steps * ws / (total_ms / 1e3), ms_per_step=total_ms / a.steps,
                         window_ms=statistics.mean(win_ms), windows=windows, launches=launches, box=box,
                         wall_s=wall, used=used)

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

    batch = None if a.no_batch else run_batch(a, dev, flush)
    warp = None if (a.no_batch or rank != 0) else run_warp(a, dev)

    if rank != 0:
        if ws > 1:
            torch.distributed.destroy_process_group()
        return

    pk, src = peaks()
    fl = window_flops(box)
    nsm = torch.cuda.get_device_properties(dev).multi_processor_count

    def roofline(form):
        r = res[form]
        form = r["used"]
        achieved = r["windows"] * fl / (r["window_ms"] / 1e3) / 1e12
        if form == "fp32":
            peak = nsm * 128 * 2 * pk.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
            return {"bound": "fp32", "kernel": f"k_window_fp32<{box}>", "achieved": achieved, "peak": peak,
                    "unit": "TFLOP/s", "frac": achieved / peak, "flops_per_window": fl,
                    "window_ms": r["window_ms"],
                    "peak_source": f"derived: {nsm} SMs x 128 FP32 lanes x 2 x {pk.get('sm_max_mhz')} MHz "
                                   f"({src} max clock); no FP32 figure in MEASURED_PEAKS.json"}
        peak = pk["bf16_tflops"]
        tensor = r["windows"] * TC_FLOPS_PER_WINDOW / (r["window_ms"] / 1e3) / 1e12
        return {"bound": "tensor", "kernel": f"k_window_tc32<{'half' if form == 'tc_fp16' else 'bf16'}>",
                "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "flops_per_window": fl, "window_ms": r["window_ms"],
                "tensor_flops_per_window": TC_FLOPS_PER_WINDOW, "tensor_achieved": tensor,
                "tensor_frac": tensor / peak, "peak_source": f"{src} bf16_tflops (dense 16-bit rate)"}

    rl = roofline(a.form)
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp):
        with open(tp) as fh:
            rl["traffic"] = json.load(fh).get(f"window_{head['used']}_n{box}")
    else:
        rl["traffic"] = None

    # accuracy against the FP64 oracle on the same frame, and the CPU baseline
    acc, cpu = {}, None
    if not a.no_cpu:
        po = oracle()
        kw = dict(sigma=SIGMA, skip=4, interpolate=True)
        ref = po.velocity(f1, f2, nthreads=os.cpu_count(), **kw)
        comp = ref[2] == 1.0
        for form, d_out in outs.items():
            got = [x.cpu().numpy() for x in d_out]
            dv = np.maximum(np.abs(got[0] - ref[0]), np.abs(got[1] - ref[1]))
            acc[form] = {"mask_equal": bool(np.array_equal(got[2], ref[2])),
                         "max_dv_computed": float(dv[comp].max()),
                         "rms_dv_computed": float(np.sqrt(np.mean(dv[comp] ** 2))),
                         "n_over_1e-3": int((dv[comp] > 1e-3).sum()),
                         "max_dv_interp": float(dv[ref[2] == 0.5].max())}
        t0 = time.perf_counter()
        po.velocity(f1, f2, nthreads=1, **kw)
        cdt = time.perf_counter() - t0
        cpu = {"value": windows / cdt, "unit": "windows/s", "cores": 1, "kind": "port",
               "sample": "one full frame (65,536 windows + interpolation), 1 thread, C restatement "
                         "of flct.c over the project double FFT (FFTW unavailable)"}

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
        "e2e": {"value": e2e_val, "unit": "windows/s", "h2d_bytes_per_step": 2 * npx * 8,
                "d2h_bytes_per_step": 3 * npx * 8},
        "roofline": rl,
        "forms": {f: {"value": r["value"], "ms_per_step": r["ms_per_step"], "window_ms": r["window_ms"],
                      "used": r["used"]} for f, r in res.items()},
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
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="auto", choices=["auto", "fp32", "tc_fp16", "tc_bf16"])
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-pair batched workload and the warp timing")
    ap.add_argument("--only", action="store_true", help="time only --form (skip the other forms)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the oracle accuracy and CPU baseline")
    a = ap.parse_args()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
