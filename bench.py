#!/usr/bin/env python
"""Benchmark: 3-D Richardson-Lucy deconvolution in FP32 on one GB300.

Workload (the 3-D RL configuration): a 256x256x64 volume of 200 ellipsoids (radii 2-20,
intensities 50-1000) on background 10, blurred by a normalised anisotropic Gaussian PSF
15x15x7 (sigma 2, 2, 1) with Poisson noise; flat start at the mean; 50 iterations of
non-separable direct convolution, zero border. One step = one complete 50-iteration run
(100 fused convolution passes). Data are synthetic and seeded.

Metric: convolution throughput in GVoxel/s = output voxels of all convolutions in the
step (2 per iteration) / time. `value` is device time (CUDA events) with inputs resident
in HBM and L2 flushed (a 256 MB write) before every step; `e2e` is the same metric through
the C-ABI host entry point (pinned host observed image in, host estimate out, both copies
inside the timed region).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
N > 1 runs under torchrun as independent replicas (the RL volume does not shard); the
reference arm times the reference's CPU implementation (the oracle port, all host threads)
on rank 0 only.
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
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

SHAPE_XYZ = (256, 256, 64)
PSF_XYZ = (15, 15, 7)
ITERATIONS = 50
EPSILON = 1e-6
VOXELS = SHAPE_XYZ[0] * SHAPE_XYZ[1] * SHAPE_XYZ[2]
TAPS = PSF_XYZ[0] * PSF_XYZ[1] * PSF_XYZ[2]
METRIC = "Conv GVoxel/s (3-D RL FP32, fused passes)"
UNIT = "GVoxel/s"
WORKLOAD = "rl3d_f32_256x256x64_psf15x15x7_50it"
CPU_ITERATIONS = 6  # CPU baseline sample: RL iterations over the full volume (13 convolutions)


def config(extra=None):
    c = {
        "workload": WORKLOAD,
        "volume_xyz": list(SHAPE_XYZ),
        "psf_xyz": list(PSF_XYZ),
        "psf_sigma_xyz": [2.0, 2.0, 1.0],
        "iterations": ITERATIONS,
        "init": "flat start at mean",
        "border": "zero",
        "l2": "flushed before every timed step (256 MB write)",
        "parallelism": "replicas",
    }
    if extra:
        c.update(extra)
    return c


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 8:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "", 1).isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "", 1).isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[4 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text()), "measured"
        except ValueError:
            pass
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


def recorded_traffic():
    """Per-launch DRAM bytes of the fused pass from the committed ncu summary, if any."""
    p = ROOT / "profiles" / "traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text()).get(WORKLOAD)
        except ValueError:
            return None
    return None


_FP32_PEAK = {}


def fp32_peak_tflops(dev):
    """The FP32 FMA ceiling of this GPU, measured by the library's probe (independent FMA
    chains on every lane; scalar FFMA and the packed two-lane form), with the nominal figure
    from the SM count and the maximum clock beside it. Measured once per process."""
    if "peak" not in _FP32_PEAK:
        import torch

        import iane_gb300

        with torch.cuda.device(dev):
            scalar = iane_gb300.fp32_peak(paired=False)
            paired = iane_gb300.fp32_peak(paired=True)
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        peaks, _ = measured_peaks()
        nominal = sms * 128 * 2 * float(peaks.get("sm_max_mhz", 2070.0)) * 1e6 / 1e12
        _FP32_PEAK.update({"peak": max(scalar, paired), "scalar_ffma": scalar, "paired_ffma2": paired,
                           "nominal": nominal, "sms": sms})
    return _FP32_PEAK


def reference_kind() -> str:
    """"reference" when the reference's own library (its headers compiled into oracle/_ref)
    loads on this host, else "port" (the C restatement pinned to it). The library is built
    where the reference's headers are; a GPU host of another CPU architecture has the port."""
    import oracle

    if oracle.reference_available():
        try:
            oracle.ref_lib()
            return "reference"
        except OSError:
            return "port"
    return "port"


def cpu_sample(observed, psf, threads, iterations):
    """The reference's RL loop (its own library where it loads, else the oracle port; all host
    threads) over the full volume: the sensitivity convolution plus `iterations` iterations of
    two convolutions each."""
    import oracle

    use_reference = reference_kind() == "reference"
    t0 = time.perf_counter()
    oracle.rl(observed, psf, iterations, EPSILON, init=oracle.abi.RL_INIT_MEAN, threads=threads,
              use_reference=use_reference)
    dt = time.perf_counter() - t0
    convs = 1 + 2 * iterations
    return convs * observed.size / dt / 1e9, dt


def max_over_ranks(value: float, dist, device) -> float:
    """The largest of every rank's `value` (the job's time is its slowest replica's); the value
    itself on a single process."""
    if dist is None:
        return value
    import torch

    t = torch.tensor([value], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(world: int, units_per_step: float, steps: int, seconds: float) -> float:
    """Whole-job throughput of `world` replicas that each ran `steps` steps of `units_per_step`
    units, the slowest taking `seconds`: giga-units per second."""
    return world * units_per_step * steps / seconds / 1e9


def run_reference(args, rank):
    """Reference arm: the reference's CPU RL path -- its own library built from its headers
    where that loads, else the oracle port pinned to it (the headers exist only where the
    reference checkout is, and the GPU host has another CPU architecture) -- on all host
    threads; each step is one RL iteration over the full volume. The reference's own CUDA
    convolution kernel is timed beside it on the GPU (`gpu_reference_kernel`)."""
    if rank != 0:
        return
    import numpy as np  # noqa: F401

    from iane_gb300 import synth
    from oracle import build as oracle_build

    import oracle

    oracle_build.build_oracle()
    threads = oracle.default_threads()
    observed, psf, _ = synth.rl_volume_workload(seed=0)
    # each step: one RL iteration over the full volume (its sensitivity convolution included)
    for _ in range(args.warmup):
        cpu_sample(observed, psf, threads, 1)
    total = 0.0
    for _ in range(args.steps):
        _, dt = cpu_sample(observed, psf, threads, 1)
        total += dt
    value = 3 * VOXELS * args.steps / total / 1e9
    sample = "one RL iteration (3 full-volume 15x15x7 convolutions incl. sensitivity) per step"
    gpu_reference = reference_gpu_kernel(observed, psf)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64 accumulate",
        "data": "synthetic", "config": config(),  # this arm's config: the sample is in cpu_baseline
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": reference_kind(), "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_reference_kernel": gpu_reference,
    }
    print(json.dumps(line), flush=True)


def reference_gpu_kernel(observed, psf, reps=3):
    """The reference's own CUDA convolution (its visit_positions kernel with the convolve functor,
    built from its headers into a cubin) timed on this GPU on the workload's convolution: the
    observed volume with the 15x15x7 PSF, zero border. CUDA events, after one warm-up. None when
    the cubin or a GPU is absent."""
    try:
        import torch

        from oracle import ref_gpu
    except ImportError:
        return None
    if not ref_gpu.available() or not torch.cuda.is_available():
        return {"unavailable": "the reference cubin is built only where the reference's headers are"}
    ref = ref_gpu.ReferenceConvolution()
    src = torch.from_numpy(observed).cuda()
    ker = torch.from_numpy(psf).cuda()
    dst = torch.empty_like(src)
    ref.convolve(src, ker, dst, "zero")
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        ref.convolve(src, ker, dst, "zero")
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / reps
    ref.close()
    return {"ms_per_convolution": ms, "gvoxel_s": VOXELS / (ms / 1e3) / 1e9,
            "kernel": "the reference's visit_positions with iane::convolve's functor (f32 views, FP64 fma per tap),"
                      " nvcc sm_103a from its headers, one thread per voxel, 256-thread blocks",
            "workload": "one 256x256x64 convolution with the 15x15x7 PSF, zero border"}


def measure_hbm_legs(dev, stream, reps=20, cpu=True):
    """HBM-bound convolutions beside the main workload: the fused separable kernel on a
    512^3 f32 volume (7-tap Gaussians, mirror border; 1 GiB in + out, larger than L2), the
    2-D 512x512 7x7 Gaussian mirror configuration, direct and separable (with the host
    baseline: the oracle port of the reference's convolve on all host threads and on one),
    and the same 2-D filter at 8192x8192 where bandwidth dominates. Device time per
    launch (CUDA events), algorithmic bytes = 8 per voxel (one read, one write)."""
    import numpy as np
    import torch

    import iane_gb300
    from iane_gb300 import synth

    peaks, _ = measured_peaks()
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    g1 = torch.from_numpy(synth.gaussian_psf((7,), (1.5,))).to(dev)
    g2 = torch.from_numpy(synth.gaussian_psf((7, 7), (1.5, 1.5))).to(dev)
    out = {}

    def timed(fn):
        for _ in range(3):
            fn()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        torch.cuda.synchronize(dev)
        return a.elapsed_time(b) / reps

    gen = torch.Generator(device=dev)
    gen.manual_seed(0)
    vol = torch.rand((512, 512, 512), generator=gen, device=dev, dtype=torch.float32)
    dst = torch.empty_like(vol)
    ms = timed(lambda: iane_gb300.convolve_separable(vol, [g1, g1, g1], dst, "mirror", stream=stream))
    gbs = 8.0 * vol.numel() / (ms / 1e3) / 1e9
    out["separable_512^3_7tap_mirror"] = {"ms": ms, "gvoxel_s": vol.numel() / (ms / 1e3) / 1e9, "gbs": gbs,
                                          "hbm_frac": gbs / hbm}
    del vol, dst
    def graph_timed(fn):
        """Device time per call of a launch too short to time one call at a time from Python
        (the host call takes longer than the kernel): `reps` calls captured in a CUDA graph and
        replayed between CUDA events. None if the capture fails."""
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        try:
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=side):
                for _ in range(reps):
                    fn()
        except Exception:
            return None
        with torch.cuda.stream(side):
            g.replay()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(side)
            g.replay()
            b.record(side)
        torch.cuda.synchronize(dev)
        return a.elapsed_time(b) / reps

    img = torch.rand((512, 512), generator=gen, device=dev, dtype=torch.float32)
    d2 = torch.empty_like(img)
    for name, fn in (("direct_512^2_7x7_mirror", lambda: iane_gb300.convolve(img, g2, d2, "mirror")),
                     ("separable_512^2_7x7_mirror", lambda: iane_gb300.convolve_separable(img, [g1, g1], d2, "mirror"))):
        with torch.cuda.stream(stream):
            call_ms = timed(fn)
        dev_ms = graph_timed(fn)
        ms = dev_ms if dev_ms is not None else call_ms
        out[name] = {"ms": ms, "gvoxel_s": img.numel() / (ms / 1e3) / 1e9, "api_call_ms": call_ms,
                     "timing": "CUDA graph of 20 calls" if dev_ms is not None else "20 calls through the Python API"}
    if cpu:
        # the 2-D configuration on the host: the reference's convolve (oracle port) with all
        # host threads and with one
        import oracle
        from oracle import build as oracle_build

        oracle_build.build_oracle()
        src_np = img.cpu().numpy()
        k_np = g2.cpu().numpy()
        ref_np = np.zeros_like(src_np)
        for threads in (oracle.default_threads(), 1):
            oracle.convolve(src_np, k_np, ref_np, "mirror", threads=threads)
            t0 = time.perf_counter()
            n = 0
            while time.perf_counter() - t0 < 1.0:
                oracle.convolve(src_np, k_np, ref_np, "mirror", threads=threads)
                n += 1
            cms = (time.perf_counter() - t0) / n * 1e3
            key = "cpu_baseline_all_threads" if threads > 1 else "cpu_baseline_1_thread"
            out["direct_512^2_7x7_mirror"][key] = {"ms": cms, "cores": threads, "kind": "port",
                                                   "gvoxel_s": img.numel() / (cms / 1e3) / 1e9}
        out["direct_512^2_7x7_mirror"]["gpu_speedup_vs_all_threads"] = (
            out["direct_512^2_7x7_mirror"]["cpu_baseline_all_threads"]["ms"] / out["direct_512^2_7x7_mirror"]["ms"])
    del img, d2
    # bandwidth at a large 2-D size (256 MiB in, 256 MiB out: larger than L2)
    big = torch.rand((8192, 8192), generator=gen, device=dev, dtype=torch.float32)
    dbig = torch.empty_like(big)
    fp32 = fp32_peak_tflops(dev)["peak"]
    for name, fn, flop in (("direct_8192^2_7x7_mirror", lambda: iane_gb300.convolve(big, g2, dbig, "mirror", stream=stream),
                            2 * 49),
                           ("separable_8192^2_7x7_mirror",
                            lambda: iane_gb300.convolve_separable(big, [g1, g1], dbig, "mirror", stream=stream), 2 * 14)):
        ms = timed(fn)
        gbs = 8.0 * big.numel() / (ms / 1e3) / 1e9
        tflops = flop * big.numel() / (ms / 1e3) / 1e12
        # 98 flop per 8 bytes puts the direct 7x7 filter at this GPU's FP32 / HBM ridge: both
        # fractions are stated
        out[name] = {"ms": ms, "gvoxel_s": big.numel() / (ms / 1e3) / 1e9, "gbs": gbs, "hbm_frac": gbs / hbm,
                     "tflops": tflops, "fp32_frac": tflops / fp32}
    del big, dbig
    return out


def measure_bf16_leg(dev, stream, reps=5, cpu=True):
    """The 3-D RL precision path: 256x256x64, PSF 9x9x9 sigma 2.5, 50 iterations, BF16
    images and PSF in tcgen05 implicit-GEMM convolutions (FP32 accumulation), beside the
    FP32 SIMT path on the same input. With `cpu`, the CPU baseline of this configuration is
    the reference's RL loop (the oracle port: FP64-accumulated convolutions, all host
    threads) run for all 50 iterations on the same input, and both GPU results state their
    max-abs and relative-L2 error against it."""
    import numpy as np
    import torch

    import iane_gb300
    from iane_gb300 import synth

    observed, psf, _ = synth.rl_volume_workload_bf16(seed=0)
    obs = torch.from_numpy(observed).to(dev)
    p = torch.from_numpy(psf).to(dev)
    out = {}
    results = {}
    for precision in ("bf16", "f32"):
        rl = iane_gb300.RichardsonLucy(p, observed.shape, precision=precision)
        scratch = torch.empty(rl.scratch_bytes, dtype=torch.uint8, device=dev)
        est = torch.empty(observed.shape, dtype=torch.float32, device=dev)
        run = lambda: rl.run(obs, est, ITERATIONS, EPSILON, init=rl.INIT_MEAN, scratch=scratch, stream=stream)
        for _ in range(2):
            run()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            run()
        b.record(stream)
        torch.cuda.synchronize(dev)
        ms = a.elapsed_time(b) / reps
        results[precision] = est.double()
        out[precision] = {"ms_per_run": ms, "gvoxel_s": 2 * ITERATIONS * observed.size / (ms / 1e3) / 1e9,
                          "tflops_useful": 2 * ITERATIONS * observed.size * 2 * psf.size / (ms / 1e3) / 1e12}
        if precision == "bf16":
            # banded-Toeplitz GEMMs: per output voxel and kernel row (ky x kz rows), an MMA
            # slice of K = 32 input columns for 16 outputs, i.e. 32 issued MACs per output
            kz, ky, kx = psf.shape
            issued = 32 * ky * kz
            out[precision]["issued_macs_per_voxel_conv"] = issued
            out[precision]["useful_macs_per_voxel_conv"] = kx * ky * kz
            out[precision]["useful_mac_fraction"] = kx * ky * kz / issued
            out[precision]["tflops_issued"] = out[precision]["tflops_useful"] * issued / (kx * ky * kz)
        rl.close()
    d = results["bf16"] - results["f32"]
    out["bf16_vs_f32"] = {"rel_l2": float(d.norm() / results["f32"].norm()), "max_abs": float(d.abs().max()),
                          "speedup": out["f32"]["ms_per_run"] / out["bf16"]["ms_per_run"]}
    if cpu:
        import oracle
        from oracle import build as oracle_build

        oracle_build.build_oracle()
        threads = oracle.default_threads()
        t0 = time.perf_counter()
        ref = oracle.rl(observed, psf, ITERATIONS, EPSILON, init=oracle.abi.RL_INIT_MEAN, threads=threads)
        dt = time.perf_counter() - t0
        ref64 = torch.from_numpy(ref.astype(np.float64)).to(dev)
        for precision in ("bf16", "f32"):
            e = results[precision] - ref64
            out[precision]["vs_fp64_oracle"] = {"rel_l2": float(e.norm() / ref64.norm()),
                                                "max_abs": float(e.abs().max()),
                                                "max_abs_rel_to_max": float(e.abs().max() / ref64.abs().max())}
        out["cpu_baseline"] = {"value": 2 * ITERATIONS * observed.size / dt / 1e9, "unit": UNIT, "cores": threads,
                               "kind": "port", "sample": f"oracle RL (FP64-accumulated convolutions), all "
                                                         f"{ITERATIONS} iterations on the full volume ({dt:.1f} s)"}
    out["config"] = "256x256x64, PSF 9x9x9 sigma 2.5, 50 iterations, flat start"
    return out


def measure_batch_leg(dev, stream, reps=3, iterations=30, cpu=True):
    """Batched uneven 2-D RL: 256 images, sides log-uniform in [64, 1024], own Gaussian PSF
    each (odd size 3-31, sigma 0.5-5), Poisson noise, 30 iterations, one CUDA-graph replay
    per run holding ONE persistent launch over the work queue of every pass of every image,
    autotuned CTAs per SM and queue order."""
    import numpy as np
    import torch

    import iane_gb300
    from iane_gb300 import synth

    truths, psfs = synth.batch_workload(count=256, seed=0)
    gen = torch.Generator(device=dev)
    gen.manual_seed(0)
    g_psfs = [torch.from_numpy(p).to(dev) for p in psfs]
    obs = []
    for t, p in zip(truths, g_psfs):
        src = torch.from_numpy(t).to(dev)
        blurred = torch.empty_like(src)
        iane_gb300.convolve(src, p, blurred, "zero", stream=stream)
        obs.append(torch.poisson(blurred.clamp_min(0), generator=gen))
    outs = [torch.empty_like(o) for o in obs]
    t0 = time.perf_counter()
    batch = iane_gb300.RichardsonLucyBatch(g_psfs, [o.shape for o in obs], autotune=True)
    prepare_s = time.perf_counter() - t0
    scratch = torch.empty(batch.scratch_bytes, dtype=torch.uint8, device=dev)
    batch.run(obs, outs, iterations, EPSILON, init=1, scratch=scratch, stream=stream)  # captures the graph
    torch.cuda.synchronize(dev)
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(reps):
        batch.run(obs, outs, iterations, EPSILON, init=1, scratch=scratch, stream=stream)
    b.record(stream)
    torch.cuda.synchronize(dev)
    ms = a.elapsed_time(b) / reps
    pixels = sum(o.numel() for o in obs)
    macs = sum(o.numel() * p.size for o, p in zip(obs, psfs)) * 2 * iterations
    bps, order, grouping = batch.launch_config()
    widths = batch.tile_widths()
    batch.close()
    assert all(bool(torch.isfinite(o).all()) for o in outs)
    peaks, _ = measured_peaks()
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    fp32 = fp32_peak_tflops(dev)["peak"]
    alg_bytes = 24.0 * pixels * iterations   # per iteration: pass A 12 B/px, pass B 12 B/px
    res = {"images": len(obs), "pixels": pixels, "iterations": iterations, "ms_per_run": ms,
           "gvoxel_s": 2 * iterations * pixels / (ms / 1e3) / 1e9, "tflops_useful": 2 * macs / (ms / 1e3) / 1e12,
           "gbs_algorithmic": alg_bytes / (ms / 1e3) / 1e9,
           "launch": {"persistent_launches_per_run": 1, "ctas_per_sm": bps,
                      "queue_order": ["largest images first", "by PSF width"][order], "grouping": grouping,
                      "images_by_item_shape": {f"{w}x64": widths.count(w) for w in sorted(set(widths))}},
           "prepare_s": prepare_s}
    res["frac_of_fp32_peak"] = res["tflops_useful"] / fp32
    res["frac_of_hbm_peak"] = res["gbs_algorithmic"] / hbm
    if cpu:
        # the reference's RL loop (oracle port, all host threads) on the first 8 images
        import oracle
        from oracle import build as oracle_build

        oracle_build.build_oracle()
        threads = oracle.default_threads()
        sample = list(range(8))
        o_np = [obs[i].cpu().numpy() for i in sample]
        t0 = time.perf_counter()
        for i, o in zip(sample, o_np):
            oracle.rl(o, psfs[i], iterations, EPSILON, init=oracle.abi.RL_INIT_MEAN, threads=threads)
        dt = time.perf_counter() - t0
        px = sum(o.size for o in o_np)
        res["cpu_baseline"] = {"value": 2 * iterations * px / dt / 1e9, "unit": "GVoxel/s", "cores": threads,
                               "kind": "port", "sample": f"oracle RL, {iterations} iterations, first 8 images "
                                                         f"({px} pixels, {dt:.1f} s)"}
    return res


def measure_fft_leg(dev, stream, reps=5):
    """Spectral against direct convolution for large kernels: the 256x256x64 volume with
    normalised 31x31x15 (sigma 4, 4, 2) and 31x31x31 (sigma 4) Gaussians, zero border; device
    time per call (CUDA events), the largest difference relative to the direct result's
    maximum, and which path `auto` picked."""
    import torch

    import iane_gb300
    from iane_gb300 import synth

    gen = torch.Generator(device=dev)
    gen.manual_seed(3)
    vol = torch.rand((64, 256, 256), generator=gen, device=dev, dtype=torch.float32) * 1000
    out = {}
    for name, ext, sig in (("psf_31x31x15", (31, 31, 15), (4.0, 4.0, 2.0)), ("psf_31x31x31", (31, 31, 31), (4.0, 4.0, 4.0))):
        psf = torch.from_numpy(synth.gaussian_psf(ext, sig)).to(dev)
        leg, res = {}, {}
        for method in ("direct", "fft", "auto"):
            dst = torch.empty_like(vol)
            run = lambda: iane_gb300.convolve(vol, psf, dst, "zero", method=method, stream=stream)
            for _ in range(2):
                run()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(reps):
                run()
            b.record(stream)
            torch.cuda.synchronize(dev)
            ms = a.elapsed_time(b) / reps
            res[method] = dst.double()
            leg[method] = {"ms": ms, "gvoxel_s": vol.numel() / (ms / 1e3) / 1e9}
        leg["fft_vs_direct_max_rel"] = float((res["fft"] - res["direct"]).abs().max() / res["direct"].abs().max())
        leg["speedup"] = leg["direct"]["ms"] / leg["fft"]["ms"]
        leg["auto_picked"] = "fft" if torch.equal(res["auto"], res["fft"]) else "direct"
        out[name] = leg
    out["config"] = "256x256x64 f32, normalised Gaussian PSFs, zero border"
    return out


def measure_reference_benchmark_leg(dev, stream, cpu=True, reps=20):
    """The reference's own convolution benchmark (benchmarks/convolution.cu:84-118): a
    2560x1920 u8 image ((i * 19) ^ (i / width)), a 9x9 f32 kernel (((i * 3) % 7 - 2) / 64),
    clamp border, from a linear device image and from a texture. Device time per call (CUDA
    events), and whether the output is byte-identical to the reference's serial CPU result
    (SHA-256 kept with the golden vectors). The CPU baseline is the oracle port on all host
    threads and on one (the reference times serial, 4 and 8 workers)."""
    import hashlib

    import numpy as np
    import torch

    import iane_gb300

    width, height = 2560, 1920
    i = np.arange(width * height, dtype=np.int64)
    image = (((i * 19) ^ (i // width)) & 0xFF).astype(np.uint8).reshape(height, width)
    k = np.arange(81, dtype=np.int64)
    kernel = (((k * 3) % 7 - 2) / 64.0).astype(np.float32).reshape(9, 9)
    golden = np.load(Path(__file__).resolve().parent / "tests" / "golden" / "golden.npz")
    want = str(golden["bench_u8_2560x1920__sha256"])
    src = torch.from_numpy(image).to(dev)
    kd = torch.from_numpy(kernel).to(dev)
    dst = torch.empty_like(src)
    tex = iane_gb300.Texture(image.shape, "uint8").upload(src, stream=stream)
    out = {}
    for name, source, exact in (("linear", src, False), ("texture", tex.view(), False), ("linear_exact_fp64", src, True)):
        run = lambda: iane_gb300.convolve(source, kd, dst, "clamp", exact=exact, stream=stream)
        for _ in range(3):
            run()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            run()
        b.record(stream)
        torch.cuda.synchronize(dev)
        ms = a.elapsed_time(b) / reps
        digest = hashlib.sha256(dst.cpu().numpy().tobytes()).hexdigest()
        out[name] = {"ms": ms, "gpixel_s": image.size / (ms / 1e3) / 1e9,
                     "tflops": 2 * 81 * image.size / (ms / 1e3) / 1e12, "bit_exact_vs_reference": digest == want}
    tex.close()
    if cpu:
        import oracle
        from oracle import build as oracle_build

        oracle_build.build_oracle()
        ref_np = np.zeros_like(image)
        for threads in (oracle.default_threads(), 1):
            t0 = time.perf_counter()
            n = 0
            while n == 0 or time.perf_counter() - t0 < 1.0:
                oracle.convolve(image, kernel, ref_np, "clamp", threads=threads)
                n += 1
            cms = (time.perf_counter() - t0) / n * 1e3
            key = "cpu_baseline_all_threads" if threads > 1 else "cpu_baseline_1_thread"
            out[key] = {"ms": cms, "cores": threads, "kind": "port", "sample": f"{n} full image(s)"}
        out["gpu_speedup_vs_all_threads"] = out["cpu_baseline_all_threads"]["ms"] / out["linear"]["ms"]
    out["config"] = "2560x1920 u8, 9x9 f32 kernel (k/64), clamp"
    return out


def measure_wiener_leg(dev, stream, cpu=True, reps=20):
    """Wiener deconvolution (the reference's examples/wiener/main.cu:44-83) of a 2560x1920 u8
    image (the reference benchmark's pattern) with a 9x9 Gaussian PSF (sigma 2), noise 0.002,
    u8 output: device time per prepared run (CUDA events; R2C, filter, C2R and the u8
    encode), and the numpy restatement (float64 DFTs, one host thread) as the CPU baseline."""
    import numpy as np
    import torch

    import iane_gb300
    from iane_gb300 import synth

    width, height = 2560, 1920
    i = np.arange(width * height, dtype=np.int64)
    image = (((i * 19) ^ (i // width)) & 0xFF).astype(np.uint8).reshape(height, width)
    psf_np = synth.gaussian_psf((9, 9), (2.0, 2.0))
    obs = torch.from_numpy(image).to(dev)
    out = torch.empty_like(obs)
    w = iane_gb300.Wiener(torch.from_numpy(psf_np).to(dev), image.shape, 0.002, stream=stream)
    scratch = torch.empty(w.scratch_bytes, dtype=torch.uint8, device=dev)
    for _ in range(3):
        w.run(obs, out, scratch=scratch, stream=stream)
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(reps):
        w.run(obs, out, scratch=scratch, stream=stream)
    b.record(stream)
    torch.cuda.synchronize(dev)
    ms = a.elapsed_time(b) / reps
    leg = {"ms": ms, "gpixel_s": image.size / (ms / 1e3) / 1e9,
           "config": "2560x1920 u8, 9x9 Gaussian PSF sigma 2, noise 0.002, u8 output"}
    if cpu:
        import oracle

        t0 = time.perf_counter()
        ref = oracle.wiener(image, psf_np, 0.002)
        cms = (time.perf_counter() - t0) * 1e3
        diff = np.abs(out.cpu().numpy().astype(np.int32) - ref.astype(np.int32))
        leg["cpu_baseline"] = {"ms": cms, "cores": 1, "kind": "port", "sample": "1 full image (numpy float64 FFT)"}
        leg["max_level_difference_vs_oracle"] = int(diff.max())
        leg["gpu_speedup_vs_cpu"] = cms / ms
    w.close()
    return leg


def measure_morphology_leg(dev, stream, reps=20):
    """Flat morphology (include/iane/algorithms/morphology/morphology.hpp): erosion of the
    2560x1920 u8 benchmark image with a 5x5 box, and erosion and opening of a 512^3 f32 volume
    with a 5x5x5 box, zero border. Device time per call (CUDA events) and the algorithmic
    bandwidth (an erosion reads and writes the image once -- the 3-D box is one fused kernel --
    and an opening twice) against the measured HBM peak."""
    import numpy as np
    import torch

    import iane_gb300

    peak = measured_peaks()[0].get("hbm_gbs") or 6800.0
    out = {}

    def timed(fn):
        for _ in range(3):
            fn()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        torch.cuda.synchronize(dev)
        return a.elapsed_time(b) / reps

    width, height = 2560, 1920
    i = np.arange(width * height, dtype=np.int64)
    img = torch.from_numpy((((i * 19) ^ (i // width)) & 0xFF).astype(np.uint8).reshape(height, width)).to(dev)
    dst = torch.empty_like(img)
    ms = timed(lambda: iane_gb300.morphology(img, dst, (2, 2), "erode", "zero", stream=stream))
    out["erode_u8_2560x1920_box5"] = {"ms": ms, "gbs": 2 * img.numel() / (ms / 1e3) / 1e9}
    gen = torch.Generator(device=dev)
    gen.manual_seed(5)
    vol = torch.rand((512, 512, 512), generator=gen, device=dev)
    vdst = torch.empty_like(vol)
    scratch = torch.empty(2 * vol.numel() * 4 + 1024, dtype=torch.uint8, device=dev)
    ms = timed(lambda: iane_gb300.morphology(vol, vdst, (2, 2, 2), "erode", "zero", stream=stream))
    gbs = 2 * vol.numel() * 4 / (ms / 1e3) / 1e9
    out["erode_f32_512cubed_box5"] = {"ms": ms, "gbs": gbs, "hbm_frac": gbs / peak}
    ms = timed(lambda: iane_gb300.morphology(vol, vdst, (2, 2, 2), "opening", "zero", scratch=scratch, stream=stream))
    gbs = 4 * vol.numel() * 4 / (ms / 1e3) / 1e9
    out["opening_f32_512cubed_box5"] = {"ms": ms, "gbs": gbs, "hbm_frac": gbs / peak}
    return out


def measure_learned_leg(dev):
    """Learned warm start: the shipped network's start + BF16 tensor-core RL against plain FP32
    RL from the flat start on the 256x256x64 ellipsoid volume (200 ellipsoids), isotropic
    Gaussian PSF sigma 2 (11^3), Poisson peak 1000; reference = 200 FP32 iterations. Stopping
    rules, iteration counts, wall times (CUDA events) and errors as iane_gb300.learned.evaluate
    reports them."""
    from iane_gb300.learned import evaluate, load_default

    return evaluate(load_default(dev), device=dev)


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return

    import numpy as np
    import torch

    import iane_gb300
    from iane_gb300 import synth

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)

    observed, psf, _ = synth.rl_volume_workload(seed=0)
    obs_host = torch.from_numpy(observed).pin_memory()
    est_host = torch.empty(observed.shape, dtype=torch.float32).pin_memory()
    obs = obs_host.to(dev)
    rl = iane_gb300.RichardsonLucy(torch.from_numpy(psf).to(dev), observed.shape)
    scratch = torch.empty(rl.scratch_bytes, dtype=torch.uint8, device=dev)
    host_scratch = torch.empty(rl.host_scratch_bytes(False), dtype=torch.uint8, device=dev)
    est = torch.empty(observed.shape, dtype=torch.float32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step():
        rl.run(obs, est, ITERATIONS, EPSILON, init=rl.INIT_MEAN, scratch=scratch, stream=stream)

    fp32_peak_tflops(dev)  # the FP32 roofline denominator, measured before the timed region
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    if dist:
        dist.barrier()
    torch.cuda.synchronize(dev)

    sampler = ClockSampler(local)
    sampler.start()
    events = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        step()
        b.record(stream)
        events.append((a, b))
    torch.cuda.synchronize(dev)
    clocks = sampler.stop()
    if dist:
        dist.barrier()
    torch.cuda.synchronize(dev)
    iane_gb300.device_status()
    step_ms = [a.elapsed_time(b) for a, b in events]
    total_ms = sum(step_ms)
    total_ms = max_over_ranks(total_ms, dist, dev)
    conv_voxels_per_step = 2 * ITERATIONS * VOXELS
    value = job_throughput(world, conv_voxels_per_step, args.steps, total_ms / 1e3)
    ms_per_step = total_ms / args.steps

    # end to end through the C-ABI host entry point
    e2e_steps = max(3, min(args.steps, 10))
    rl.run_host(obs_host, est_host, ITERATIONS, EPSILON, init=rl.INIT_MEAN, scratch=host_scratch)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        rl.run_host(obs_host, est_host, ITERATIONS, EPSILON, init=rl.INIT_MEAN, scratch=host_scratch)
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist, dev)
    e2e_value = job_throughput(world, conv_voxels_per_step, e2e_steps, e2e_s)

    with_cpu = rank == 0 and world == 1 and not args.no_cpu_baseline
    hbm_legs = measure_hbm_legs(dev, stream, cpu=with_cpu)
    bf16_leg = measure_bf16_leg(dev, stream, cpu=with_cpu)
    batch_leg = measure_batch_leg(dev, stream, cpu=with_cpu)
    learned_leg = measure_learned_leg(dev)
    fft_leg = measure_fft_leg(dev, stream)
    reference_benchmark_leg = measure_reference_benchmark_leg(dev, stream, cpu=with_cpu)
    wiener_leg = measure_wiener_leg(dev, stream, cpu=with_cpu)
    morphology_leg = measure_morphology_leg(dev, stream)

    # result sanity: the run converged to something finite and positive
    est_np = est.cpu().numpy()
    assert np.isfinite(est_np).all() and est_np.min() >= 0.0

    # roofline of the fused pass (the 100 passes of a step run in one persistent launch after
    # the two small start kernels, so step time / 100 bounds the average pass time from above)
    peaks, peak_kind = measured_peaks()
    fp32 = fp32_peak_tflops(dev)
    fp32_peak = fp32["peak"]
    pass_ms = ms_per_step / (2 * ITERATIONS)
    flops_per_pass = 2.0 * TAPS * VOXELS
    achieved = flops_per_pass / (pass_ms / 1e3) / 1e12
    alg_bytes_pass = 12.0 * VOXELS
    hbm_achieved = alg_bytes_pass / (pass_ms / 1e3) / 1e9
    traffic = recorded_traffic()
    roofline = {
        "bound": "fp32",
        "achieved": achieved,
        "peak": fp32_peak,
        "unit": "TFLOP/s",
        "frac": achieved / fp32_peak,
        "traffic": traffic,
        "kernel": "rl_persist_kernel<15> (RL passes A/B, all 100 in one persistent launch)",
        "peak_source": (f"measured in this run: FP32 FMA probe (iane_gb_fp32_peak_probe), scalar FFMA "
                        f"{fp32['scalar_ffma']:.1f} and paired fma.rn.f32x2 {fp32['paired_ffma2']:.1f} TFLOP/s, "
                        f"the larger taken; nominal {fp32['sms']} SMs x 128 FMA/clk x 2 x max clock = "
                        f"{fp32['nominal']:.1f}"),
        "peak_nominal": fp32["nominal"],
        "hbm": {"achieved_gbs": hbm_achieved, "peak_gbs": float(peaks.get("hbm_gbs", 6800.0)),
                "frac": hbm_achieved / float(peaks.get("hbm_gbs", 6800.0)), "alg_bytes_per_pass": alg_bytes_pass,
                "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peak_kind})"},
    }

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import oracle
        from oracle import build as oracle_build

        oracle_build.build_oracle()
        threads = oracle.default_threads()
        v, dt = cpu_sample(observed, psf, threads, CPU_ITERATIONS)
        kind = reference_kind()
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": kind,
               "sample": f"{'the reference library' if kind == 'reference' else 'oracle port'} RL, "
                         f"{CPU_ITERATIONS} iterations + sensitivity on the full volume "
                         f"({1 + 2 * CPU_ITERATIONS} convolutions, {dt:.1f} s)"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded ellipsoid phantom, Poisson)",
            "config": config(), "rl_iterations_per_s": world * ITERATIONS * args.steps / (total_ms / 1e3),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(observed.nbytes),
                    "d2h_bytes_per_step": int(observed.nbytes), "steps": e2e_steps},
            "gpu_launches": 3 * args.steps,  # flat-start mean, start, the persistent run
            "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks,
            "step_ms": {"min": min(step_ms), "median": statistics.median(step_ms), "max": max(step_ms)},
            "hbm_legs": hbm_legs,
            "bf16_tensor_leg": bf16_leg,
            "batch_leg": batch_leg,
            "learned_warm_start_leg": learned_leg,
            "fft_leg": fft_leg,
            "reference_benchmark_leg": reference_benchmark_leg,
            "wiener_leg": wiener_leg,
            "morphology_leg": morphology_leg,
        }
        print(json.dumps(line), flush=True)
    rl.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
