#!/usr/bin/env python3
"""Benchmark of the dense g2 correlator (tensor-core Gram path) on GB300.

Workload: 514 x 1030 uint8 frames, 10,000 frames, 16 equal annular q-bins with
radii 20-400 px around (257, 515); synthetic AR(1) speckle (rho 0.99, mean 0.1
photons/pixel), generated on the device with a fixed seed.  One step = one
full correlation of the stack through the public API
(``MatMulCorrelator.correlate_device``: pack + bin sums, tensor-core Gram with
fused lag sums, denominator, g2), inputs resident in HBM.  ``e2e`` repeats it
with the frames in pinned host memory (``MatMulCorrelator.correlate``: H2D copy,
pipeline, g2 back to the host).  The stack (5.3 GB) is larger than L2, so no
flush is needed between steps.

``--impl reference`` times the CPU reference instead: the reference's own
MatMulCorrelator (numpy BLAS on all host cores; its float32 restatement when
the reference package is not installed) on all 10,000 frames of the same
stack, one full-size call.

Multi-GPU (torchrun): independent replicas, one stack per GPU ("weak" scaling).
"""
from __future__ import annotations

import argparse
import contextlib
import gc
import json
import math
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = {
    "workload": "dense_514x1030_u8_T10000_16bins",
    "frame_shape": [514, 1030], "nframes": 10000, "dtype": "uint8", "n_bins": 16,
    "qmask": "16 equal annuli r 20-400 px around (257, 515)", "rho": 0.99, "mean_photons": 0.1, "seed": 1,
    "l2": "inputs (5.3 GB) larger than L2; no flush",
}
CPU_SAMPLE_FRAMES = 2048
SPARSE_WORKLOAD = {
    "workload": "sparse_2162x2068_u8_T20000_32bins",
    "frame_shape": [2162, 2068], "nframes": 20000, "dtype": "uint8", "n_bins": 32,
    "qmask": "32 equal annuli r 20-1000 px around (1081, 1034)", "rho": 0.99, "mean_photons": 0.005, "seed": 4,
    "layout": "per-frame CSR (uint8 values, int32 column indices and row pointers, int64 frame offsets)",
    "l2": "inputs (~2.4 GB CSR, ~2.3 GB event lists) larger than L2; no flush",
}
CPU_SAMPLE_PIXEL_STRIDE = 16



@contextlib.contextmanager
def no_gc():
    """A timed region runs with Python's cyclic garbage collector paused (as
    timeit does): single calls of the end-to-end loops run after the dense
    line otherwise showed stalls of 7-33 ms (collections of the bench
    process's heap, not work of the call)."""
    gc.collect()
    was = gc.isenabled()
    gc.disable()
    try:
        yield
    finally:
        if was:
            gc.enable()

def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--no-plain", action="store_true", help="skip the plain-kernel comparator")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-extra", action="store_true",
                   help="dense line only: skip the u16 / sparse / event sub-lines (configurations 3 and 4)")
    p.add_argument("--frames", type=int, default=None, help="override T (testing only)")
    p.add_argument("--shape", default=None, help="H,W of the sparse/event frames (profiling only)")
    p.add_argument("--tile", default=None, choices=["pair", "wide", "single"],
                   help="tensor-core block of the dense Gram (default: the engine's)")
    p.add_argument("--workload", default="dense", choices=["dense", "u16", "sparse", "event", "serving", "compress"],
                   help="dense: 514x1030x10k u8 Gram path (default); sparse / event: 2162x2068x20k CSR or "
                        "per-pixel event lists through the pair-sum path")
    return p.parse_args()


def dist_info():
    from dynamix_gb300.replicas import rank_info
    return rank_info()


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def profile_traffic(name, key="traffic_bytes_per_launch"):
    """Per-launch DRAM bytes of a kernel from a committed ncu summary (or None)."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(path):
            parts = line.split("=")
            if len(parts) >= 2 and parts[0].strip() == key:
                return float(parts[1].split()[0])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons every 100 ms during the timed region,
    for this process's GPU only (matched by UUID); when no sample matches the
    UUID the clocks are reported as unavailable rather than taken from the
    other GPUs of the machine."""

    FIELDS = ("uuid,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")
    REASONS = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")

    def __init__(self, uuid):
        self.uuid = (uuid or "").lower()
        self.proc = None
        self.out = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            cmd = ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits", "-lms", "100"]
            self.proc = subprocess.Popen(cmd, stdout=self.out, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.flush()
        self.out.seek(0)
        rows = [[x.strip() for x in line.split(",")] for line in self.out.read().splitlines()]
        os.unlink(self.out.name)
        rows = [r for r in rows if len(r) >= 8]
        rows = [r for r in rows if self.uuid and self.uuid in r[0].lower()]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None,
                    "reasons": ["unavailable: no nvidia-smi sample matched this GPU's UUID"]}
        sm, smax, power, reasons = [], [], [], set()
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
                power.append(float(r[3]))
            except ValueError:
                continue
            for n, v in zip(self.REASONS, r[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None, "samples": len(sm), "reasons": sorted(reasons)}


def tc_rate(dev, kind, iters=40000, reps=5):
    """Dense MMA rate (TFLOP/s, 2 ops per MAC) of this GPU for the Gram's
    operand kind, from the library's own tcgen05 probe (M128 N256, operands
    resident in shared memory, one CTA per SM; best of ``reps`` launches timed
    with CUDA events on the launching stream)."""
    import ctypes
    import torch
    from dynamix_gb300 import _lib
    lib = _lib.load()
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    h = ctypes.c_void_p(stream.cuda_stream)
    _lib.check(lib.g2_tc_rate_probe(kind, 2000, 0, ctypes.c_void_p(err.data_ptr()), h), "g2_tc_rate_probe")
    best = float("inf")
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _lib.check(lib.g2_tc_rate_probe(kind, iters, 0, ctypes.c_void_p(err.data_ptr()), h), "g2_tc_rate_probe")
        e1.record(stream)
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    if int(err.item()):
        raise RuntimeError("tensor-core probe: " + _lib.device_error_message(int(err.item())))
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    k = 32 if kind == _lib.KIND_E4M3 else 16
    macs = sms * iters * 4 * 128 * 256 * k
    return 2.0 * macs / (best / 1e3) / 1e12, {"launch_ms": best, "ctas": sms, "iters": iters,
                                              "mma": "tcgen05 M128 N256 K%d x4 per iteration" % k}


def make_workload(dev, T):
    from dynamix_gb300.speckle import annular_qmask, speckle_torch
    H, W = WORKLOAD["frame_shape"]
    qmask = annular_qmask((H, W), WORKLOAD["n_bins"], 20.0, 400.0, center=(257, 515))
    frames = speckle_torch(T, (H, W), WORKLOAD["rho"], WORKLOAD["mean_photons"], seed=WORKLOAD["seed"],
                           device=dev)
    return frames, qmask


def reference_matmul():
    """(correlate(frames, qmask) callable, kind, label) of the CPU MatMul
    correlator: the reference's own ``MatMulCorrelator`` (dense.py:118-142,
    imported from the installed reference package behind inert OpenCL stubs)
    when the package is present, else its float32 restatement."""
    try:
        from oracle.ref_import import import_module
        dense = import_module("dynamix.correlator.dense")

        def run(frames, qmask):
            return dense.MatMulCorrelator(frames.shape[1:], frames.shape[0], qmask=qmask).correlate(frames)
        return run, "reference", "the reference's own MatMulCorrelator.correlate (numpy float32 BLAS)"
    except ImportError:
        from oracle.g2_oracle import matmul_correlator_port

        def run(frames, qmask):
            return matmul_correlator_port(frames, qmask)
        return run, "port", "float32 restatement of MatMulCorrelator (numpy BLAS)"


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count()


def cpu_port_time(frames_host, qmask, repeats=1):
    """Seconds per call of the CPU MatMul correlator (all host threads), with its kind and label."""
    run, kind, label = reference_matmul()
    ts = []
    for _ in range(repeats):
        t0 = time.perf_counter()
        with __import__("numpy").errstate(all="ignore"):
            run(frames_host, qmask)
        ts.append(time.perf_counter() - t0)
    return ts, kind, label


def cpu_scale(T_full, t_sample, T_sample):
    # cost of the MatMul correlator is O(T^2) (Gram and per-lag diagonal loop)
    return T_full / (t_sample * (T_full / T_sample) ** 2)


REF_WARMUP_FRAMES = 256


def run_reference(args):
    """The CPU reference on the whole workload: one call of the MatMul
    correlator on all 10,000 frames (all host cores), after a warm-up call on
    the first frames.  One full-size call takes minutes, so the run measures
    exactly one step whatever --steps asks for, and says so."""
    import numpy as np
    import torch
    rank, world, local = dist_info()
    if rank != 0:
        return 0
    T_full = args.frames
    dev = torch.device("cuda", local) if torch.cuda.is_available() else torch.device("cpu")
    frames, qmask = make_workload(dev, T_full)
    host = frames.cpu().numpy()
    del frames
    Tw = min(REF_WARMUP_FRAMES, T_full)
    cpu_port_time(np.ascontiguousarray(host[:Tw]), qmask)
    ts, kind, label = cpu_port_time(host, qmask, repeats=1)
    t = ts[0]
    v = T_full / t
    ncores = host_cores()
    line = {
        "metric": "g2_frames_per_s", "value": v, "unit": "frames/s", "impl": "reference", "n_gpus": args.gpus,
        "steps": 1, "warmup": 1, "steps_requested": args.steps, "warmup_requested": args.warmup,
        "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dict(WORKLOAD, nframes=T_full, parallelism="replicas" if world > 1 else "single"),
        "note": "one full-size call (all %d frames, all 16 bins) timed; a warm-up call on the first %d frames "
                "before it; more steps would take minutes each" % (T_full, Tw),
        "cpu_baseline": {"value": v, "unit": "frames/s", "cores": ncores, "kind": kind,
                         "sample": "the whole workload: %s on all %d frames, %d host threads, %.1f s"
                                   % (label, T_full, ncores, t)},
        "e2e": {"value": v, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_ours(args):
    import numpy as np
    import torch

    from dynamix_gb300 import build as b
    from dynamix_gb300.correlator import MatMulCorrelator
    from dynamix_gb300.plan import gram_macs

    rank, world, local = dist_info()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    b.build(force=False)

    T = args.frames
    frames, qmask = make_workload(dev, T)
    H, W = WORKLOAD["frame_shape"]
    corr = MatMulCorrelator((H, W), T, qmask=qmask, extra_options={"tile": args.tile} if args.tile else {})
    eng = corr.engine
    npix = np.bincount(qmask.ravel(), minlength=17)[1:]
    macs = gram_macs(T, npix)

    def barrier():
        torch.cuda.synchronize(dev)
        if dist is not None:
            dist.barrier()

    def max_over_ranks(x):
        from dynamix_gb300.replicas import max_over_ranks as mx
        return mx(x, dist, dev)

    # ---- device-resident steps
    for _ in range(max(args.warmup, 3)):
        corr.correlate_device(frames)
    eng.check_error()
    stream = torch.cuda.current_stream(dev)
    uuid = None
    try:
        uuid = "GPU-" + str(torch.cuda.get_device_properties(dev).uuid)
    except Exception:
        pass
    sampler = ClockSampler(uuid)
    barrier()
    sampler.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with no_gc():
        e0.record(stream)
        for _ in range(args.steps):
            corr.correlate_device(frames)
        e1.record(stream)
        barrier()
    clocks = sampler.stop()
    eng.check_error()
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps)
    from dynamix_gb300.replicas import whole_job_rate
    value = whole_job_rate(T, ms, world)
    info = dict(eng.last)
    chunks = int(info.get("pipeline_chunks", 1))
    # a pack per frame chunk, a Gram per chunk (the first chunks' Grams in one
    # launch), denominator, finalize
    merged = max(1, min(int(eng.PIPE_MERGE_FIRST), chunks)) - 1
    launches_per_step = 2 * chunks - merged + 2 if "pipeline_chunks" in info else 4

    # stage attribution: the same step run as one pack and one Gram launch,
    # with CUDA events on the launching stream around each stage
    eng.profile = True
    eng.pipeline = False
    n_attr = max(3, min(args.steps, 10))
    tile0 = eng.tile
    by_tile = {}
    for tile in [tile0] + [t for t in ("pair", "wide", "single") if t != tile0]:
        eng.tile = tile
        g_ms, p_ms = [], []
        corr.correlate_device(frames)
        eng.take_events()
        for _ in range(n_attr):
            corr.correlate_device(frames)
            st = eng.stage_times(eng.take_events())
            g_ms.append(st.get("gram_tc", float("nan")))
            p_ms.append(st.get("pack", float("nan")))
        eng.check_error()
        by_tile[tile] = (g_ms, p_ms)
    eng.tile = tile0
    gram_ms, pack_ms = by_tile[tile0]
    # one pipelined step with events at every pack and Gram launch of it
    eng.pipeline = True
    corr.correlate_device(frames)
    eng.take_events()
    timeline = eng.take_timeline()
    eng.profile = False

    peaks, peak_kind = measured_peaks()
    gram_avg = sum(gram_ms) / len(gram_ms)
    achieved = 2.0 * macs / (gram_avg / 1e3) / 1e12
    # Denominator of the Gram roofline: the dense rate of the MMA kind the Gram
    # ran on, measured in this run by the library's own tcgen05 probe (the
    # kernel runs at full clock, below the power cap, like the probe).
    from dynamix_gb300 import _lib as L
    kind = L.KIND_E4M3 if info.get("mode") == "e4m3" else L.KIND_FP16
    peak, probe = tc_rate(dev, kind)
    peak_f16, _ = tc_rate(dev, L.KIND_FP16) if kind == L.KIND_E4M3 else (peak, None)
    peak_src = ("tcgen05 kind::%s rate measured in this run (g2_tc_rate_probe: %d CTAs x %d iterations of "
                "4 x M128 N256 MMAs on shared-memory operands, best of 5, %.3f ms)"
                % ("f8f6f4 e4m3" if kind == L.KIND_E4M3 else "f16", probe["ctas"], probe["iters"],
                   probe["launch_ms"]))
    pack_bytes = T * H * W + T * info["packed_cols"] * (1 if info.get("mode") == "e4m3" else 2)
    pack_avg = sum(pack_ms) / len(pack_ms)
    # DRAM bytes of one Gram launch from the committed ncu summary of the tile measured there
    traffic = profile_traffic("gram_pair_dense_514x1030_%s.md" % info.get("mode")) if tile0 == "pair" else None

    line = {
        "metric": "g2_frames_per_s", "value": value, "unit": "frames/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": dict(WORKLOAD, nframes=T, parallelism="replicas" if world > 1 else "single"),
        "mma_kind": {"e4m3": "tcgen05 kind::f8f6f4 (e4m3 counts <= 16, fp32 accumulate, exact below 2^24)",
                     "fp16": "tcgen05 kind::f16 (fp16 counts <= 2048, fp32 accumulate, exact below 2^24)",
                     "bytes": "tcgen05 kind::f16 on hi/lo byte planes (4 Grams)"}[info["mode"]],
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "kernel": {"pair": "g2_gram_tc_pair", "wide": "g2_gram_tc_wide"}.get(tile0, "g2_gram_tc"),
                     "peak_source": peak_src,
                     "algorithmic_ops_per_launch": 2 * macs, "launch_ms": gram_avg,
                     "other_peaks": {"tcgen05_f16_probe": peak_f16, "bf16_cublas_" + peak_kind: peaks.get(
                         "bf16_tflops")}},
        "gram_ms_by_tile": {t: sum(v[0]) / len(v[0]) for t, v in by_tile.items()},
        "pipeline_timeline_ms": {k: round(v, 4) for k, v in timeline.items()},
        "stages_ms": {"pack": pack_avg, "gram_tc": gram_avg, "tile": tile0,
                      "note": "stage times from %d steps run unpipelined (one pack, one Gram launch); the timed "
                              "steps overlap the pack of frame chunk c+1 with the Gram tiles chunk c completes "
                              "(%d chunks)" % (n_attr, chunks)},
        "dtype_detail": "integer counts (u8) packed as %s, N/S/D int64, g2 float64 -> float32" % info.get("mode"),
        "pack_roofline": {"bound": "hbm", "achieved": pack_bytes / (pack_avg / 1e3) / 1e9,
                          "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                          "frac": pack_bytes / (pack_avg / 1e3) / 1e9 / peaks.get("hbm_gbs")},
        "clocks": clocks, "gpu_launches": launches_per_step * args.steps, "plan": info,
    }

    # ---- end to end through the public API, frames in pinned host memory
    if not args.no_e2e:
        host = frames.cpu().pin_memory()
        for _ in range(max(3, args.warmup)):
            corr.correlate(host)
        barrier()
        with no_gc():
            t0 = time.perf_counter()
            e0.record(stream)
            per_call = []
            for _ in range(args.steps):
                t1 = time.perf_counter()
                corr.correlate(host)                   # returns host arrays: synchronous
                per_call.append((time.perf_counter() - t1) * 1e3)
            e1.record(stream)
            barrier()
            e2e_ms = max_over_ranks((time.perf_counter() - t0) * 1e3 / args.steps)
        # g2, the error word, S for the int64 range check (and the segment
        # energies when the step is not pipelined)
        d2h = eng.n_bins * T * 4 + 4 + eng.n_bins * T * 8
        if "pipeline_chunks" not in eng.last:
            d2h += info["packed_cols"] // 64 * 4
        # the bytes that crossed the host link: the frames cropped to the
        # q-mask's column window (u8 stacks with a narrower binned region)
        h2d = int(eng.last.get("h2d_bytes") or host.numel() * host.element_size())
        line["e2e"] = {"value": world * T / (e2e_ms / 1e3), "unit": "frames/s",
                       "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_ms,
                       "ms_per_call_min_median_max": [min(per_call), sorted(per_call)[len(per_call) // 2],
                                                      max(per_call)],
                       "input": "the whole (T, H, W) u8 stack in pinned host memory, correlate(host_tensor); "
                                "copied in cropped to the q-mask's columns %s" % (eng.last.get("crop"),)}
        del host

    # ---- same-GPU plain (CUDA-core) comparators: the u8 __dp4a kernel (four
    # byte products per instruction) and the 32-bit IMAD kernel on fp16-packed
    # counts; the speed-up is stated against the faster of the two
    if not args.no_plain:
        plain = {}
        for method in ("dp4a", "plain"):
            pc = MatMulCorrelator((H, W), T, qmask=qmask, extra_options={"method": method})
            pc.correlate_device(frames)
            barrier()
            e0.record(stream)
            nplain = 2
            for _ in range(nplain):
                pc.correlate_device(frames)
            e1.record(stream)
            barrier()
            pc.engine.check_error()
            pms = max_over_ranks(e0.elapsed_time(e1) / nplain)
            same = bool(torch.equal(pc.engine.numer, eng.numer) and torch.equal(pc.engine.denom, eng.denom)
                        and torch.equal(pc.engine.sums, eng.sums))
            plain[method] = {"ms_per_step": pms, "value": world * T / (pms / 1e3), "unit": "frames/s",
                             "bit_identical_N_S_D": same,
                             "kernel": {"dp4a": "g2_plain_dp4a (u8 counts, __dp4a, 128x128 blocks)",
                                        "plain": "g2_plain_direct (fp16-packed counts, 32-bit IMAD)"}[method],
                             "int_tops": 2.0 * macs / (pms / 1e3) / 1e12}
            del pc
        best = min(plain, key=lambda m: plain[m]["ms_per_step"])
        line["plain"] = dict(plain[best], method=best, speedup_tc_vs_plain=plain[best]["ms_per_step"] / ms,
                             bit_identical_N_D=plain[best]["bit_identical_N_S_D"], comparators=plain)

    # ---- CPU baseline (rank 0, bounded sample)
    if not args.no_cpu and rank == 0:
        Ts = min(CPU_SAMPLE_FRAMES, T)
        host = frames[:Ts].cpu().numpy()
        ts, kind, label = cpu_port_time(host, qmask)
        ncores = host_cores()
        line["cpu_baseline"] = {
            "value": cpu_scale(T, ts[0], Ts), "unit": "frames/s", "cores": ncores, "kind": kind,
            "sample": "first %d of the %d frames, all 16 bins; %s, %d threads, took %.2f s; O(T^2) cost scaled "
                      "to %d frames (the reference arm times all %d frames)" % (Ts, T, label, ncores, ts[0], T,
                                                                               T)}
    # ---- configurations 3 (u16 precision stress) and 4 (CSR and event lists),
    # measured in the same run so that every configuration has a line
    if not args.no_extra:
        del frames
        torch.cuda.empty_cache()
        extra_steps = max(3, min(args.steps, 10))
        configs = {"u16": measure_u16(args, dev, U16_WORKLOAD["nframes"], extra_steps, args.warmup,
                                      cpu=not args.no_cpu and rank == 0, e2e=not args.no_e2e)}
        configs.update(measure_sparse(args, dev, SPARSE_WORKLOAD["nframes"], extra_steps, args.warmup, dist=dist,
                                      world=world, rank=rank, cpu=not args.no_cpu, e2e=not args.no_e2e))
        line["configs"] = configs
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


# ---------------------------------------------------------------- sparse / event
def sparse_shape(args):
    """Frame shape of the sparse/event workloads: 2162 x 2068, or a smaller
    one given with --shape (profiling at the same density)."""
    if getattr(args, "shape", None):
        h, w = (int(x) for x in args.shape.split(","))
        return h, w
    return tuple(SPARSE_WORKLOAD["frame_shape"])


def make_sparse_workload(dev, T, shape=None):
    from dynamix_gb300.speckle import annular_qmask, speckle_csr_torch
    H, W = shape or SPARSE_WORKLOAD["frame_shape"]
    if (H, W) == tuple(SPARSE_WORKLOAD["frame_shape"]):
        qmask = annular_qmask((H, W), SPARSE_WORKLOAD["n_bins"], 20.0, 1000.0, center=(1081, 1034))
    else:  # the same number of annuli over the smaller frame
        qmask = annular_qmask((H, W), SPARSE_WORKLOAD["n_bins"], 10.0, min(H, W) / 2 - 2, center=(H // 2, W // 2))
    csr = speckle_csr_torch(T, (H, W), SPARSE_WORKLOAD["rho"], SPARSE_WORKLOAD["mean_photons"],
                            seed=SPARSE_WORKLOAD["seed"], device=dev)
    return csr, qmask


def event_stats(ev_off, qmask):
    """(binned events, pair operations sum_p n_p (n_p + 1) / 2 over binned pixels)."""
    import torch
    n = (ev_off[1:].to(torch.int64) - ev_off[:-1].to(torch.int64))
    binned = torch.from_numpy((qmask.ravel() > 0)).to(n.device)
    nb = n[binned]
    return int(nb.sum().item()), int((nb * (nb + 1) // 2).sum().item())


def cpu_event_sample(times, data, offs, qmask, shape, T, stride):
    """Seconds of the C pair-sum restatement on every ``stride``-th binned
    pixel (all host threads), and the pair operations of that sample."""
    import numpy as np
    from oracle.g2_oracle import event_pairsum_c
    pix = np.flatnonzero(qmask.ravel() > 0)[::stride]
    n = (offs[pix + 1].astype(np.int64) - offs[pix].astype(np.int64))
    pairs = int((n * (n + 1) // 2).sum())
    t0 = time.perf_counter()
    event_pairsum_c(times, data, offs, qmask, shape, T, pixels=pix)
    return time.perf_counter() - t0, pairs


def event_rows_sample(ev_times, ev_data, ev_off, qmask, shape, row_stride):
    """The event lists of every ``row_stride``-th image row (rows below the
    frame width: the rows the reference's event launch reaches, event.py:183)
    as a smaller image on the host: (times, data, offsets, qmask, shape, pair
    operations).  A row's events are one contiguous slice of the lists."""
    import numpy as np
    import torch
    H, W = shape
    rows = np.arange(0, min(H, W), row_stride)
    off = ev_off.to(torch.int64).cpu().numpy()
    sl = [(int(off[y * W]), int(off[(y + 1) * W])) for y in rows]
    times = torch.cat([ev_times[a:b] for a, b in sl]).cpu().numpy()
    data = torch.cat([ev_data[a:b] for a, b in sl]).cpu().numpy()
    counts = np.concatenate([np.diff(off[y * W:(y + 1) * W + 1]) for y in rows])
    offs = np.zeros(counts.size + 1, dtype=np.uint32)
    offs[1:] = np.cumsum(counts)
    qm = np.ascontiguousarray(qmask[rows])
    binned = qm.ravel() > 0
    pairs = int((counts[binned] * (counts[binned] + 1) // 2).sum())
    return times, data, offs, qm, (rows.size, W), pairs


CPU_EVENT_ROW_STRIDE = 16


def cpu_event_baseline(ev_times, ev_data, ev_off, qmask, shape, T, all_pairs):
    """frames/s of the CPU pair sums on a sample of rows, scaled by pair
    operations to the whole stack: the reference's own evtcorrelator.cl
    (event_correlator + normalize_correlation compiled as C, all host threads;
    the OpenCL runtime is not available) when its sources are installed, else
    the C restatement."""
    from oracle.g2_oracle import event_pairsum_c, reference_event_correlate
    ncores = host_cores()
    t_h, d_h, o_h, qm, sub_shape, sp = event_rows_sample(ev_times, ev_data, ev_off, qmask, shape,
                                                         CPU_EVENT_ROW_STRIDE)
    kind, label = "reference", ("the reference's own evtcorrelator.cl (event_correlator + normalize_correlation, "
                                "compiled as C through the OpenCL shim, %d threads)" % ncores)
    t0 = time.perf_counter()
    try:
        ok = reference_event_correlate(t_h, d_h, o_h, qm, sub_shape, T, n_threads=ncores) is not None
    except ValueError:
        ok = False
    secs = time.perf_counter() - t0
    if not ok:
        kind, label = "port", "the C restatement of evtcorrelator.cl:3-47 (int64, %d threads)" % ncores
        t0 = time.perf_counter()
        event_pairsum_c(t_h, d_h, o_h, qm, sub_shape, T)
        secs = time.perf_counter() - t0
    full = secs * all_pairs / max(sp, 1)
    return {"value": T / full, "unit": "frames/s", "cores": ncores, "kind": kind,
            "sample": "event pair sums of every %dth image row (%d pair ops of %d) by %s in %.2f s, scaled by pair "
                      "ops to all %d frames; the CSR-to-event step is not included" % (
                          CPU_EVENT_ROW_STRIDE, sp, all_pairs, label, secs, T)}


def measure_sparse(args, dev, T, steps, warmup, which=("sparse", "event"), shape=None, dist=None, world=1,
                   rank=0, cpu=True, e2e=True):
    """Lines of the CSR workload (SparseCorrelator: CSR -> event lists on the
    device, pair sums, normalisation) and of the event-list workload
    (EventCorrelator on the same stack's lists), from one generated stack.
    Returns {kind: line} for the kinds in ``which``."""
    import torch
    from dynamix_gb300.correlator import EventCorrelator, SparseCorrelator

    H, W = shape or tuple(SPARSE_WORKLOAD["frame_shape"])
    (data, indices, indptr, offsets), qmask = make_sparse_workload(dev, T, (H, W))
    offsets = offsets.to(torch.int32)              # one index type (int32) for the whole CSR stack
    sc = SparseCorrelator((H, W), T, qmask=qmask)
    ev_times, ev_data, ev_off = (x.clone() for x in sc.engine.to_events(data, indices, indptr, offsets, 4,
                                                                          int(data.numel())))
    torch.cuda.synchronize(dev)
    n_elem = int(data.numel())
    n_binned_events, pairs = event_stats(ev_off, qmask)
    stream = torch.cuda.current_stream(dev)
    uuid = None
    try:
        uuid = "GPU-" + str(torch.cuda.get_device_properties(dev).uuid)
    except Exception:
        pass

    def barrier():
        torch.cuda.synchronize(dev)
        if dist is not None:
            dist.barrier()

    def max_over_ranks(x):
        from dynamix_gb300.replicas import max_over_ranks as mx
        return mx(x, dist, dev)

    npix = H * W
    P_b = int((qmask > 0).sum())
    n_bins = SPARSE_WORKLOAD["n_bins"]
    transpose_bytes = 14 * n_elem + 8 * (H + 1) * T + 16 * npix
    pair_bytes = 5 * n_binned_events + 12 * P_b + 16 * n_bins * T
    norm_bytes = 6 * 8 * n_bins * T
    peaks, peak_kind = measured_peaks()
    hbm = peaks.get("hbm_gbs")
    cpu_line = cpu_event_baseline(ev_times, ev_data, ev_off, qmask, (H, W), T, pairs) if cpu and rank == 0 else None
    out = {}
    for kind in which:
        if kind == "event":
            corr = EventCorrelator((H, W), T, 1, qmask=qmask)
            inputs = (ev_times, ev_data, ev_off)
            events_engine = corr.engine
        else:
            corr = sc
            inputs = (data, indices, indptr, offsets)
            events_engine = sc.engine.events
        for _ in range(max(warmup, 3)):
            corr.correlate_device(*inputs)
        corr.engine.check_error()
        sampler = ClockSampler(uuid)
        events_engine.profile = True
        barrier()
        sampler.start()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with no_gc():
            e0.record(stream)
            step_events = []
            for _ in range(steps):
                corr.correlate_device(*inputs)
                step_events.append(events_engine.take_events())
            e1.record(stream)
            barrier()
        clocks = sampler.stop()
        events_engine.profile = False
        corr.engine.check_error()
        ms = max_over_ranks(e0.elapsed_time(e1) / steps)
        stages = {}
        for ev in step_events:
            for k, v in events_engine.stage_times(ev).items():
                stages[k] = stages.get(k, 0.0) + v / steps
        info = dict(events_engine.last)
        step_bytes = pair_bytes + norm_bytes + (transpose_bytes if kind == "sparse" else 0)
        pair_ms = stages.get("pairsum", float("nan"))
        achieved = pair_bytes / (pair_ms / 1e3) / 1e9
        stage_report = {"pairsum": {"ms": pair_ms, "GB_per_s": achieved, "bytes": pair_bytes,
                                    "pair_ops_per_s": pairs / (pair_ms / 1e3)},
                        "normalize": {"ms": stages.get("normalize", float("nan")), "bytes": norm_bytes}}
        launches = 3   # pair sums, denominator, finalize
        if kind == "sparse":
            tms = stages.get("transpose", float("nan"))
            stage_report["transpose"] = {"ms": tms, "GB_per_s": transpose_bytes / (tms / 1e3) / 1e9,
                                         "bytes": transpose_bytes,
                                         "kernels": "row bounds, row counts, sub-block sums, two scans (3 each), "
                                                    "stage, gather"}
            launches += 11
        cfg = dict(SPARSE_WORKLOAD, nframes=T, frame_shape=[H, W], workload=SPARSE_WORKLOAD["workload"].replace(
            "sparse", "sparse_csr" if kind == "sparse" else "event_lists"),
            parallelism="replicas" if world > 1 else "single", n_elements=n_elem,
            binned_pixels=P_b, binned_events=n_binned_events, pair_ops=pairs)
        line = {
            "metric": "g2_frames_per_s", "value": world * T / (ms / 1e3), "unit": "frames/s", "n_gpus": world,
            "steps": steps, "warmup": max(warmup, 3), "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic", "config": cfg,
            "hbm_GB_per_s_step": step_bytes / (ms / 1e3) / 1e9,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                         "traffic": profile_traffic("event_pairsum_2162x2068_T20000.md",
                                                    "traffic_bytes_per_launch" if kind == "event"
                                                    else "traffic_bytes_per_launch_packed"),
                         "kernel": "g2_event_pairsum",
                         "peak_source": "%s hbm_gbs" % peak_kind, "algorithmic_bytes_per_launch": pair_bytes,
                         "launch_ms": pair_ms,
                         "note": "bound by shared-memory atomics (one per event pair), not by HBM"},
            "stages": stage_report, "clocks": clocks, "gpu_launches": launches * steps, "plan": info,
        }
        if e2e:
            host = [x.cpu().pin_memory() for x in inputs]
            for _ in range(max(3, warmup)):
                corr.correlate(*host)
            barrier()
            with no_gc():
                t0 = time.perf_counter()
                per_call = []
                for _ in range(steps):
                    t1 = time.perf_counter()
                    corr.correlate(*host)              # returns host arrays: synchronous
                    per_call.append((time.perf_counter() - t1) * 1e3)
                barrier()
            e2e_ms = max_over_ranks((time.perf_counter() - t0) * 1e3 / steps)
            line["e2e"] = {"value": world * T / (e2e_ms / 1e3), "unit": "frames/s",
                           "h2d_bytes_per_step": int(sum(x.numel() * x.element_size() for x in host)),
                           "d2h_bytes_per_step": int(n_bins * T * 4 + 4), "ms_per_step": e2e_ms,
                           "ms_per_call_min_median_max": [min(per_call), sorted(per_call)[len(per_call) // 2],
                                                          max(per_call)]}
            del host
        if cpu_line is not None:
            line["cpu_baseline"] = dict(cpu_line)
        out[kind] = line
        del corr
    return out


def run_sparse(args):
    import torch
    from dynamix_gb300 import build as b
    rank, world, local = dist_info()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    b.build(force=False)
    lines = measure_sparse(args, dev, args.frames, args.steps, args.warmup, which=(args.workload,),
                           shape=sparse_shape(args), dist=dist, world=world, rank=rank, cpu=not args.no_cpu,
                           e2e=not args.no_e2e)
    if rank == 0:
        print(json.dumps(lines[args.workload]))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_sparse_reference(args):
    """The CPU reference of the event pair sums (the reference's own
    evtcorrelator.cl compiled as C, else the C restatement), each step a
    sample of rows scaled by pair operations to the whole stack."""
    import torch
    rank, world, local = dist_info()
    if rank != 0:
        return 0
    T = args.frames
    H, W = sparse_shape(args)
    dev = torch.device("cuda", local)
    from dynamix_gb300 import build as b
    from dynamix_gb300.correlator import SparseCorrelator
    b.build(force=False)
    # the CSR stack is generated on the device and turned into event lists there
    (data, indices, indptr, offsets), qmask = make_sparse_workload(dev, T, (H, W))
    offsets = offsets.to(torch.int32)
    sc = SparseCorrelator((H, W), T, qmask=qmask)
    ev = [x.clone() for x in sc.engine.to_events(data, indices, indptr, offsets, 4, int(data.numel()))]
    del data, indices, indptr, offsets, sc
    _, pairs = event_stats(ev[2], qmask)
    for _ in range(args.warmup):
        cpu_event_baseline(*ev, qmask, (H, W), T, pairs)
    vals = [cpu_event_baseline(*ev, qmask, (H, W), T, pairs) for _ in range(args.steps)]
    v = sum(x["value"] for x in vals) / len(vals)
    line = {
        "metric": "g2_frames_per_s", "value": v, "unit": "frames/s", "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": T / v * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": dict(SPARSE_WORKLOAD, nframes=T, workload=SPARSE_WORKLOAD["workload"].replace(
            "sparse", "event_lists")),
        "cpu_baseline": dict(vals[-1], value=v),
        "e2e": {"value": v, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------- serving mix
SERVING_WORKLOAD = {
    "workload": "serving_mix",
    "frame_shapes": [[256, 256], [514, 1030], [1062, 1028]], "nframes": "log-uniform 500-20000",
    "n_bins": "uniform 4-64", "dtype": "uint8 or uint16 (even odds)", "rho": 0.99, "mean_photons": 1.0,
    "qmask": "n_bins equal annuli r 0 to 0.4 min(H, W) around the frame centre", "seed": 5, "jobs": 24,
    "hbm_budget_gb": 150,
    "inputs": "device-resident frame pools (one per shape and dtype, 20,000 frames); a job's frames are the "
              "first T frames of its pool, used in place (the server copies nothing in); the host_submission "
              "point submits the same frames from page-locked host pools, so each job's copy to the device is "
              "inside its latency, at 0.8 x the one-at-a-time capacity of host submission",
    "policies": "batched = oldest job first while at most 4 jobs are queued, packing or running, shortest "
                "remaining first beyond (G2Server policy 'auto'); batched_srpt = shortest remaining first always",
}


def make_serving_jobs(dev, n_jobs, seed):
    import numpy as np
    import torch
    from dynamix_gb300.speckle import annular_qmask, speckle_torch
    rng = np.random.default_rng(seed)
    shapes = [tuple(s) for s in SERVING_WORKLOAD["frame_shapes"]]
    spec = []
    for _ in range(n_jobs):
        shape = shapes[int(rng.integers(len(shapes)))]
        T = int(round(math.exp(rng.uniform(math.log(500), math.log(20000)))))
        nb = int(rng.integers(4, 65))
        u16 = bool(rng.integers(2))
        spec.append((shape, T, nb, u16))
    pools = {}
    for shape in shapes:
        need = [T for s, T, _, _ in spec if s == shape]
        if not need:
            continue
        u8 = speckle_torch(max(need), shape, SERVING_WORKLOAD["rho"], SERVING_WORKLOAD["mean_photons"],
                           seed=seed + shapes.index(shape), device=dev)
        pools[(shape, False)] = u8
        if any(s == shape and u for s, _, _, u in spec):
            w = torch.empty(u8.shape, dtype=torch.int16, device=dev)
            w.copy_(u8)
            pools[(shape, True)] = w.view(torch.uint16)
    masks = {}
    jobs = []
    for shape, T, nb, u16 in spec:
        if (shape, nb) not in masks:
            masks[(shape, nb)] = annular_qmask(shape, nb, 0.0, 0.4 * min(shape))
        qm = masks[(shape, nb)]
        npx = int((qm > 0).sum())
        jobs.append({"frames": pools[(shape, u16)][:T], "qmask": qm, "shape": shape, "T": T, "n_bins": nb,
                     "dtype": "uint16" if u16 else "uint8", "gram_ops": float(npx) * T * (T + 1)})
    return jobs, pools


def drive(server, jobs, arrivals):
    """Submit job i at ``arrivals[i]`` seconds after the start, serve until all
    are done; returns (requests, wall seconds)."""
    t0 = time.perf_counter()
    reqs = [None] * len(jobs)
    nxt = 0
    while True:
        now = time.perf_counter() - t0
        while nxt < len(jobs) and arrivals[nxt] <= now:
            reqs[nxt] = server.submit(jobs[nxt]["frames"], jobs[nxt]["qmask"])
            reqs[nxt].t_submit = t0 + arrivals[nxt]
            nxt += 1
        worked = server.step()
        if nxt == len(jobs) and server.idle():
            break
        if not worked:
            time.sleep(0.0001)
    wall = time.perf_counter() - t0
    for r in reqs:
        r.wait()
    return reqs, wall


def latency_summary(reqs, wall, jobs):
    import numpy as np
    lat = np.array([r.latency for r in reqs]) * 1e3
    frames = sum(j["T"] for j in jobs)
    ops = sum(j["gram_ops"] for j in jobs)
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "max_ms": float(lat.max()), "wall_s": wall,
            "jobs_per_s": len(reqs) / wall, "frames_per_s": frames / wall, "gram_tops": ops / wall / 1e12}


def host_pools(pools, jobs):
    """Page-locked host copies of the frame pools, each as long as its longest
    job: numpy arrays registered with the CUDA runtime (torch's pinned
    allocator would round every pool up to a power of two).  None when they
    would take more than half of the host's available memory."""
    import numpy as np
    import torch
    need = {}
    for j in jobs:
        key = (tuple(j["shape"]), j["dtype"] == "uint16")
        need[key] = max(need.get(key, 0), j["T"])
    total = sum(pools[k][:T].numel() * pools[k].element_size() for k, T in need.items())
    avail = None
    try:
        with open("/proc/meminfo") as f:
            for ln in f:
                if ln.startswith("MemAvailable:"):
                    avail = int(ln.split()[1]) * 1024
    except OSError:
        pass
    if avail is None or total > avail // 2:
        return None, total, avail
    cudart = torch.cuda.cudart()
    out = {}
    for k, T in need.items():
        src = pools[k][:T]
        host = np.empty(tuple(src.shape), dtype=np.uint16 if k[1] else np.uint8)
        t = torch.from_numpy(host.view(np.int16) if k[1] else host)
        rc = cudart.cudaHostRegister(t.data_ptr(), host.nbytes, 0)
        if int(rc) != 0:
            for h, _ in out.values():
                cudart.cudaHostUnregister(h.ctypes.data)
            return None, total, avail
        t.copy_(src.view(torch.int16) if k[1] else src)
        out[k] = (host, t.view(torch.uint16) if k[1] else t)
    return out, total, avail


def serving_host_point(jobs, pools, gaps, server, ref, load=0.8):
    """One sweep point with every job submitted from page-locked host memory
    (its copy to the device inside its latency): the one-at-a-time capacity
    of host submission first (all jobs queued at once), then Poisson
    arrivals at ``load`` x that capacity for both servers."""
    import gc

    import numpy as np
    import torch
    hp, total, avail = host_pools(pools, jobs)
    if hp is None:
        return {"skipped": "host pools of %.1f GB do not fit half of the %s available" % (
            total / 1e9, "unknown" if avail is None else "%.1f GB" % (avail / 1e9))}
    try:
        torch.cuda.synchronize()
        hjobs = [dict(j, frames=hp[(tuple(j["shape"]), j["dtype"] == "uint16")][1][:j["T"]]) for j in jobs]

        def fresh(kind):
            # each run's server starts from a released allocator cache: the
            # servers of the device sweep and earlier runs (staging arenas,
            # packed operands) leave it close to the whole device
            gc.collect()
            torch.cuda.synchronize()
            torch.cuda.empty_cache()
            return server(kind)

        drive(fresh("batched"), hjobs, [0.0] * len(hjobs))      # warm-up
        q_reqs, q_wall = drive(fresh("one_at_a_time"), hjobs, [0.0] * len(hjobs))
        capacity = len(hjobs) / q_wall
        rate = load * capacity
        arrivals = np.cumsum(gaps / rate) - gaps[0] / rate
        row = {"one_at_a_time_capacity_jobs_per_s": capacity, "load_vs_one_at_a_time_capacity": load,
               "rate_jobs_per_s": rate,
               "h2d_bytes": int(sum(j["frames"].numel() * j["frames"].element_size() for j in hjobs))}
        identical = all(np.array_equal(r.numerator, q.numerator) for r, q in zip(q_reqs, ref))
        for kind in ("batched", "one_at_a_time"):
            reqs, wall = drive(fresh(kind), hjobs, arrivals)
            row[kind] = latency_summary(reqs, wall, hjobs)
            identical &= all(np.array_equal(r.numerator, q.numerator) and np.array_equal(r.denominator, q.denominator)
                             for r, q in zip(reqs, ref))
        row["p99_speedup"] = row["one_at_a_time"]["p99_ms"] / row["batched"]["p99_ms"]
        row["identical"] = identical
        return row
    finally:
        torch.cuda.synchronize()
        cudart = torch.cuda.cudart()
        for host, _ in hp.values():
            cudart.cudaHostUnregister(host.ctypes.data)


def run_serving(args):
    import numpy as np
    import torch

    from dynamix_gb300 import build as b
    from dynamix_gb300.serving import G2Server

    rank, world, local = dist_info()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    b.build(force=False)
    n_jobs = SERVING_WORKLOAD["jobs"]
    t_gen = time.perf_counter()
    jobs, pools = make_serving_jobs(dev, n_jobs, SERVING_WORKLOAD["seed"])
    torch.cuda.synchronize(dev)
    t_gen = time.perf_counter() - t_gen
    budget = SERVING_WORKLOAD["hbm_budget_gb"] * 1e9
    uuid = None
    try:
        uuid = "GPU-" + str(torch.cuda.get_device_properties(dev).uuid)
    except Exception:
        pass

    def server(kind):
        if kind == "batched":
            return G2Server(hbm_budget=budget)
        if kind == "batched_srpt":
            return G2Server(hbm_budget=budget, policy="srpt")
        if kind == "one_at_a_time":
            return G2Server(hbm_budget=budget, max_active=1, slice_ops=1e30)
        return G2Server(hbm_budget=budget, max_active=1, slice_ops=1e30, method="plain")

    # warm-up (layouts of every q-mask, allocator pools) and the reference results
    ref, _ = drive(server("batched"), jobs, [0.0] * n_jobs)
    # service capacity of one-job-at-a-time execution (all jobs queued at t = 0)
    seq_reqs, seq_wall = drive(server("one_at_a_time"), jobs, [0.0] * n_jobs)
    capacity = n_jobs / seq_wall
    rng = np.random.default_rng(SERVING_WORKLOAD["seed"] + 100)
    gaps = rng.exponential(1.0, n_jobs)
    sampler = ClockSampler(uuid)
    sampler.start()
    sweep = []
    identical = True
    for load in (0.5, 0.8, 1.0, 1.5):
        rate = load * capacity
        arrivals = np.cumsum(gaps / rate) - gaps[0] / rate
        row = {"load_vs_one_at_a_time_capacity": load, "rate_jobs_per_s": rate}
        for kind in ("batched", "batched_srpt", "one_at_a_time"):
            reqs, wall = drive(server(kind), jobs, arrivals)
            row[kind] = latency_summary(reqs, wall, jobs)
            identical &= all(np.array_equal(r.numerator, q.numerator) and np.array_equal(r.denominator, q.denominator)
                             for r, q in zip(reqs, ref))
        row["p99_speedup"] = row["one_at_a_time"]["p99_ms"] / row["batched"]["p99_ms"]
        sweep.append(row)
    host_point = serving_host_point(jobs, pools, gaps, server, ref)
    if host_point is not None:
        identical &= host_point.pop("identical")
    clocks = sampler.stop()
    plain = None
    if not args.no_plain:
        p_reqs, p_wall = drive(server("plain"), jobs, [0.0] * n_jobs)
        plain = latency_summary(p_reqs, p_wall, jobs)
        identical &= all(np.array_equal(r.numerator, q.numerator) for r, q in zip(p_reqs, ref))
    top = sweep[-1]
    line = {
        "metric": "serving_p99_latency_ms", "value": top["batched"]["p99_ms"], "unit": "ms", "n_gpus": 1,
        "steps": n_jobs, "warmup": 1, "higher_is_better": False, "scaling": "none", "vs_baseline": None,
        "dtype": "u8/u16", "data": "synthetic",
        "config": dict(SERVING_WORKLOAD, pool_generation_s=t_gen),
        "jobs": [{k: (list(v) if k == "shape" else v) for k, v in j.items() if k not in ("frames", "qmask")}
                 for j in jobs],
        "one_at_a_time_capacity_jobs_per_s": capacity, "sweep": sweep, "host_submission": host_point,
        "plain_one_at_a_time_all_queued": plain, "results_identical_across_runs": bool(identical),
        "clocks": clocks,
    }
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------- u16 precision stress
U16_WORKLOAD = {
    "workload": "dense_256x256_u16_T5000_12bins",
    "frame_shape": [256, 256], "nframes": 5000, "dtype": "uint16", "max_count": 4095, "n_bins": 12,
    "qmask": "12 equal annuli r 8-128 px around (128, 128)", "rho": 0.995, "mean_photons": 50.0, "seed": 3,
    "l2": "inputs (655 MB) larger than L2; no flush",
}
U16_ORACLE_FRAMES = 1024


def measure_u16(args, dev, T, steps, warmup, cpu=True, e2e=True):
    """The precision-stress line: 256 x 256 u16 counts <= 4095 (mean 50), 12
    bins, through MatMulCorrelator (the operand the counts allow: fp16 counts
    <= 2048 here), plus the same stack forced onto the hi/lo byte planes
    (4 Grams per bin, the split the configuration is meant to exercise), each
    with the float32 g2's largest relative error per bin against the FP64
    oracle on the first frames and N/D bit-exactness there."""
    import numpy as np
    import torch

    from dynamix_gb300 import _lib as L
    from dynamix_gb300.correlator import MatMulCorrelator
    from dynamix_gb300.plan import gram_macs
    from dynamix_gb300.speckle import annular_qmask, speckle_torch
    from oracle.g2_oracle import g2_exact

    H, W = U16_WORKLOAD["frame_shape"]
    qmask = annular_qmask((H, W), U16_WORKLOAD["n_bins"], 8.0, 128.0, center=(128, 128))
    frames = speckle_torch(T, (H, W), U16_WORKLOAD["rho"], U16_WORKLOAD["mean_photons"], seed=U16_WORKLOAD["seed"],
                           dtype="uint16", max_count=U16_WORKLOAD["max_count"], device=dev)
    npix = np.bincount(qmask.ravel(), minlength=U16_WORKLOAD["n_bins"] + 1)[1:]
    macs = gram_macs(T, npix)
    stream = torch.cuda.current_stream(dev)
    peak_f16, _ = tc_rate(dev, L.KIND_FP16)
    Ts = min(U16_ORACLE_FRAMES, T)
    sub = frames[:Ts].cpu().numpy()
    ref = g2_exact(sub, qmask)

    def one(operand):
        corr = MatMulCorrelator((H, W), T, qmask=qmask, extra_options={"operand": operand})
        eng = corr.engine
        for _ in range(max(warmup, 3)):
            corr.correlate_device(frames)
        eng.check_error()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        with no_gc():
            e0.record(stream)
            for _ in range(steps):
                corr.correlate_device(frames)
            e1.record(stream)
            torch.cuda.synchronize(dev)
        eng.check_error()
        ms = e0.elapsed_time(e1) / steps
        info = dict(eng.last)
        eng.profile = True
        corr.correlate_device(frames)
        st = eng.stage_times(eng.take_events())
        eng.profile = False
        planes = 4 if info["mode"] == "bytes" else 1
        gram = st.get("gram_tc", float("nan"))
        executed = 2.0 * macs * planes / (gram / 1e3) / 1e12
        c2 = MatMulCorrelator((H, W), Ts, qmask=qmask, extra_options={"operand": operand})
        g32 = c2.correlate(sub)
        exact = bool(np.array_equal(c2.numerator, ref["numerator"]) and np.array_equal(c2.denominator,
                                                                                        ref["denominator"]))
        with np.errstate(divide="ignore", invalid="ignore"):
            rel = np.abs(g32.astype(np.float64) - ref["g2"]) / np.abs(ref["g2"])
        per_bin = [float(np.nanmax(r)) if np.isfinite(r).any() else None for r in rel]
        out = {
            "metric": "g2_frames_per_s", "value": T / (ms / 1e3), "unit": "frames/s", "n_gpus": 1, "steps": steps,
            "warmup": max(warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u16", "data": "synthetic", "config": dict(U16_WORKLOAD, nframes=T),
            "plan": info, "stages_ms": st,
            "tiles": {"block": {"pair": "256 x n (tcgen05 cta_group::2 M256)",
                                "wide": "256 x 512 (two tcgen05 cta_group::2 M256 N256)",
                                "single": "128 x 256 (tcgen05 M128 N256)"}[info.get("tile", "single")],
                      "k_stage": "64 fp16 columns per TMA stage",
                      "operand": info["mode"], "grams_per_bin": planes, "k_split_chunks": info.get("n_grams"),
                      "autotuner_candidates": "tile, pipeline chunks, operand (dynamix_gb300.tune)"},
            "roofline": {"bound": "tensor", "achieved": executed, "peak": peak_f16, "unit": "TFLOP/s",
                         "frac": executed / peak_f16,
                         "kernel": {"pair": "g2_gram_tc_pair", "wide": "g2_gram_tc_wide"}.get(info.get("tile"),
                                                                                             "g2_gram_tc"),
                         "launch_ms": gram,
                         "peak_source": "tcgen05 kind::f16 rate measured in this run (g2_tc_rate_probe); executed "
                                        "ops = %d x the algorithmic %.3e" % (planes, 2.0 * macs)},
            "fp64_check": {"frames": Ts, "numerator_denominator_bit_exact": exact,
                           "max_rel_err_float32_g2_vs_fp64_per_bin": per_bin},
            "gpu_launches": 4 * steps,
        }
        return corr, out

    corr, line = one("auto")
    if e2e:
        host = frames.cpu().pin_memory()
        for _ in range(max(3, warmup)):
            corr.correlate(host)
        torch.cuda.synchronize(dev)
        with no_gc():
            t0 = time.perf_counter()
            per_call = []
            for _ in range(steps):
                t1 = time.perf_counter()
                corr.correlate(host)                   # returns host arrays: synchronous
                per_call.append((time.perf_counter() - t1) * 1e3)
            torch.cuda.synchronize(dev)
        e2e_ms = (time.perf_counter() - t0) * 1e3 / steps
        line["e2e"] = {"value": T / (e2e_ms / 1e3), "unit": "frames/s", "ms_per_step": e2e_ms,
                       "h2d_bytes_per_step": int(host.numel() * host.element_size()),
                       "d2h_bytes_per_step": int(U16_WORKLOAD["n_bins"] * T * 12 + 4),
                       "ms_per_call_min_median_max": [min(per_call), sorted(per_call)[len(per_call) // 2],
                                                      max(per_call)]}
        del host
    del corr
    _, line["byte_planes"] = one("bytes")
    if cpu:
        ts, kind, label = cpu_port_time(frames.cpu().numpy(), qmask)
        ncores = host_cores()
        line["cpu_baseline"] = {"value": T / ts[0], "unit": "frames/s", "cores": ncores, "kind": kind,
                                "sample": "the whole stack (all %d frames, 12 bins): %s, %d threads, %.2f s"
                                          % (T, label, ncores, ts[0])}
    return line


def run_u16(args):
    import torch
    from dynamix_gb300 import build as b
    rank, world, local = dist_info()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    b.build(force=False)
    print(json.dumps(measure_u16(args, dev, args.frames, args.steps, args.warmup, cpu=not args.no_cpu,
                                 e2e=not args.no_e2e)))
    return 0


COMPRESS_WORKLOAD = {
    "workload": "compress_514x1030_u8_T10000",
    "frame_shape": [514, 1030], "nframes": 10000, "dtype": "uint8", "rho": 0.99, "mean_photons": 0.1, "seed": 1,
    "operation": "compress_all_stack (dense stack -> per-pixel event lists, times int32 + values u8 + offsets)",
    "l2": "input stack (5.3 GB) larger than L2; no flush",
}


def compress_config(T, **extra):
    """The compression workload's config for a stack of T frames."""
    H, W = COMPRESS_WORKLOAD["frame_shape"]
    cfg = dict(COMPRESS_WORKLOAD, nframes=T, workload="compress_%dx%d_u8_T%d" % (H, W, T),
               l2="input stack (%.2f GB) %s than L2; no flush" % (T * H * W / 1e9,
                                                                 "larger" if T * H * W > 129e6 else "smaller"))
    cfg.update(extra)
    return cfg
COMPRESS_CPU_FRAMES = 256


def run_compress(args):
    """Device frame compression of the 514 x 1030 x 10,000 u8 stack (frames already in
    HBM for ``value``; from pinned host memory, events copied back, for e2e)."""
    import numpy as np
    import torch

    from dynamix_gb300 import build as b
    from dynamix_gb300.compress import StackCompressor
    from dynamix_gb300.speckle import speckle_torch

    rank, world, local = dist_info()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    b.build(force=False)
    T = args.frames
    H, W = COMPRESS_WORKLOAD["frame_shape"]
    npix = H * W
    frames = speckle_torch(T, (H, W), COMPRESS_WORKLOAD["rho"], COMPRESS_WORKLOAD["mean_photons"],
                           seed=COMPRESS_WORKLOAD["seed"], dtype="uint8", device=dev).reshape(T, npix)
    comp = StackCompressor(T, npix, device=dev)
    stream = torch.cuda.current_stream(dev)

    def barrier():
        torch.cuda.synchronize(dev)
        if dist is not None:
            dist.barrier()

    def max_over_ranks(x):
        from dynamix_gb300.replicas import max_over_ranks as mx
        return mx(x, dist, dev)

    for _ in range(max(args.warmup, 3)):
        comp.run(frames)
    n_ev = comp.n_events
    uuid = None
    try:
        uuid = "GPU-" + str(torch.cuda.get_device_properties(dev).uuid)
    except Exception:
        pass
    sampler = ClockSampler(uuid)
    barrier()
    sampler.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    comp.profile = True  # CUDA events between the passes of every timed call
    with no_gc():
        e0.record(stream)
        for _ in range(args.steps):
            comp.run(frames)
        e1.record(stream)
        barrier()
    clocks = sampler.stop()
    comp.profile = False
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps)
    st = comp.stage_times(calls=args.steps)
    stack_bytes = T * npix
    out_bytes = n_ev * 5 + (npix + 1) * 8
    peaks, peak_kind = measured_peaks()
    # dominant kernel: the stage pass (reads the stack, writes a 4-byte word per event);
    # the count pass reads the stack once more, the gather moves the words to the lists
    count_gbs = stack_bytes / (st["count"] / 1e3) / 1e9
    stage_bytes = stack_bytes + n_ev * 4
    stage_gbs = stage_bytes / (st["stage"] / 1e3) / 1e9
    traffic = profile_traffic("launches_compress_514x1030_T10000.md")
    if traffic is not None:
        traffic *= T / COMPRESS_WORKLOAD["nframes"]
    line = {
        "metric": "compress_frames_per_s", "value": world * T / (ms / 1e3), "unit": "frames/s", "n_gpus": world,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": compress_config(T, n_events=n_ev, parallelism="replicas" if world > 1 else "single"),
        "hbm_GB_per_s_step": (stack_bytes + out_bytes) / (ms / 1e3) / 1e9,
        "stages_ms": st,
        "roofline": {"bound": "hbm", "achieved": stage_gbs, "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                     "frac": stage_gbs / peaks.get("hbm_gbs"), "traffic": traffic, "kernel": "g2_compress_stage",
                     "peak_source": "%s hbm_gbs" % peak_kind,
                     "algorithmic_bytes_per_launch": stage_bytes, "launch_ms": st["stage"],
                     "count_pass_GB_per_s": count_gbs,
                     "note": "two passes read the stack (count, stage); the algorithmic minimum reads it once"},
        "clocks": clocks, "gpu_launches": 8 * args.steps,
    }
    if rank == 0 and not args.no_e2e:
        host = torch.empty((T, npix), dtype=torch.uint8, pin_memory=True)
        host.copy_(frames)
        dfr = torch.empty_like(frames)
        out_h = {}

        def e2e_step():
            dfr.copy_(host, non_blocking=True)
            d, t, off = comp.run(dfr)
            for k, x in (("d", d), ("t", t), ("o", off)):
                buf = out_h.get(k)
                if buf is None or buf.numel() < x.numel() or buf.dtype != x.dtype:
                    buf = out_h[k] = torch.empty(x.numel() + 1024, dtype=x.dtype, pin_memory=True)
                buf[:x.numel()].copy_(x, non_blocking=True)
            torch.cuda.synchronize(dev)
            return d.numel() * 5 + off.numel() * 8

        for _ in range(2):
            e2e_step()
        with no_gc():
            t0 = time.perf_counter()
            d2h = 0
            for _ in range(args.steps):
                d2h = e2e_step()
            e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
        line["e2e"] = {"value": T / (e2e_ms / 1e3), "unit": "frames/s", "ms_per_step": e2e_ms,
                       "h2d_bytes_per_step": stack_bytes, "d2h_bytes_per_step": d2h,
                       "path": "pinned host stack -> device -> StackCompressor.run -> pinned host events"}
        del host, dfr
    if rank == 0 and not args.no_cpu:
        from oracle.g2_oracle import compress_all_stack
        Ts = min(COMPRESS_CPU_FRAMES, T)
        sample = frames[:Ts].reshape(Ts, H, W).cpu().numpy()
        t0 = time.perf_counter()
        compress_all_stack(sample)
        sec = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": Ts / sec, "unit": "frames/s", "cores": 1, "kind": "port",
                                "sample": "numpy restatement of compress_all_stack on the first %d frames" % Ts}
    if rank == 0:
        print(json.dumps(line))
    return 0


def run_compress_reference(args):
    """The reference's compress_all_stack is numpy on the host (event.py:267-284):
    its restatement timed on a bounded sample of the same stack."""
    import torch
    rank, world, local = dist_info()
    if rank != 0:
        return 0
    from dynamix_gb300.speckle import speckle_torch
    from oracle.g2_oracle import compress_all_stack
    T = args.frames
    H, W = COMPRESS_WORKLOAD["frame_shape"]
    dev = torch.device("cuda", local)
    Ts = min(COMPRESS_CPU_FRAMES, T)
    sample = speckle_torch(T, (H, W), COMPRESS_WORKLOAD["rho"], COMPRESS_WORKLOAD["mean_photons"],
                           seed=COMPRESS_WORKLOAD["seed"], dtype="uint8", device=dev)[:Ts].cpu().numpy()
    for _ in range(args.warmup):
        compress_all_stack(sample)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        compress_all_stack(sample)
    sec = (time.perf_counter() - t0) / args.steps
    v = Ts / sec
    line = {
        "metric": "compress_frames_per_s", "value": v, "unit": "frames/s", "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": T / v * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": compress_config(T),
        "cpu_baseline": {"value": v, "unit": "frames/s", "cores": 1, "kind": "port",
                         "sample": "each step: numpy compress_all_stack on the first %d of %d frames" % (Ts, T)},
        "e2e": {"value": v, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def main():
    args = parse()
    if args.workload == "serving":
        return run_serving(args)
    if args.workload == "compress":
        if args.frames is None:
            args.frames = COMPRESS_WORKLOAD["nframes"]
        if args.impl == "reference":
            return run_compress_reference(args)
        return run_compress(args)
    if args.workload == "u16":
        if args.frames is None:
            args.frames = U16_WORKLOAD["nframes"]
        return run_u16(args)
    if args.workload in ("sparse", "event"):
        if args.frames is None:
            args.frames = SPARSE_WORKLOAD["nframes"]
        return (run_sparse_reference if args.impl == "reference" else run_sparse)(args)
    if args.frames is None:
        args.frames = WORKLOAD["nframes"]
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
