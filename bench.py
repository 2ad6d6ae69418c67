#!/usr/bin/env python
"""Throughput of the BriefMatch flow engine on GB300: output flow Mpx/s.

Workload (one "step"): a seeded synthetic 8-frame 1024x436 8-bit sequence (7
consecutive pairs, flow redrawn per pair, |v| <= 15 px), up-sampling 2.9x2.9,
feature_length 128, FP32 flow output, temporal initialisation between pairs --
the reference's "moderate" setting.  Synthetic frames stand in for the public
benchmark sequences.

  value    7 pairs * 1024*436 output pixels / device time per step (frames
           already in HBM as uint8, outputs left in HBM); L2 flushed between steps.
           Two engines are measured: the plain engine (the reference's method and
           schedule) and the learned-seeded engine (the trained proposal seeds
           matching; its schedule is the fastest whose EPE on each of three separate
           calibration sequences is at most the plain engine's).  The headline is
           the learned-seeded engine when its EPE on the measured sequence is at
           most the plain engine's, else the plain engine; both are reported.
  e2e      the same through the public C ABI with pinned host frames in and host
           flow out (H2D and D2H inside the timed region)
  roofline the dominant kernel's algorithmic bytes per launch over its mean
           CUDA-event duration, against the measured HBM copy bandwidth
  cpu_baseline  the oracle (scalar C + OpenMP transcription of the reference
           kernels) on a bounded sample of the same workload, host cores

`--impl reference` times the reference's own implementation of the path.  The
reference has no CPU path, so its CPU-timed arm is the oracle transcription (all
host threads), per the one-pair sample per step; the line also carries the
reference's own CUDA kernels (compiled from its sources) timed on the GPU over
the full step, when that build is present.

Multi-GPU: one process per GPU (torchrun); each rank runs an independent
replica on its own sequence (pairs shard with no exchange), value = all ranks'
pixels / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "output flow Mpx/s at fixed EPE: batched+learned-seeded vs plain, same GB300"
UNIT = "Mpx/s"
# the workload configurations: width, height, frames per sequence, up-sampling,
# feature_length, max |v|.  "2" is the one the metric is quoted on (the default);
# "1" and "3" are the reference's small case and the 1920x1080 u4.9 N512 stress case,
# timed beside the reference's own kernels with --config.
CONFIGS = {"1": (584, 388, 2, 1.5, 32, 10.0), "2": (1024, 436, 8, 2.9, 128, 15.0), "3": (1920, 1080, 5, 4.9, 512, 24.0)}
SEED = 20261203


def set_config(name):
    global W, H, FRAMES, UP, NBITS, VMAX, PAIRS
    W, H, FRAMES, UP, NBITS, VMAX = CONFIGS[name]
    PAIRS = FRAMES - 1


set_config("2")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-pairs", type=int, default=2, help="pairs in the CPU-baseline sample")
    ap.add_argument("--no-batched", action="store_true", help="skip the 64-pair batched workload")
    ap.add_argument("--batch-pairs", type=int, default=64)
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-seeded engine")
    ap.add_argument("--no-pipelined", action="store_true", help="finish every frame before the next")
    ap.add_argument("--config", default="2", choices=sorted(CONFIGS),
                    help="workload: 1 = 584x388 u1.5 N32 pair, 2 = 1024x436 u2.9 N128 8-frame sequence (default), "
                         "3 = 1920x1080 u4.9 N512 5-frame sequence; 1 and 3 run the plain engine beside the "
                         "reference's own kernels")
    ap.add_argument("--schedule", default=None,
                    help="ITERATIONS/JFMAX[/LOCAL_STEPS[/REDUCE]] for the learned-seeded engine instead of choosing "
                         "it by calibration")
    return ap.parse_args()


def dist_init(torch):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return world, rank


def barrier(torch, world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(torch, world, v):
    if world == 1:
        return v
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_value(world, px_per_rank_step, max_ms_per_step):
    """Whole-job throughput of `world` replicas: all ranks' output pixels per step
    over the slowest rank's step time, in Mpx/s."""
    return world * px_per_rank_step / (max_ms_per_step * 1e-3) / 1e6


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.p:
            time.sleep(0.25)
            self.p.terminate()
            try:
                self.out, _ = self.p.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
                self.out = ""

    def summary(self):
        rows = [r.split(", ") for r in getattr(self, "out", "").strip().splitlines() if r.strip()]
        rows = [r for r in rows if len(r) >= 9]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if "Active" in r[5 + k] and "Not" not in r[5 + k]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, if any.  The
    file's `workload W H up N` line names the workload it was captured on; other
    workloads get None (their working sets sit differently against L2, so the
    traffic does not scale with the pixel count)."""
    path = os.path.join(ROOT, "profiles", "traffic_per_launch.txt")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        lines = [ln.split() for ln in f if ln.strip()]
    for parts in lines:
        if parts[0] == "workload":
            try:
                w, h, up, n = int(parts[1]), int(parts[2]), float(parts[3]), int(parts[4])
            except (IndexError, ValueError):
                return None
            if (w, h, up, n) != (W, H, UP, NBITS):
                return None
    for parts in lines:
        if len(parts) >= 2 and parts[0] == kernel:
                try:
                    return float(parts[1])
                except ValueError:
                    return None
    return None


def synth_module():
    """The seeded synthetic generator (briefmatch_gb300/synth.py, numpy and scipy
    only), loaded from its file so that the reference arm does not import the engine
    package."""
    import importlib.util

    mod = sys.modules.get("bm_bench_synth")
    if mod is None:
        spec = importlib.util.spec_from_file_location("bm_bench_synth", os.path.join(ROOT, "briefmatch_gb300",
                                                                                     "synth.py"))
        mod = importlib.util.module_from_spec(spec)
        sys.modules["bm_bench_synth"] = mod
        spec.loader.exec_module(mod)
    return mod


def make_workload(rank):
    return synth_module().make_sequence(SEED + rank, W, H, FRAMES, vmax=VMAX)


def bench_config(world):
    """The workload both arms report (identical in the engine and reference lines)."""
    return {"workload": "synthetic %dx%d 8-bit sequence of %d frames (%d pair%s, |v|<=%g px), up-sampling %gx%g, "
                        "feature_length %d, temporal init, FP32 flow out"
                        % (W, H, FRAMES, PAIRS, "s" if PAIRS > 1 else "", VMAX, UP, UP, NBITS),
            "width": W, "height": H, "frames_per_step": FRAMES, "pairs_per_step": PAIRS, "upsampling": UP,
            "feature_length": NBITS, "l2": "flushed (256 MB write) before every timed step",
            "parallelism": "replicas" if world > 1 else "single GPU"}


def algorithmic_bytes(kernel, prm):
    """Bytes one launch must move at minimum: per unit (pixel), the data the kernel
    must read and write once."""
    n = prm.sx * prm.sy
    ni = prm.sx_in * prm.sy_in
    ns = (prm.N + 31) // 32
    table = {
        # per pixel and level, the working set each level moves at least once: own
        # descriptor, the gathered frame's descriptor footprint, field read and
        # written (4 B each), cost read and written (2 B each); 44 B at N=128
        "jump_level": n * (2 * ns * 4 + 2 * 4 + 2 * 2),
        "jump_level_rs": n * (2 * ns * 4 + 2 * 4 + 2 * 2),
        # up-sampled image read once, descriptors written once
        "features": n * (4 + ns * 4),
        "initialize": n * (2 * ns * 4 + 4 + 2),
        "upsample_u8": ni + n * 4,
        # five float planes read, two written
        "trilateral": ni * 7 * 4,
        "median_pass": ni * 2 * 2 * 4,
        "downsample": n * 4 + ni * 2 * 4,
        "u8_to_f32": ni * 5,
    }
    return table.get(kernel)


# FP32 operations per output pixel and window tap of the cross-trilateral filter,
# counting a fused multiply-add as two: three differences; the exponent
# cE*(du^2 + dv^2) + cI*dI^2 + cS*d^2 (du^2, dv^2 and dI^2: 3; their scaled sum: 4;
# the spatial term: 1); and the accumulation of w*u, w*v (2 FMA) and w (1) -- 16, plus
# the exponential on the special-function unit.
TRI_FLOP_PER_TAP = 16


def trilateral_flops(prm):
    """Algorithmic FP32 FLOPs of one cross-trilateral launch: every output pixel
    visits a (2s)^2 window, s = ceil(2.5 * sS) (briefmatch_cuda.cu:266)."""
    import math

    s = int(math.ceil(2.5 * prm.sS))
    return prm.sx_in * prm.sy_in * (2 * s) ** 2 * TRI_FLOP_PER_TAP


def fp32_peak_tflops(torch, sm_mhz):
    """Nominal FP32 FMA throughput of the device: SMs x 128 lanes x 2 FLOP x SM clock."""
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    return sms * 128 * 2 * (sm_mhz or 2070.0) * 1e6 / 1e12


def roofline_entry(torch, kernel, n_launch, k_ms, total_k, prm, clocks):
    """Roofline of one kernel: FP32-bound for the trilateral filter (against the
    nominal FP32 FMA rate: no measured FP32 peak exists), HBM-bound for the rest
    (against the measured copy bandwidth)."""
    per_launch_ms = k_ms / n_launch
    if kernel == "trilateral":
        flops = trilateral_flops(prm)
        peak = fp32_peak_tflops(torch, clocks.get("sm_max_mhz"))
        achieved = flops / (per_launch_ms * 1e-3) / 1e12
        return {"kernel": kernel, "bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "peak_source": "nominal (SMs x 128 FP32 lanes x 2 FLOP x max SM clock); "
                "MEASURED_PEAKS.json has no FP32 figure", "algorithmic_flops_per_launch": flops,
                "flop_per_tap": TRI_FLOP_PER_TAP, "launch_ms": per_launch_ms, "launches": n_launch,
                "share_of_kernel_time": k_ms / total_k if total_k else None, "traffic": ncu_traffic(kernel)}
    abytes = algorithmic_bytes(kernel, prm)
    peak, peak_src = measured_peaks()
    achieved = abytes / (per_launch_ms * 1e-3) / 1e9 if abytes else None
    return {"kernel": kernel, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None,
            "peak_source": peak_src + " (MEASURED_PEAKS.json hbm_gbs)", "algorithmic_bytes_per_launch": abytes,
            "launch_ms": per_launch_ms, "launches": n_launch,
            "share_of_kernel_time": k_ms / total_k if total_k else None, "traffic": ncu_traffic(kernel)}


PROPOSAL_CONF = 0.5
PIPELINED = True   # each pair's refinement overlaps the next frame (bm_set_pipelined)
# (iterations, jfMax, local refinement steps starting at radius 2, input reduction of
# the network).  The sequence's frames are close to the network's 512x384 training
# frames, so its input is not reduced: reduction 2 (cells of 8 px) passed all three
# calibration sequences at 1/16 and then lost to the plain engine on the measured one
CANDIDATE_REDUCE = 1
SCHEDULE_CANDIDATES = tuple((it, jf, ls, CANDIDATE_REDUCE) for it, jf in ((1, 16), (1, 32), (1, 64), (1, 128), (1, 256),
                                                                         (2, 16), (2, 32), (2, 64)) for ls in (0, 2))


def open_engine(torch, prm, pattern, stream, net=None, schedule=None):
    import briefmatch_gb300 as bm

    eng = bm.BriefMatch(prm)
    eng.setup()
    eng.set_pattern(pattern)
    eng.set_stream(stream.cuda_stream)
    if net is not None:
        bm.set_proposal(eng, net, PROPOSAL_CONF, schedule[0], schedule[1])
        if len(schedule) > 2 and schedule[2]:
            bm.set_local_steps(eng, schedule[2], 2)
        if len(schedule) > 3 and schedule[3] != 1:
            bm.set_proposal_reduce(eng, schedule[3])
    if PIPELINED:
        eng.set_pipelined(True)
    return eng


def sequence_step(eng, frame_ptrs, u_ptrs, v_ptrs, on_device):
    """One step: the whole sequence from the same random-stream position.  With
    pipelined frames the engine stream then waits for the last refinement, so work
    queued after the step (the end event) follows all of it."""
    eng.reset_sequence()
    eng.set_rng_position(0)
    eng.frame(frame_ptrs[0], on_device)
    for k in range(1, len(frame_ptrs)):
        eng.frame(frame_ptrs[k], on_device, u_ptrs[k - 1], v_ptrs[k - 1], on_device)
    eng.join()


def mean_epe(u, v, flows):
    import numpy as np

    return [float(np.mean(np.hypot(u[k] - flows[k][0], v[k] - flows[k][1]))) for k in range(len(flows))]


def measure(args, torch, world, eng, d_frames, flows, stream, flush):
    """Device throughput of one engine over the sequence: W warm-up steps, then K
    steps timed with CUDA events on the engine stream, L2 flushed before each step
    (outside the events), SM clocks sampled over the timed region.  A second run of
    K steps records a CUDA event pair around every launch (the engine's per-kernel
    profile, which the roofline uses); its own step time is reported beside the
    first, which carries no per-launch events."""
    npairs = d_frames.shape[0] - 1
    d_u = torch.empty(npairs, H, W, device="cuda")
    d_v = torch.empty(npairs, H, W, device="cuda")
    fp = [d_frames[k].data_ptr() for k in range(npairs + 1)]
    up = [d_u[k].data_ptr() for k in range(npairs)]
    vp = [d_v[k].data_ptr() for k in range(npairs)]
    for _ in range(args.warmup):
        sequence_step(eng, fp, up, vp, True)
    torch.cuda.synchronize()

    def timed(profiled):
        if profiled:
            eng.profile(True)
            eng.profile_reset()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        launches0 = eng.launch_count()
        with ClockSampler(torch.cuda.current_device()) as clk:
            barrier(torch, world)
            torch.cuda.synchronize()
            for i in range(args.steps):
                flush.zero_()
                starts[i].record(stream)
                sequence_step(eng, fp, up, vp, True)
                ends[i].record(stream)
            torch.cuda.synchronize()
            barrier(torch, world)
        launches = eng.launch_count() - launches0
        total_ms = max_over_ranks(torch, world, sum(s.elapsed_time(e) for s, e in zip(starts, ends)))
        kstats = None
        if profiled:
            kstats = eng.profile_read()
            eng.profile(False)
        return total_ms / args.steps, launches, clk.summary(), kstats

    ms, launches, clocks, _ = timed(False)
    # the per-kernel profile (roofline, kernel table) with each frame finished before
    # the next: with pipelined frames a launch's events would also span the work of
    # the other stream running beside it
    if PIPELINED:
        eng.set_pipelined(False)
    ms_prof, _, _, kstats = timed(True)
    if PIPELINED:
        eng.set_pipelined(True)
    u, v = d_u.cpu().numpy(), d_v.cpu().numpy()
    return {"ms_per_step": ms, "value": aggregate_value(world, npairs * W * H, ms), "launches": launches,
            "kstats": kstats, "ms_per_step_profiled": ms_prof, "clocks": clocks, "epe": mean_epe(u, v, flows),
            "u": u, "v": v}


def measure_e2e(args, torch, world, eng, frames, u_dev, v_dev, flush):
    """The same step through the public C ABI with pinned host frames in and host
    flow out: host-to-device and device-to-host copies inside the timed region."""
    import numpy as np

    npairs = len(frames) - 1
    h_frames = torch.from_numpy(np.stack(frames)).pin_memory()
    h_u = torch.empty(npairs, H, W).pin_memory()
    h_v = torch.empty(npairs, H, W).pin_memory()
    fp = [h_frames[k].data_ptr() for k in range(npairs + 1)]
    up = [h_u[k].data_ptr() for k in range(npairs)]
    vp = [h_v[k].data_ptr() for k in range(npairs)]
    for _ in range(max(1, args.warmup)):
        sequence_step(eng, fp, up, vp, False)
    torch.cuda.synchronize()
    e2e_ms = 0.0
    barrier(torch, world)
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sequence_step(eng, fp, up, vp, False)
        torch.cuda.synchronize()
        e2e_ms += (time.perf_counter() - t0) * 1e3
    e2e_ms = max_over_ranks(torch, world, e2e_ms)
    assert np.array_equal(h_u.numpy(), u_dev) and np.array_equal(h_v.numpy(), v_dev), "host and device paths disagree"
    return {"value": world * npairs * W * H / (e2e_ms / args.steps * 1e-3) / 1e6, "unit": UNIT,
            "h2d_bytes_per_step": int((npairs + 1) * W * H), "d2h_bytes_per_step": int(npairs * 2 * W * H * 4)}


CALIBRATION_SEEDS = (SEED + 7777, SEED + 8888, SEED + 9999)


def choose_schedule(torch, prm, pattern, net, stream):
    """The fastest seeded schedule whose mean EPE on each of three calibration
    sequences (other seeds of the same generator) is at most the plain engine's
    there.  Returns (schedule or None, table)."""
    import numpy as np

    seqs = []
    for sd in CALIBRATION_SEEDS:
        frames, flows = synth_module().make_sequence(sd, W, H, FRAMES, vmax=VMAX)
        d = torch.from_numpy(np.stack(frames)).cuda()
        seqs.append(([d[k].data_ptr() for k in range(FRAMES)], flows, d))
    u = torch.empty(PAIRS, H, W, device="cuda")
    v = torch.empty(PAIRS, H, W, device="cuda")
    up = [u[k].data_ptr() for k in range(PAIRS)]
    vp = [v[k].data_ptr() for k in range(PAIRS)]

    def run(eng):
        """(ms per step summed over the sequences, [mean EPE per sequence])"""
        ms, epes = 0.0, []
        for fp, flows, _ in seqs:
            sequence_step(eng, fp, up, vp, True)   # warm
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(3):
                sequence_step(eng, fp, up, vp, True)
            e1.record(stream)
            torch.cuda.synchronize()
            ms += e0.elapsed_time(e1) / 3
            epes.append(float(np.mean(mean_epe(u.cpu().numpy(), v.cpu().numpy(), flows))))
        eng.clean()
        return ms, epes

    plain_ms, plain_epe = run(open_engine(torch, prm, pattern, stream))
    table = [{"schedule": "plain %d/%d" % (prm.iterations, prm.jfMax), "ms": plain_ms, "epe": plain_epe}]
    best = None
    for sch in SCHEDULE_CANDIDATES:
        ms, epe = run(open_engine(torch, prm, pattern, stream, net, sch))
        table.append({"schedule": "seeded %d/%d/ls%d/x%d" % sch, "ms": ms, "epe": epe})
        if all(e <= p for e, p in zip(epe, plain_epe)) and (best is None or ms < best[1]):
            best = (sch, ms)
    return (best[0] if best else None), table


def net_forward_timing(torch, net, d_frames, stream, reps=50, reduce=1):
    """Device time of the proposal network's input preparation + forward pass for one
    1024x436 pair (256x109 cells of 4 pixels with reduce 1), and its tensor-core rate."""
    from briefmatch_gb300.proposal import flops_per_pixel

    h4, w4 = H // reduce // 4, W // reduce // 4
    out = torch.empty(1, h4, w4, 3, device="cuda")
    st = stream.cuda_stream

    def once():
        net.prepare(0, d_frames[0].data_ptr(), d_frames[1].data_ptr(), W, H, st, reduce=reduce)
        net.forward(1, h4, w4, out.data_ptr(), st)

    for _ in range(5):
        once()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        once()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    flops = flops_per_pixel() * h4 * w4
    return {"ms_per_pair": ms, "gflop_per_pair": flops / 1e9, "tflop_s": flops / (ms * 1e-3) / 1e12,
            "path": {2: "tcgen05, one cooperative launch", 1: "tcgen05, a launch per layer", 0: "mma.sync"}[net.umma],
            "note": "input preparation + 6 conv layers, 1 pair, back to back", "reduce": reduce,
            "cells": [h4, w4]}


def run_engine(args, torch, world, rank):
    import numpy as np

    import briefmatch_gb300 as bm
    from briefmatch_gb300 import learn

    frames, flows = make_workload(rank)
    batch_inputs = None if args.no_batched else make_batch_workload(args.batch_pairs)
    prm = bm.BMParams.derive(W, H, UP, UP, N=NBITS)
    pattern = prm.make_pattern(SEED)
    # one explicit (non-default) stream carries the engine's work, the L2 flush and
    # the timing events
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    d_frames = torch.from_numpy(np.stack(frames)).cuda()
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")  # > 129 MB L2

    # plain engine (the reference's method and schedule)
    plain = open_engine(torch, prm, pattern, stream)
    rp = measure(args, torch, world, plain, d_frames, flows, stream, flush)

    # learned-seeded engine: schedule chosen on calibration sequences, then measured
    learned = None
    head, head_eng, head_name = rp, plain, "plain"
    net = None
    if not args.no_learned and os.path.exists(learn.DEFAULT_WEIGHTS):
        net = learn.load_net(learn.DEFAULT_WEIGHTS, 1, H // 4, W // 4)
        if args.schedule:
            sch = tuple(int(x) for x in args.schedule.split("/"))
            sch, table = (sch + (0, 1)[len(sch) - 2:])[:4], "given on the command line"
        else:
            sch, table = choose_schedule(torch, prm, pattern, net, stream)
        # the network's forward on both tensor-core paths (tcgen05 is the engine's)
        nf = {}
        default_mode = net.umma
        for path, mode in (("mma_sync", 0), ("tcgen05_fused", 2), ("tcgen05_per_layer", 1)):
            net.set_umma(mode)
            nf[path] = net_forward_timing(torch, net, d_frames, stream, reduce=sch[3] if sch else 1)
        net.set_umma(default_mode)  # the engines below run the network's default path
        net.check(stream.cuda_stream)
        nf["tcgen05_fused"]["ctas"] = net.fused_ctas
        nf["engine_path"] = {2: "tcgen05_fused", 1: "tcgen05_per_layer", 0: "mma_sync"}[net.umma]
        learned = {"weights": os.path.relpath(learn.DEFAULT_WEIGHTS, ROOT), "confidence": PROPOSAL_CONF,
                   "calibration": table, "schedule": None, "net_forward": nf}
        if sch is not None:
            seng = open_engine(torch, prm, pattern, stream, net, sch)
            rl = measure(args, torch, world, seng, d_frames, flows, stream, flush)
            learned.update({"schedule": {"iterations": sch[0], "jfMax": sch[1], "local_steps": sch[2], "reduce": sch[3]},
                            "value": rl["value"],
                            "ms_per_step": rl["ms_per_step"], "epe_mean": float(np.mean(rl["epe"])),
                            "speedup_vs_plain": rp["ms_per_step"] / rl["ms_per_step"],
                            "gpu_launches": int(rl["launches"])})
            if np.mean(rl["epe"]) <= np.mean(rp["epe"]):
                head, head_eng, head_name = rl, seng, "learned-seeded"
            else:
                seng.clean()

    e2e = measure_e2e(args, torch, world, head_eng, frames, head["u"], head["v"], flush)

    # roofline of the headline engine's dominant kernel (by total device time in the timed region)
    kstats = head["kstats"]
    total_k = sum(t for _, t in kstats.values())
    ranked = sorted(kstats.items(), key=lambda kv: -kv[1][1])
    dom, (n_launch, dom_ms) = ranked[0]
    roofline = roofline_entry(torch, dom, n_launch, dom_ms, total_k, prm, head["clocks"])
    roofline["timed_region"] = ("second run of the K timed steps with a CUDA event pair around every launch, frames "
                                "not pipelined so that no other kernel shares a launch's time (%.3f ms per step "
                                "there vs %.3f in the pipelined timed run)"
                                % (head["ms_per_step_profiled"], head["ms_per_step"]))
    # the other large kernels' rooflines beside the dominant one
    roofline["others"] = [roofline_entry(torch, k, c, t, total_k, prm, head["clocks"]) for k, (c, t) in ranked[1:4]]
    def kernel_table(stats):
        """Per kernel: launches and device ms over the K profiled steps, share of the
        kernel time, and ms per pair (the stage costs of the engine)."""
        tot = sum(t for _, t in stats.values())
        return {k: {"launches": c, "ms": round(t, 4), "share": round(t / tot, 4),
                    "ms_per_pair": round(t / (args.steps * PAIRS), 5)}
                for k, (c, t) in sorted(stats.items(), key=lambda kv: -kv[1][1])}

    kernels = kernel_table(kstats)
    kernels_plain = kernel_table(rp["kstats"]) if head_name != "plain" else None

    batched = None
    if batch_inputs is not None:
        batched = run_batched(args, torch, *batch_inputs, net=net)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(prm, pattern, frames, args.cpu_pairs)

    sched = learned["schedule"] if head_name != "plain" else {"iterations": prm.iterations, "jfMax": prm.jfMax}
    # the reference's own kernels (compiled from its sources) over the same step on this GPU
    ref_cuda = None
    if rank == 0 and world == 1:
        try:
            ref_cuda = reference_cuda(torch, prm.as_dict(), pattern, prm.gauss_taps(), frames, args)
        except Exception as e:  # the reference kernel build is optional
            ref_cuda = {"unavailable": str(e)[:200]}
    vs_ref = None
    if ref_cuda and ref_cuda.get("value"):
        rv = ref_cuda["value"]
        vs_ref = {"headline": head["value"] / rv, "plain": rp["value"] / rv, "e2e": e2e["value"] / rv,
                  "reference_mpx_s": rv}
        if learned and learned.get("value"):
            vs_ref["learned"] = learned["value"] / rv
    # long strings (autotune reports) go to stderr so the line's head stays short
    if batched:
        for key, rep in (("batched", batched.get("autotune")),
                         ("batched learned", (batched.get("learned") or {}).get("autotune"))):
            if rep:
                print("autotune %s: %s" % (key, rep), file=sys.stderr, flush=True)
        batched.pop("autotune", None)
        if batched.get("learned"):
            batched["learned"].pop("autotune", None)
    line = {
        "metric": METRIC, "value": head["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32 descriptors / int16 field / f32 flow",
        "data": "synthetic (seeded generator; see bench.py)",
        "config": bench_config(world),
        "engine": {"name": head_name, "iterations": sched["iterations"], "jfMax": sched["jfMax"],
                   "local_steps": sched.get("local_steps", 0), "proposal_reduce": sched.get("reduce"),
                   "grid": [prm.sx, prm.sy], "fsize": prm.fsize,
                   "pipelined": PIPELINED},
        "plain": {"value": rp["value"], "ms_per_step": rp["ms_per_step"], "epe_mean": float(np.mean(rp["epe"])),
                  "gpu_launches": int(rp["launches"]), "iterations": prm.iterations, "jfMax": prm.jfMax},
        "learned_vs_plain": (learned["speedup_vs_plain"] if learned and learned.get("value") else None),
        "batched_learned_vs_plain_batch": ((batched.get("learned") or {}).get("speedup_vs_plain_batch")
                                           if batched else None),
        "vs_reference_cuda_build": vs_ref,
        "e2e": e2e,
        "gpu_launches": int(head["launches"]),
        "clocks": head["clocks"],
        "roofline": roofline,
        "cpu_baseline": cpu,
        "epe": {"mean": float(np.mean(head["epe"])), "per_pair": [round(e, 4) for e in head["epe"]],
                "plain_mean": float(np.mean(rp["epe"]))},
        "reference_cuda_build": ref_cuda,
        "learned": learned,
        "kernels": kernels,
        "kernels_plain": kernels_plain,
        "batched": batched,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    plain.clean()
    if head_eng is not plain:
        head_eng.clean()
    if net is not None:
        net.close()


BATCH_SEED = 20261204


def _make_batch_pair(args):
    seed, w, h = args
    f0, f1, u, v = synth_module().make_pair(seed, w, h, vmax=15.0)
    return f0, f1, u, v


def make_batch_workload(pairs, seed=None):
    """Pairs of uneven size (widths U[320,1920], heights U[240,1080], multiples of 4)
    drawn from `seed` (default: the batched workload's), generated in a
    spawn-started process pool."""
    import multiprocessing as mp

    seed = BATCH_SEED if seed is None else seed
    sizes = synth_module().make_batch_sizes(seed, count=pairs)
    jobs = [(seed + k, w, h) for k, (w, h) in enumerate(sizes)]
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
        data = pool.map(_make_batch_pair, jobs)
    return sizes, data


# seeded batch schedules: (input reduction of the network, iterations, jfMax, local
# steps).  Fresh pairs start from the zero field, and the network's motions on frames
# much larger than its 512x384 training frames exceed what it saw: reduction 2
# (cells of 8 pixels) brings them back into its range
BATCH_CANDIDATES = ((1, 2, 64, 0), (1, 2, 64, 2), (1, 1, 128, 2), (2, 2, 64, 0), (2, 1, 128, 0), (2, 1, 64, 0),
                    (2, 1, 32, 0), (2, 1, 16, 0), (2, 1, 64, 2), (2, 1, 32, 2), (2, 1, 16, 2))


def batch_step_ms_epe(torch, b, data, stream, reps):
    """Device ms per step and mean EPE of a loaded, scheduled batch."""
    import numpy as np

    b.run()
    b.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        b.run()
    e1.record(stream)
    b.synchronize()
    flows = b.read_flows()
    epe = float(np.mean([np.mean(np.hypot(f[0] - d[2], f[1] - d[3])) for f, d in zip(flows, data)]))
    return e0.elapsed_time(e1) / reps, epe


def choose_batch_schedule(torch, net, stream, pairs=16):
    """The fastest seeded (reduction, iterations, jfMax, local steps) whose mean EPE on
    a separate calibration batch (other seeds of the same uneven-size generator) is at
    most the plain batch's there."""
    import briefmatch_gb300 as bm
    from briefmatch_gb300.proposal import ProposalNet

    sizes, data = make_batch_workload(pairs, seed=BATCH_SEED + 1000)
    params = [bm.BMParams.derive(w, h, UP, UP, N=NBITS) for w, h in sizes]
    b = bm.Batch(params)
    b.set_stream(stream.cuda_stream)
    b.load_frames(b.pack_frames([(d[0], d[1]) for d in data]))
    b.set_schedule(per_pair=1, use_graph=1, streams=2)
    plain_ms, plain_epe = batch_step_ms_epe(torch, b, data, stream, 2)
    table = [{"schedule": "plain", "ms": plain_ms, "epe": plain_epe}]
    bnet = ProposalNet(1, max(h for _, h in sizes) // 4, max(w for w, _ in sizes) // 4)
    bnet.set_params(net.params())
    best = None
    for sch in BATCH_CANDIDATES:
        b.set_proposal(bnet, PROPOSAL_CONF, sch[1], sch[2])
        b.set_proposal_reduce(sch[0])
        b.set_local_steps(sch[3], 2)
        b.set_schedule(per_pair=1, use_graph=1, streams=2)
        ms, epe = batch_step_ms_epe(torch, b, data, stream, 2)
        table.append({"schedule": "seeded x%d %d/%d/ls%d" % sch, "ms": ms, "epe": epe})
        if epe <= plain_epe and (best is None or ms < best[1]):
            best = (sch, ms)
    b.set_proposal(None)
    b.close()
    bnet.close()
    return (best[0] if best else None), table


def run_batched(args, torch, sizes, data, net=None, schedule=None):
    """The batched workload: all pairs through one autotuned batch step (persistent
    matching launch and/or per-level launches, replayed as a CUDA graph) against the
    same pairs run one after another through per-pair contexts (plain launches); with
    a proposal network, the same batch again with every pair seeded by it at the
    given (iterations, jfMax)."""
    import numpy as np

    import briefmatch_gb300 as bm

    params = [bm.BMParams.derive(w, h, UP, UP, N=NBITS) for w, h in sizes]
    out_px = sum(w * h for w, h in sizes)
    stream = torch.cuda.current_stream()
    b = bm.Batch(params)
    b.set_stream(stream.cuda_stream)
    packed = b.pack_frames([(d[0], d[1]) for d in data])
    d_packed = torch.from_numpy(packed).cuda()
    b.load_frames(d_packed.data_ptr(), on_device=True)
    report = b.autotune(None, reps=2)
    for _ in range(args.warmup):
        b.run()
    b.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    launches0 = b.launch_count()
    for s0, s1 in ev:
        s0.record(stream)
        b.run()
        s1.record(stream)
    b.synchronize()
    batch_ms = sum(s0.elapsed_time(s1) for s0, s1 in ev) / args.steps
    flows = b.read_flows()
    epe = float(np.mean([np.mean(np.hypot(f[0] - d[2], f[1] - d[3])) for f, d in zip(flows, data)]))
    sched = b.schedule()
    # the same pairs with almost no matching (one iteration, jump maximum 1: a single
    # level fused with the random search) on the plain batch's schedule: the cost of
    # every stage that a proposal cannot shorten, so batch_ms / floor_ms bounds the gain
    # of any seeded schedule on this workload
    fb = bm.Batch([bm.BMParams.derive(w, h, UP, UP, N=NBITS, iterations=1, jfMax=1) for w, h in sizes])
    fb.set_stream(stream.cuda_stream)
    fb.load_frames(d_packed.data_ptr(), on_device=True)
    fb.set_schedule(**sched)
    floor_ms, floor_epe = batch_step_ms_epe(torch, fb, data, stream, max(1, args.steps))
    fb.close()
    learned = None
    calibration = None
    if net is not None:
        schedule, calibration = choose_batch_schedule(torch, net, stream)
    if net is not None and schedule is not None:
        from briefmatch_gb300.proposal import ProposalNet

        bnet = ProposalNet(1, max(h for _, h in sizes) // 4, max(w for w, _ in sizes) // 4)
        bnet.set_params(net.params())
        b.set_proposal(bnet, PROPOSAL_CONF, schedule[1], schedule[2])
        b.set_proposal_reduce(schedule[0])
        b.set_local_steps(schedule[3], 2)
        lrep = b.autotune(None, reps=2)
        for _ in range(args.warmup):
            b.run()
        b.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        for s0, s1 in ev:
            s0.record(stream)
            b.run()
            s1.record(stream)
        b.synchronize()
        lms = sum(s0.elapsed_time(s1) for s0, s1 in ev) / args.steps
        lflows = b.read_flows()
        lepe = float(np.mean([np.mean(np.hypot(f[0] - d[2], f[1] - d[3])) for f, d in zip(lflows, data)]))
        learned = {"schedule": {"reduce": schedule[0], "iterations": schedule[1], "jfMax": schedule[2],
                                "local_steps": schedule[3]},
                   "value": out_px / (lms * 1e-3) / 1e6,
                   "ms_per_step": lms, "epe_mean": lepe, "speedup_vs_plain_batch": batch_ms / lms,
                   "autotune": lrep, "batch_schedule": b.schedule(), "calibration": calibration}
        b.set_proposal(None)
        bnet.close()
    b.close()
    del d_packed

    # the same pairs, one after another, each through its own plain context
    engines = []
    d_frames = []
    for p, d in zip(params, data):
        e = bm.BriefMatch(p)
        e.setup()
        e.set_stream(stream.cuda_stream)
        engines.append(e)
        d_frames.append((torch.from_numpy(d[0]).cuda(), torch.from_numpy(d[1]).cuda()))

    def seq_step():
        for e, (f0, f1) in zip(engines, d_frames):
            e.reset_sequence()
            e.set_rng_position(0)
            e.frame(f0.data_ptr(), True)
            e.frame(f1.data_ptr(), True)

    for _ in range(args.warmup):
        seq_step()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for s0, s1 in ev:
        s0.record(stream)
        seq_step()
        s1.record(stream)
    torch.cuda.synchronize()
    seq_ms = sum(s0.elapsed_time(s1) for s0, s1 in ev) / args.steps
    for e in engines:
        e.clean()
    return {
        "workload": "%d pairs, widths U[320,1920] x heights U[240,1080] (multiples of 4), u2.9, N128, one pair "
                    "(2 frames) each" % len(sizes),
        "output_mpx_per_step": out_px / 1e6,
        "value": out_px / (batch_ms * 1e-3) / 1e6, "unit": UNIT, "ms_per_step": batch_ms,
        "sequential_value": out_px / (seq_ms * 1e-3) / 1e6, "sequential_ms_per_step": seq_ms,
        "speedup_vs_sequential": seq_ms / batch_ms,
        "schedule": sched, "autotune": report, "epe_mean": epe,
        "matching_floor": {"what": "1 iteration, jump maximum 1, no proposal, plain schedule", "ms_per_step": floor_ms,
                           "epe_mean": floor_epe, "ceiling_vs_plain_batch": batch_ms / floor_ms},
        "learned": dict(learned, speedup_vs_plain_sequential=seq_ms / learned["ms_per_step"]) if learned else
        ({"schedule": None, "calibration": calibration} if calibration else None),
    }


def cpu_baseline(prm, pattern, frames, pairs):
    """The oracle over `pairs` pairs of the workload on all host threads."""
    import numpy as np

    import oracle

    nt = oracle.num_threads()
    p = prm.as_dict()
    n = prm.sx * prm.sy
    seq = oracle.Sequence(p, pattern, lambda call, cnt: oracle.normals(1000 + call, 2 * cnt))
    seq.frame(frames[0])
    t0 = time.perf_counter()
    for k in range(1, pairs + 1):
        seq.frame(frames[k])
    dt = time.perf_counter() - t0
    return {"value": pairs * W * H / dt / 1e6, "unit": UNIT, "cores": nt, "kind": "port",
            "sample": "%d consecutive pair(s) of the 1024x436 sequence (after priming frame 0), %.1f s" % (pairs, dt)}


def run_reference(args, torch, world, rank):
    """The reference's own implementation of the path, timed on the host cores: the
    reference has no CPU path of its own, so this is the oracle's transcription of its
    kernels (all host threads), one pair of the workload per step.  Parameters and the
    pattern come from the oracle's restatement of the reference's derivation, so this
    arm loads no engine code.  Only rank 0 works."""
    if rank != 0:
        return
    import oracle

    frames, flows = make_workload(rank)
    p = oracle.derive_params(W, H, UP, UP, N=NBITS)
    pattern = oracle.make_pattern(p, SEED)
    nt = oracle.num_threads()
    seq = oracle.Sequence(p, pattern, lambda call, cnt: oracle.normals(1000 + call, 2 * cnt))
    k = 0
    seq.frame(frames[0])

    def one_pair():
        nonlocal k
        k += 1
        if k >= FRAMES:
            seq.__init__(p, pattern, seq.normals_fn)
            seq.frame(frames[0])
            k = 1
        t0 = time.perf_counter()
        seq.frame(frames[k])
        return time.perf_counter() - t0

    for _ in range(args.warmup):
        one_pair()
    times = [one_pair() for _ in range(args.steps)]
    tot = sum(times)
    value = args.steps * W * H / tot / 1e6
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": tot / args.steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "impl": "reference", "dtype": "u32 descriptors / int16 field / f32 flow",
        "data": "synthetic (seeded generator; see bench.py)",
        "config": bench_config(world),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nt, "kind": "port",
                         "sample": "one pair of the %dx%d sequence per step (bounded sample of the %d-pair step), "
                                   "%d threads" % (W, H, PAIRS, nt)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    try:
        line["reference_cuda_build"] = reference_cuda(torch, p, pattern, oracle.gauss_taps(p["sigma"]), frames, args)
    except Exception as e:  # the reference kernel build is optional
        line["reference_cuda_build"] = {"unavailable": str(e)[:200]}
    print(json.dumps(line), flush=True)


def reference_cuda(torch, params, pattern, taps, frames, args):
    """The reference's kernels (compiled from its sources) over the full step on the GPU:
    `params` a parameter dict, `taps` the Gaussian down-sampling taps."""
    import numpy as np

    from oracle import refshim

    if not torch.cuda.is_available():
        return {"unavailable": "no GPU"}
    if not refshim.available():
        return {"unavailable": "reference kernel build (oracle/_ref) not present"}
    # the shim launches on the legacy default stream: record the timing events there
    with torch.cuda.stream(torch.cuda.default_stream()):
        return _reference_cuda_timed(torch, refshim.RefPipeline(torch, params, pattern, taps), frames, args)


def _reference_cuda_timed(torch, pipe, frames, args):
    import numpy as np

    d_frames = [torch.from_numpy(f.astype(np.float32)).cuda() for f in frames]
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    def step():
        pipe.primed = False
        pipe.first = True
        for f in d_frames:
            pipe.frame(f)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    tot = 0.0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record()
        step()
        e.record()
        torch.cuda.synchronize()
        tot += s.elapsed_time(e)
    ms = tot / args.steps
    return {"value": PAIRS * W * H / (ms * 1e-3) / 1e6, "unit": UNIT, "ms_per_step": ms,
            "how": "reference kernels/briefmatch_cuda.cu + util_cuda.cu compiled unmodified (-O3 -use_fast_math, "
                   "sm_103a), launched with the reference's 32x32 blocks and a device sync after every launch"}


def main():
    args = parse()
    set_config(args.config)
    global PIPELINED
    PIPELINED = not args.no_pipelined
    if args.config != "2":
        args.no_learned = args.no_batched = args.no_cpu_baseline = True
    import torch

    world, rank = dist_init(torch)
    if args.impl == "reference":
        run_reference(args, torch, world, rank)
    else:
        run_engine(args, torch, world, rank)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
