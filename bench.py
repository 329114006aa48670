"""Benchmark of the GB300 draw path (one JSON line on rank 0).

Workload (one step = one frame, the DrawModel::draw sequence: 2048^2 shadow pass, then the
main pass): displaced icosphere subdivision 7 (327,680 triangles) + a 2-triangle ground
plane submitted after it, 1024^2 RGBA8 diffuse + 1024^2 tangent-space normal map,
1920x1080 FP32 depth + RGBA8 colour + prim ids, NormalMap + shadow shader; both clears
are part of the frame.  Inputs are seeded synthetic data of those sizes.

value     frames/s with inputs resident in HBM: K frames, device time from CUDA events on
          the library's stream around each frame, L2 flushed (512 MB write) between frames.
e2e       frames/s through the public C ABI with host buffers: uniforms go host -> device
          inside every frame and the frame's colour + depth come back into page-locked host
          memory; wall-clock time.
roofline  the kernel with the largest share of the frame: algorithmic bytes per launch /
          its CUDA-event duration, against the measured HBM copy bandwidth.
cpu_baseline  the oracle (C restatement of the reference) on the host cores, bounded sample.

--impl reference times the reference's CPU implementation of the path (the oracle port
on a GPU host: the reference's Win32 sources do not build there) with every host thread.

Multi-GPU (torchrun): each rank renders its own frames (replicas, no collective on the
data path); value = all frames / slowest rank's time.
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
sys.path.insert(0, os.path.join(ROOT, "hana-softwarerenderer_gb300"))

METRIC = "frames/s + p50/p99 latency, batched serve vs plain per-frame; bit-exact depth"
WORKLOAD = ("displaced icosphere-7 (327,680 tris) + 2-tri ground plane, 1920x1080, 2048^2 shadow map, "
            "NormalMap + shadow, 1024^2 diffuse + normal map")


def peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self._t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "power_w_max": max(power),
                "samples": len(sm), "reasons": sorted(reasons)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
    return world, rank, local


def dist_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_barrier(world: int):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def kernel_bytes(t: dict) -> dict:
    """Algorithmic bytes per launch of each kernel of one frame (both passes).

    vertex : 12 B read + 16 B clip written per position, +16 B world position where the
             shader reads it; 12 B read + 16 B written per normal.
    setup  : 16 B index read + 16 B clip read per face corner set (each vertex once) + a
             64 B record written per triangle that reaches the raster.
    scan   : 4 B read + 4 B written per tile.
    scatter: 16 B of each record read + 4 B written per (triangle, tile) pair.
    raster : 12 B written per pixel (colour, depth, prim id; the clear is fused), 4 B read
             per (triangle, tile) pair + the 64 B record, and per shaded pixel the texels it
             samples (diffuse, normal map, shadow map: 4 B each) — vertex attributes of the
             visible triangles are counted once per record (3 corners x 56 B).
    """
    px, rec, pairs = t["pixels"], t["records"], t["bin_pairs"]
    tiles = px / 64.0  # tiles of the scan, counted as 8x8 (the 16x16 grid has fewer)
    return {
        "vertex": t["vertices"] * 28 + t["vertices"] * 8 + t["normals"] * 28,
        "setup": t["faces"] * 16 + t["vertices"] * 16 + rec * 64,
        "scan": tiles * 8,
        "scatter": rec * 16 + pairs * 4,
        "raster": px * 12 + pairs * 4 + rec * (64 + 3 * 56) + t["shaded_pixels"] * 12,
    }


def ncu_traffic(kernel: str):
    """DRAM bytes per launch of `kernel` from the committed ncu capture of this workload."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        return json.load(f)["dram_bytes_per_launch"].get(kernel)


def run_ours(args, world, rank, local):
    import torch

    import hsr
    from hsr import frame as hframe
    from hsr import scenes

    torch.cuda.set_device(local)
    hsr.init(local)
    t0 = time.time()
    fr = scenes.displaced_frame()
    gen_s = time.time() - t0
    g = hframe.GpuFrame(fr)
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")

    tuned = None
    if args.tile:
        hsr.set_tuning(tile=args.tile, warps_per_cta=4 if args.tile == 16 else 8)
    elif not args.no_autotune:
        tuned = hsr.autotune(g.descs, reps=3)  # outside the timed region
    hsr.set_profiling(True)
    for _ in range(args.warmup):
        g.render()
    # ---- timed region (device) ----------------------------------------------------------
    sampler = ClockSampler(local)
    dist_barrier(world)
    torch.cuda.synchronize()
    sampler.start()
    frame_ms, kernel_ms, timings = [], {k: [] for k in hsr.KERNELS}, None
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        g.render()
        timings = hsr.last_timing()
        frame_ms.append(timings["batch_ms"])
        for k, v in timings["kernel_ms"].items():
            kernel_ms[k].append(v)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    dist_barrier(world)
    total_s = sum(frame_ms) / 1000.0
    total_s_max = dist_max(total_s, world)
    value = world * args.steps / total_s_max

    # ---- plain per-frame path: one hsr_draw per pass (two synchronous calls) ------------
    plain_ms = []
    for _ in range(max(3, args.steps // 2)):
        flush.zero_()
        torch.cuda.synchronize()
        s0 = time.perf_counter()
        g.render(batched=False)
        plain_ms.append((time.perf_counter() - s0) * 1000.0)

    # ---- end to end through the C ABI with host buffers ---------------------------------
    hsr.set_profiling(False)
    pc = hsr.PinnedArray((fr.height, fr.width, 4), np.uint8)
    pd = hsr.PinnedArray((fr.height, fr.width), np.float32)
    e2e_ms = []
    for i in range(args.warmup + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        s0 = time.perf_counter()
        g.render()
        g.main.download(color=True, depth=True, prim=False, out={"color": pc.array, "depth": pd.array})
        if i >= args.warmup:
            e2e_ms.append((time.perf_counter() - s0) * 1000.0)
    e2e_t = hsr.last_timing()
    h2d = int(e2e_t["h2d_bytes"])
    d2h = int(pc.array.nbytes + pd.array.nbytes + e2e_t["d2h_bytes"])
    e2e_s = dist_max(sum(e2e_ms) / 1000.0, world)
    pc.release()
    pd.release()

    # ---- roofline of the dominant kernel ------------------------------------------------
    mean_k = {k: statistics.mean(v) for k, v in kernel_ms.items()}
    top = max(mean_k, key=mean_k.get)
    kb = kernel_bytes(timings)
    pk = peaks()
    achieved = kb[top] / (mean_k[top] * 1e-3) / 1e9
    roof = {"kernel": top, "bound": "hbm", "achieved": round(achieved, 1), "peak": pk["hbm_gbs"],
            "peak_source": pk["source"], "unit": "GB/s", "frac": round(achieved / pk["hbm_gbs"], 4),
            "algorithmic_bytes": int(kb[top]), "ms": round(mean_k[top], 5),
            "traffic": args.traffic_bytes if args.traffic_bytes else ncu_traffic(top),
            "share": {k: round(v / sum(mean_k.values()), 4) for k, v in mean_k.items()}}

    out = {
        "metric": METRIC, "value": round(value, 2), "unit": "frames/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(statistics.mean(frame_ms), 5),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "frames_per_step": 1, "l2": "flushed (512 MB write) between timed frames",
                   "tuning": {k: getattr(hsr.get_tuning(), k) for k in ("tile", "warps_per_cta", "ctas_per_sm",
                                                                      "bin_factor")},
                   "autotuned": tuned is not None, "parallelism": f"replicas x{world}"},
        "latency_ms": {"p50": round(float(np.percentile(frame_ms, 50)), 5),
                       "p99": round(float(np.percentile(frame_ms, 99)), 5)},
        "plain_per_frame": {"ms_p50": round(float(np.percentile(plain_ms, 50)), 4),
                            "frames_per_s": round(1000.0 / statistics.mean(plain_ms), 2),
                            "note": "two synchronous hsr_draw calls per frame, wall clock"},
        "e2e": {"value": round(world * args.steps / e2e_s, 2), "unit": "frames/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "p50_ms": round(float(np.percentile(e2e_ms, 50)), 4)},
        "roofline": roof,
        "kernel_ms": {k: round(v, 5) for k, v in mean_k.items()},
        "counts": {k: int(timings[k]) for k in ("faces", "vertices", "records", "bin_pairs", "pixels",
                                                  "shaded_pixels", "clipped_faces")},
        "gpu_launches": int(timings["launches"]) * args.steps,
        "clocks": clocks,
    }
    g.release()
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(fr, args.cpu_seconds)
    out["gen_s"] = round(gen_s, 2)
    return out


def cpu_baseline(fr, seconds: float, threads: int | None = None) -> dict:
    """The oracle (C restatement, 1 frame per thread per round) on this host's cores."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    threads = threads or os.cpu_count() or 1
    one = oracle.bench_frames(fr, 1, 1)
    rounds = max(1, int(round(seconds / max(one, 1e-3))))
    s = oracle.bench_frames(fr, rounds, threads)
    frames = rounds * threads
    return {"value": round(frames / s, 4), "unit": "frames/s", "cores": threads, "kind": "port",
            "sample": f"{frames} frames of the benchmark workload ({rounds} per thread), {s:.1f} s wall; "
                      f"1 frame on 1 core = {one * 1000:.0f} ms"}


def run_reference(args, world, rank):
    """The reference's CPU implementation of the path with every host thread."""
    if rank != 0:
        return None
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from hsr import scenes

    fr = scenes.displaced_frame()
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        oracle.bench_frames(fr, 1, threads)
    secs = [oracle.bench_frames(fr, 1, threads) for _ in range(args.steps)]
    value = args.steps * threads / sum(secs)
    per = [s * 1000.0 for s in secs]
    return {
        "metric": METRIC, "value": round(value, 4), "unit": "frames/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(statistics.mean(per), 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
        "config": {"workload": WORKLOAD, "frames_per_step": threads, "l2": "n/a (host)"},
        "cpu_baseline": {"value": round(value, 4), "unit": "frames/s", "cores": threads, "kind": "port",
                         "sample": f"{threads} frames per step ({threads} threads x 1 frame), {args.steps} steps"},
        "e2e": {"value": round(value, 4), "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--tile", type=int, default=0, help="fix the raster tile (8 or 16) instead of autotuning")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--traffic-bytes", type=float, default=0.0,
                    help="DRAM bytes of the dominant kernel per launch from an ncu capture")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world, rank, local = dist_setup()
    if args.impl == "reference":
        out = run_reference(args, world, rank)
    else:
        out = run_ours(args, world, rank, local)
    if rank == 0 and out is not None:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
