"""Benchmark of the GB300 draw path (one JSON line on rank 0).

Headline workload — serving mixed render requests (each request is one DrawModel::draw,
scene.h:53-99: an optional shadow pass, then the main pass):
  16 resident meshes, 8,241,152 triangles in all (3x displaced icosphere-8, 6x icosphere-7,
  4x 512^2 height-field grid, 3x icosphere-6), 4 texture pairs of 1024^2 (RGBA8 diffuse +
  RGB8 tangent normal map); requests with mesh uniform over the pool, width / height
  log-uniform over 128-3840 / 128-2160, shader uniform over ground / toon / texture /
  texture-with-light / blinn / normal-map, a shadow pass on half of them (square map, next
  power of two of the larger side, 256-2048); the colour of each request is read back.
  Seeded synthetic data of those sizes (no public dataset is involved).

value     frames/s of the batched path with meshes and textures resident in HBM: each step
          renders 64 requests of the stream as one launch sequence (the batch the server
          forms); device time from CUDA events on the library's stream; L2 flushed (512 MB
          write) before every step.
e2e       frames/s through the public serving API (hsr_server_*) with host buffers: the
          same requests submitted at once, uniforms host -> device and every colour
          device -> page-locked host inside the timed region; wall clock.
plain_per_frame   the same requests one at a time through the per-frame drop-in path
          (targets created, both passes drawn, colour read back, targets released).
serve     10,000 Poisson arrivals at two offered loads (80% of the plain path's capacity and
          80% of the server's): frames/s and p50 / p99 latency from scheduled arrival, for
          the server and for the plain path.
roofline  every kernel of the batched step: algorithmic bytes per launch / its CUDA-event
          duration, against the measured HBM copy bandwidth; the headline is the kernel with
          the largest share.
frame_1080p / batched_views_64   the single 1080p frame and the 64-view batched launch.
cpu_baseline  the oracle (C restatement of the reference) on this host's cores, bounded
          sample of the same request stream.

--impl reference times the reference's CPU implementation of the path (the oracle port
on a GPU host: the reference's Win32 sources do not build there) with every host thread.

Multi-GPU (torchrun): each rank serves its own requests (replicas, no collective on the data
path); value = all frames / slowest rank's time.  The sub-results run on world size 1 only.
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
SERVE_WORKLOAD = ("serving: 16 resident meshes (8,241,152 tris), 1024^2 diffuse + normal maps; requests with "
                  "log-uniform 128-3840 x 128-2160 targets, 6 shaders, shadow pass on 50%, colour read back")
FRAME_WORKLOAD = ("displaced icosphere-7 (327,680 tris) + 2-tri ground plane, 1920x1080, 2048^2 shadow map, "
                  "NormalMap + shadow, 1024^2 diffuse + normal map")
SOUP_WORKLOAD = ("triangle soup, 4,000,000 tris at 3840x2160, centroids uniform, lognormal edges (median 2 px), "
                 "constant NDC depth U[0,1] (~8x depth complexity), 1% exact duplicates submitted later, flat shader")
BATCH = 64          # requests per launch sequence (the server's max_batch)
COUNT_KEYS = ("faces", "vertices", "normals", "records", "bin_pairs", "pixels", "shaded_pixels", "clipped_faces",
              "raster_pixels", "fragments", "tiles", "split_triangles", "payload_bytes")
N_REQUESTS = 10000  # Poisson stream length
SEED = 5


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
    """Algorithmic bytes per launch of each kernel of one launch sequence (the floor a kernel
    must move to or from HBM; intermediate results the design keeps in L2 still count).

    vertex : 12 B position read + 16 B screen vertex written per position.
    cull   : 16 B face indices per face + 16 B screen vertex per position (each gathered
             once) + a 64 B record written per triangle that reaches the raster.
    emit   : per surviving triangle 32 B of its record and 16 B face indices read, a 4 B
             payload index written, and the shading payload written (payload_bytes, counted
             by the kernels: 0-128 B by shader); the packed position, normal and uv (one
             32 B sector) of each vertex of a surviving triangle read once, records / 2
             vertices (a closed triangle mesh has half as many vertices as faces).
    clip   : per clipped face 48 B of indices and 3 x 56 B of corner attributes.
    split  : per split triangle its 192 B queue entry read.
    scan   : 4 B read + 12 B written per tile (offset, non-empty prefix, list entry).
    scatter: 16 B of each record read + 4 B written per (triangle, tile) pair, and the fused
             clear of the tiles without triangles: 12 B written per pixel (colour, depth,
             prim id) outside the raster's tiles.
    raster : 12 B written per pixel of the tiles it visits, 4 B read per (triangle, tile)
             pair, the 64 B record and the shading payload of each triangle, and one 4 B
             texel per shaded pixel (the diffuse map; normal and shadow maps not counted).
    """
    px, rec, pairs = t["pixels"], t["records"], t["bin_pairs"]
    rpx = t.get("raster_pixels", px)
    pay = t.get("payload_bytes", rec * 128)
    return {
        "vertex": t["vertices"] * 28 + t["normals"] * 28,
        "cull": t["faces"] * 16 + t["vertices"] * 16 + rec * 64,
        "emit": rec * 52 + pay + (rec // 2) * 32,
        "clip": t["clipped_faces"] * (48 + 3 * 56),
        "split": t.get("split_triangles", 0) * 192,
        "scan": t.get("tiles", px / 64.0) * 16,
        "scatter": rec * 16 + pairs * 4 + (px - rpx) * 12,
        "raster": rpx * 12 + pairs * 4 + rec * 64 + pay + t["shaded_pixels"] * 4,
    }


def _ncu_record(workload: str) -> dict:
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if not os.path.exists(p):
        return {}
    with open(p) as f:
        return json.load(f).get("workloads", {}).get(workload, {})


def ncu_traffic(workload: str, kernel: str):
    """DRAM bytes per launch of `kernel` from the committed ncu capture of `workload`."""
    return _ncu_record(workload).get("dram_bytes_per_launch", {}).get(kernel)


def ncu_utilisation(workload: str, kernel: str):
    """Issue-active and pipe utilisation of `kernel` from the committed ncu capture (or None)."""
    return _ncu_record(workload).get("utilisation", {}).get(kernel)


def roofline(kernel_ms: dict, counts: dict, workload: str) -> dict:
    """The kernel with the largest share of the launch sequence, against the measured HBM
    copy bandwidth, and every kernel's own figures beside it."""
    mean_k = {k: statistics.mean(v) for k, v in kernel_ms.items()}
    kb = kernel_bytes(counts)
    pk = peaks()
    total = sum(mean_k.values())
    per = {}
    for k, ms in mean_k.items():
        gbs = kb[k] / (ms * 1e-3) / 1e9 if ms > 0 else 0.0
        per[k] = {"ms": round(ms, 5), "share": round(ms / total, 4) if total else 0.0,
                  "algorithmic_bytes": int(kb[k]), "achieved_gbs": round(gbs, 1),
                  "frac": round(gbs / pk["hbm_gbs"], 4), "traffic": ncu_traffic(workload, k)}
        u = ncu_utilisation(workload, k)
        if u:
            per[k]["ncu"] = u
    top = max(mean_k, key=mean_k.get)
    return {"kernel": top, "bound": "hbm", "achieved": per[top]["achieved_gbs"], "peak": pk["hbm_gbs"],
            "peak_source": pk["source"], "unit": "GB/s", "frac": per[top]["frac"],
            "algorithmic_bytes": per[top]["algorithmic_bytes"], "ms": per[top]["ms"], "traffic": per[top]["traffic"],
            "issue": per[top].get("ncu"),
            "kernels": per,
            "note": "the kernel with the largest share of the step; every kernel's share, algorithmic bytes and "
                    "fraction of the measured copy bandwidth under 'kernels'; the raster and the cull pass are "
                    "issue-bound: 'issue' / kernels[*].ncu give issue-active and FP32 (fma) / ALU pipe utilisation "
                    "from the committed ncu capture (profiles/kernels_serve_small.md)"}


def serve_inputs(n: int):
    from hsr import scenes

    pool = scenes.mesh_pool(scenes.SERVE_POOL_SPEC, seed=1)
    tex = scenes.pool_textures(4, 1024, seed=17)
    reqs = scenes.request_stream(pool, n, rate_per_s=1000.0, seed=SEED)
    return pool, tex, reqs


# ------------------------------------------------------------------------------------------
# batched steps of the serving workload (value) + server / plain path (e2e, serve)
# ------------------------------------------------------------------------------------------
def run_ours(args, world, rank, local):
    import torch

    import hsr
    from hsr import scenes
    from hsr import serve as hserve

    torch.cuda.set_device(local)
    hsr.init(local)
    t0 = time.time()
    pool, tex, reqs = serve_inputs(N_REQUESTS)
    rp = hserve.ResidentPool(pool, tex)
    gen_s = time.time() - t0
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")
    # each rank serves its own slice of the stream
    off = (rank * (args.warmup + args.steps) * BATCH) % len(reqs)
    chunks = [[reqs[(off + i * BATCH + j) % len(reqs)] for j in range(BATCH)]
              for i in range(args.warmup + args.steps)]

    tuned = None
    if args.tile:
        hsr.set_tuning(tile=args.tile, warps_per_cta=args.warps or (4 if args.tile == 16 else 8),
                       ctas_per_sm=args.ctas or None)
    elif not args.no_autotune:
        vb = hserve.ViewBatch(rp, chunks[0])
        tuned = hsr.autotune(vb.descs, reps=2)  # outside the timed region
        vb.release()
    hsr.set_profiling(True)
    retries0 = None

    # ---- value: one launch sequence of 64 requests per step ------------------------------
    step_ms, kernel_ms, launches, h2d, d2h = [], {k: [] for k in hsr.KERNELS}, 0, [], []
    counts_sum: dict = {}
    sampler = ClockSampler(local)
    for i, chunk in enumerate(chunks):
        timed = i >= args.warmup
        vb = hserve.ViewBatch(rp, chunk)  # targets from the pool (untimed)
        if timed and i == args.warmup:
            dist_barrier(world)
            torch.cuda.synchronize()
            sampler.start()
            retries0 = hsr.stats()["retries"]
        flush.zero_()
        torch.cuda.synchronize()
        vb.draw_all()
        t = hsr.last_timing()
        vb.release()
        if not timed:
            continue
        step_ms.append(t["batch_ms"])
        for k, v in t["kernel_ms"].items():
            kernel_ms[k].append(v)
        launches += int(t["launches"])
        h2d.append(int(t["h2d_bytes"]))
        d2h.append(sum(r.width * r.height * 4 for r in chunk) + int(t["d2h_bytes"]))
        for k in COUNT_KEYS:
            counts_sum[k] = counts_sum.get(k, 0) + int(t[k])
    torch.cuda.synchronize()
    clocks = sampler.stop()
    retries = hsr.stats()["retries"] - (retries0 or 0)  # scratch overflows re-run inside the timed steps
    dist_barrier(world)
    frames = args.steps * BATCH
    total_s = dist_max(sum(step_ms) / 1000.0, world)
    value = world * frames / total_s
    counts = {k: v / args.steps for k, v in counts_sum.items()}  # per step
    roof = roofline(kernel_ms, counts, "serve_batch64")
    hsr.set_profiling(False)

    # ---- e2e: the same requests through hsr_server (all submitted at once) ----------------
    timed_reqs = [r for c in chunks[args.warmup:] for r in c]
    sat = scenes.retime(timed_reqs, 1e9)
    # one long-running server: the warm-up requests pass through it first (its scratch and the
    # memory pool reach their working size there), then the timed ones
    srv = hsr.Server(40 << 30, BATCH, 2)
    ring = hserve.PinnedRing(1 << 30)
    try:
        hserve.serve_batched(rp, scenes.retime([r for c in chunks[:args.warmup] for r in c], 1e9), server=srv,
                             ring=ring)
        dist_barrier(world)
        e2e_run = hserve.serve_batched(rp, sat, server=srv, ring=ring)
    finally:
        srv.close()
        ring.release()
    e2e_s = dist_max(e2e_run["wall_s"], world)
    e2e = {"value": round(world * frames / e2e_s, 2), "unit": "frames/s",
           "h2d_bytes_per_step": int(statistics.mean(h2d)), "d2h_bytes_per_step": int(statistics.mean(d2h)),
           "p50_ms": round(float(np.percentile(e2e_run["latency_ms"], 50)), 3),
           "p99_ms": round(float(np.percentile(e2e_run["latency_ms"], 99)), 3),
           "batches": e2e_run["batches"], "ok": e2e_run["ok"],
           "note": "hsr_server, max_batch 64, 2 slots, warmed by the warm-up steps' requests; all timed "
                   "requests submitted at t=0; wall clock"}

    out = {
        "metric": METRIC, "value": round(value, 2), "unit": "frames/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(statistics.mean(step_ms), 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": SERVE_WORKLOAD, "frames_per_step": BATCH,
                   "l2": "flushed (512 MB write) before every step; a step also writes ~1 GB of targets",
                   "tuning": {k: getattr(hsr.get_tuning(), k) for k in ("tile", "warps_per_cta", "ctas_per_sm",
                                                                      "bin_factor")},
                   "autotuned": tuned is not None, "parallelism": f"replicas x{world}"},
        "e2e": e2e,
        "roofline": roof,
        "kernel_ms": {k: round(statistics.mean(v), 4) for k, v in kernel_ms.items()},
        "counts_per_step": {k: int(v) for k, v in counts.items()},
        "gpu_launches": launches,
        "scratch_retries": retries,
        "clocks": clocks,
    }

    if world == 1 and not args.quick:
        # ---- plain per-frame path on the same requests, then the Poisson streams ----------
        hserve.serve_plain(rp, scenes.retime(chunks[0], 1e9))
        plain_sat = hserve.serve_plain(rp, sat)
        plain_fps = frames / plain_sat["wall_s"]
        out["plain_per_frame"] = {
            "frames_per_s": round(plain_fps, 2),
            "p50_ms": round(float(np.percentile(plain_sat["latency_ms"], 50)), 3),
            "p99_ms": round(float(np.percentile(plain_sat["latency_ms"], 99)), 3),
            "batched_over_plain_e2e": round(e2e["value"] / plain_fps, 3),
            "batched_over_plain_device": round(value / plain_fps, 3),
            "note": "same requests, all at t=0, one at a time: hsr_target_create x2, hsr_draw_batch (shadow + "
                    "main), hsr_target_download (colour), hsr_target_release x2; wall clock"}
        out["serve"] = serve_poisson(rp, reqs, plain_fps, e2e["value"], args)
        at = out["serve"]["load_server80"]
        e2e["poisson_at_server_load"] = {
            "rate_per_s": at["rate_per_s"], "server_p50_ms": at["server"]["p50_ms"],
            "server_p99_ms": at["server"]["p99_ms"], "plain_p50_ms": at["plain"]["p50_ms"],
            "plain_p99_ms": at["plain"]["p99_ms"],
            "note": "10,000 Poisson arrivals at 80% of the server's measured capacity; latency from each "
                    "request's scheduled arrival to its colour on the host"}
        out["frame_1080p"] = run_frame(args)
        out["batched_views_64"] = run_views(args)
        out["depth_stress_4m"] = run_soup(args)
    rp.release()
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args.cpu_seconds)
    out["gen_s"] = round(gen_s, 2)
    return out


def serve_poisson(rp, reqs, plain_fps: float, server_fps: float, args) -> dict:
    """The 10,000-request Poisson stream at two offered loads, server vs plain path.  One
    long-running server serves both loads; it is warmed first with the whole stream at once
    (untimed), so that its scratch and staging have reached the working size of this stream's
    batches, as they would have in a server that has been running."""
    import hsr
    from hsr import scenes
    from hsr import serve as hserve

    res = {"requests": len(reqs), "arrivals": "Poisson", "server_warmup_requests": len(reqs)}
    srv = hsr.Server(40 << 30, BATCH, 2)
    ring = hserve.PinnedRing(1 << 30)
    try:
        hserve.serve_batched(rp, scenes.retime(reqs, 1e9), server=srv, ring=ring)
        for name, rate in (("load_plain80", 0.8 * plain_fps), ("load_server80", 0.8 * server_fps)):
            stream = scenes.retime(reqs, rate, seed=11)
            b = hserve.serve_batched(rp, stream, server=srv, ring=ring)
            p = hserve.serve_plain(rp, stream)
            sb = hserve.latency_summary(b, len(stream))
            sp = hserve.latency_summary(p, len(stream))
            res[name] = {"rate_per_s": round(rate, 1),
                         "server": {k: round(v, 3) for k, v in sb.items()} | {"mean_batch": round(b["mean_batch"], 2),
                                                                             "ok": b["ok"]},
                         "plain": {k: round(v, 3) for k, v in sp.items()}}
    finally:
        srv.close()
        ring.release()
    return res


def run_frame(args) -> dict:
    """The single 1080p frame with its 2048^2 shadow pass (device time + plain calls)."""
    import torch

    import hsr
    from hsr import frame as hframe
    from hsr import scenes

    fr = scenes.displaced_frame()
    g = hframe.GpuFrame(fr)
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    old = hsr.get_tuning()
    if not args.tile:
        hsr.autotune(g.descs, reps=3)
    hsr.set_profiling(True)
    for _ in range(3):
        g.render()
    ms, kms, t = [], {k: [] for k in hsr.KERNELS}, None
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        g.render()
        t = hsr.last_timing()
        ms.append(t["batch_ms"])
        for k, v in t["kernel_ms"].items():
            kms[k].append(v)
    plain = []
    for _ in range(max(3, args.steps // 2)):
        flush.zero_()
        torch.cuda.synchronize()
        s0 = time.perf_counter()
        g.render(batched=False)
        plain.append((time.perf_counter() - s0) * 1000.0)
    hsr.set_profiling(False)
    counts = {k: int(t[k]) for k in COUNT_KEYS}
    res = {"workload": FRAME_WORKLOAD, "frames_per_s": round(1000.0 / statistics.mean(ms), 2),
           "ms_p50": round(float(np.percentile(ms, 50)), 4), "ms_p99": round(float(np.percentile(ms, 99)), 4),
           "plain_two_draw_calls_frames_per_s": round(1000.0 / statistics.mean(plain), 2),
           "kernel_ms": {k: round(statistics.mean(v), 4) for k, v in kms.items()},
           "roofline": roofline(kms, counts, "frame_1080p"), "counts": counts,
           "tuning": {k: getattr(hsr.get_tuning(), k) for k in ("tile", "warps_per_cta", "ctas_per_sm")}}
    g.release()
    hsr.set_tuning(tile=old.tile, warps_per_cta=old.warps_per_cta, ctas_per_sm=old.ctas_per_sm)
    return res


def run_soup(args) -> dict:
    """The depth-order stress frame: 4M-triangle soup at 3840x2160 (lognormal edges, median
    2 px, ~8x depth complexity, 1% equal-depth duplicates), flat shader; device time."""
    import torch

    import hsr
    from hsr import frame as hframe
    from hsr import scenes

    fr = scenes.soup_frame()
    g = hframe.GpuFrame(fr)
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    old = hsr.get_tuning()
    tuned = hsr.autotune(g.descs, reps=2) if not args.tile else None
    hsr.set_profiling(True)
    for _ in range(3):
        g.render()
    ms, kms, t = [], {k: [] for k in hsr.KERNELS}, None
    for _ in range(max(5, args.steps // 3)):
        flush.zero_()
        torch.cuda.synchronize()
        g.render()
        t = hsr.last_timing()
        ms.append(t["batch_ms"])
        for k, v in t["kernel_ms"].items():
            kms[k].append(v)
    hsr.set_profiling(False)
    counts = {k: int(t[k]) for k in COUNT_KEYS}
    s = statistics.mean(ms) / 1000.0
    res = {"workload": SOUP_WORKLOAD, "frames_per_s": round(1.0 / s, 2), "ms": round(s * 1000.0, 4),
           "mtris_per_s": round(counts["faces"] / s / 1e6, 1),
           "gfrags_per_s": round(counts["fragments"] / s / 1e9, 2),
           "note": "Gfrag/s counts covered (pixel, triangle) pairs, each tested against the depth buffer",
           "kernel_ms": {k: round(statistics.mean(v), 4) for k, v in kms.items()},
           "roofline": roofline(kms, counts, "soup_4m_2160p"), "counts": counts, "tuning": tuned}
    g.release()
    hsr.set_tuning(tile=old.tile, warps_per_cta=old.warps_per_cta, ctas_per_sm=old.ctas_per_sm)
    return res


def run_noclear(args) -> dict:
    """The cost of reading a target's prior contents in the raster: the 1920x1080 frame's main
    pass drawn with the fused clear (the raster reads nothing of the target) and drawn into a
    target cleared beforehand to the same values without the clear flag (each visited tile
    loads its prior depth, each shaded pixel its prior alpha).  Both give the same pixels; the
    raster-time difference bounds what staging the prior tile contents could save."""
    import torch

    import hsr
    from hsr import frame as hframe
    from hsr import scenes

    fr = scenes.displaced_frame()
    g = hframe.GpuFrame(fr)
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    hsr.set_profiling(True)
    main = g.descs[-1]
    noclear = hsr.DrawDesc.from_buffer_copy(main)
    noclear._keep = main._keep  # noqa: SLF001  the uniforms stay referenced
    noclear.flags = 0
    res = {}
    for name, desc in (("fused_clear", main), ("prior_contents", noclear)):
        kms = []
        for i in range(3 + args.steps):
            if desc is noclear:
                g.main.clear(fr.clear_rgba, fr.clear_depth)
            flush.zero_()
            torch.cuda.synchronize()
            hsr.draw_batch(g.descs[:-1] + [desc])
            if i >= 3:
                kms.append(hsr.last_timing()["kernel_ms"]["raster"])
        res[name] = {"raster_ms": round(statistics.mean(kms), 4)}
    hsr.set_profiling(False)
    g.release()
    res["difference_ms"] = round(res["prior_contents"]["raster_ms"] - res["fused_clear"]["raster_ms"], 4)
    res["workload"] = FRAME_WORKLOAD
    return res


def run_serve_small(args) -> dict:
    """Profiling case of the serving workload that fits a few GB of device memory: the 16
    resident meshes and ONE batch of 8 requests (320-327 of the stream), drawn 3 times with tile
    16, 4 warps, 8 CTAs per SM; returns the last draw's timing and counts."""
    import hsr
    from hsr import serve as hserve

    pool, tex, reqs = serve_inputs(328)
    reqs = reqs[320:328]
    rp = hserve.ResidentPool(pool, tex)
    hsr.set_tuning(tile=16, warps_per_cta=4, ctas_per_sm=8, bin_factor=4.0)
    hsr.set_profiling(True)
    vb = hserve.ViewBatch(rp, reqs)
    for _ in range(3):
        vb.draw_all()
    t = hsr.last_timing()
    hsr.set_profiling(False)
    vb.release()
    rp.release()
    return {"workload": "serving pool, one batch of requests 320-327, drawn 3 times",
            "batch_ms": round(t["batch_ms"], 4), "kernel_ms": {k: round(v, 4) for k, v in t["kernel_ms"].items()},
            "counts": {k: int(t[k]) for k in COUNT_KEYS}}


def run_soup_small(args) -> dict:
    """Profiling case of the depth-order stress workload that fits a few GB: the soup at a
    quarter of its size (1,000,000 triangles at 1920x1080: the same triangles per pixel, edge
    lengths and depth complexity), drawn 3 times with tile 16, 4 warps, 8 CTAs per SM."""
    import hsr
    from hsr import frame as hframe
    from hsr import scenes

    fr = scenes.soup_frame(1_000_000, 1920, 1080)
    g = hframe.GpuFrame(fr)
    hsr.set_tuning(tile=16, warps_per_cta=4, ctas_per_sm=8, bin_factor=4.0)
    hsr.set_profiling(True)
    for _ in range(3):
        g.render()
    t = hsr.last_timing()
    hsr.set_profiling(False)
    g.release()
    return {"workload": "triangle soup, 1,000,000 tris at 1920x1080 (a quarter of the stress frame), drawn 3 times",
            "batch_ms": round(t["batch_ms"], 4), "kernel_ms": {k: round(v, 4) for k, v in t["kernel_ms"].items()},
            "counts": {k: int(t[k]) for k in COUNT_KEYS}}


def run_views(args) -> dict:
    """64 views in one launch sequence: replayed CUDA graph vs one hsr_draw_batch vs one view
    at a time (8 meshes of 2,048-1,310,720 triangles, 256^2-1920x1080, Blinn / NormalMap,
    2048^2 shadow pass on half of them)."""
    import torch

    import hsr
    from hsr import scenes
    from hsr import serve as hserve

    pool = scenes.mesh_pool(scenes.VIEW_POOL_SPEC, seed=1)
    tex = scenes.pool_textures(4, 1024, seed=17)
    rp = hserve.ResidentPool(pool, tex)
    views = scenes.view_set(pool, 64, seed=3)
    vb = hserve.ViewBatch(rp, views)
    old = hsr.get_tuning()
    tuned = hsr.autotune(vb.descs, reps=2)
    plan = vb.plan()

    def timed(fn, k):
        torch.cuda.synchronize()
        s0 = time.perf_counter()
        for _ in range(k):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - s0) / k

    def replay():
        plan.launch()
        plan.wait()

    for fn in (vb.draw_each, vb.draw_all, replay):
        for _ in range(3):
            fn()
    k = max(5, args.steps // 3)
    te, ta, tp = timed(vb.draw_each, k), timed(vb.draw_all, k), timed(replay, k)
    res = {"views": 64, "pixels_per_batch": vb.pixels(),
           "triangles_in_pool": int(sum(p.mesh.nfaces for p in pool)),
           "graph_replay_frames_per_s": round(64 / tp, 1), "draw_batch_frames_per_s": round(64 / ta, 1),
           "per_view_frames_per_s": round(64 / te, 1), "graph_over_per_view": round(te / tp, 3),
           "tuning": tuned, "note": "wall clock per batch; per view = one hsr_draw_batch (shadow + main) per view"}
    plan.release()
    vb.release()
    rp.release()
    hsr.set_tuning(tile=old.tile, warps_per_cta=old.warps_per_cta, ctas_per_sm=old.ctas_per_sm)
    return res


# ------------------------------------------------------------------------------------------
# CPU: the oracle (C restatement of the reference's path) on this host's cores
# ------------------------------------------------------------------------------------------
def _serve_seeds() -> dict:
    """What a worker process needs to rebuild the serving workload (serve_inputs)."""
    from hsr import scenes

    return {"pool_spec": scenes.SERVE_POOL_SPEC, "pool_seed": 1, "ntex": 4, "tex_size": 1024, "tex_seed": 17,
            "nreq": N_REQUESTS, "req_seed": SEED}


def _process_renderer(procs: int):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import cpu_runner

    return cpu_runner.ProcessRenderer(procs, **_serve_seeds())


def cpu_latency() -> dict:
    """The reference path's single-frame latency on one core (one frame at a time): the plain
    512x512 frame, the 1920x1080 + 2048^2 shadow frame and the 4M-triangle soup."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import cpu_runner
    from hsr import scenes

    frames = {"plain_512": scenes.sphere_frame(4, 512, 512, seed=1), "frame_1080p": scenes.displaced_frame(),
              "soup_4m_2160p": scenes.soup_frame()}
    return cpu_runner.latency(frames, {"plain_512": 40, "frame_1080p": 6, "soup_4m_2160p": 3})


def cpu_baseline(seconds: float) -> dict:
    """Throughput: one oracle process per host core on the serving stream (independent
    processes, each taking the next request as it frees up; no request starts after
    `seconds`); latency: single frames on one core."""
    procs = os.cpu_count() or 1
    pr = _process_renderer(procs)
    try:
        n, s = pr.render_for(range(N_REQUESTS), seconds)
    finally:
        pr.close()
    return {"value": round(n / s, 4), "unit": "frames/s", "cores": procs, "kind": "port",
            "sample": f"the first {n} requests of the serving stream on {procs} independent processes (one per "
                      f"core), {s:.1f} s wall, no request started after {seconds:.0f} s",
            "latency_1core": cpu_latency()}


def run_reference(args, world, rank):
    """The reference's CPU implementation of the path (the oracle port) on every host core, on
    the same request stream: one process per core, each step the next 64 requests, each
    request taken by whichever process frees up first."""
    if rank != 0:
        return None
    procs = os.cpu_count() or 1
    pr = _process_renderer(procs)
    pos = 0
    secs = []
    try:
        for i in range(args.warmup + args.steps):
            s, _ = pr.render(range(pos, pos + BATCH))
            pos = (pos + BATCH) % (N_REQUESTS - BATCH)
            if i >= args.warmup:
                secs.append(s)
    finally:
        pr.close()
    value = args.steps * BATCH / sum(secs)
    per = [s * 1000.0 for s in secs]
    return {
        "metric": METRIC, "value": round(value, 4), "unit": "frames/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(statistics.mean(per), 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
        "config": {"workload": SERVE_WORKLOAD, "frames_per_step": BATCH, "l2": "n/a (host)"},
        "cpu_baseline": {"value": round(value, 4), "unit": "frames/s", "cores": procs, "kind": "port",
                         "sample": f"{BATCH} distinct requests per step on {procs} independent processes (one per "
                                   f"core), {args.steps} steps"},
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
    ap.add_argument("--quick", action="store_true", help="headline only (no plain / Poisson / sub-workloads)")
    ap.add_argument("--tile", type=int, default=0, help="fix the raster tile (8 or 16) instead of autotuning")
    ap.add_argument("--warps", type=int, default=0, help="with --tile: warps per CTA of the raster (4 or 8)")
    ap.add_argument("--ctas", type=int, default=0, help="with --tile: raster CTAs per SM")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--only", choices=["frame", "views", "soup", "noclear", "serve_small", "soup_small"], default=None,
                    help="run one sub-workload alone and print its result (for profiling)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world, rank, local = dist_setup()
    if args.impl == "reference":
        out = run_reference(args, world, rank)
    elif args.only:
        import torch

        import hsr

        torch.cuda.set_device(local)
        hsr.init(local)
        if args.tile:
            hsr.set_tuning(tile=args.tile, warps_per_cta=args.warps or (4 if args.tile == 16 else 8),
                           ctas_per_sm=args.ctas or None)
        out = {"frame": run_frame, "views": run_views, "soup": run_soup, "noclear": run_noclear,
               "serve_small": run_serve_small, "soup_small": run_soup_small}[args.only](args)
    else:
        out = run_ours(args, world, rank, local)
    if rank == 0 and out is not None:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
