"""CPU: the bench.py contract pieces that need no GPU — the roofline's choice and byte model,
the max-over-ranks timing on two gloo ranks, and the reference arm launched under torchrun
with two ranks (rank 0 alone measures and prints one JSON line)."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402

COUNTS = {"faces": 50_884_881, "vertices": 25_466_468, "normals": 0, "records": 9_128_663, "bin_pairs": 13_002_767,
          "pixels": 133_068_066, "shaded_pixels": 51_022_263, "clipped_faces": 84_957, "raster_pixels": 52_734_190,
          "tiles": 1_842_000, "split_triangles": 1_200, "payload_bytes": 9_128_663 * 96}


def test_roofline_reports_every_kernel_and_the_largest():
    """Every kernel of the launch sequence gets its share, algorithmic bytes and fraction of
    the peak; the headline is the kernel with the largest share, frac = achieved / peak with
    achieved = algorithmic bytes / the kernel's time."""
    km = {"vertex": [0.12], "cull": [0.87], "emit": [0.51], "clip": [0.2], "split": [0.05], "scan": [0.02],
          "scatter": [0.39], "raster": [2.1]}
    r = bench.roofline(km, COUNTS, "serve_batch64")
    assert r["kernel"] == "raster"
    kb = bench.kernel_bytes(COUNTS)
    assert r["algorithmic_bytes"] == int(kb["raster"])
    assert abs(r["achieved"] - kb["raster"] / 2.1e-3 / 1e9) < 0.1
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-3
    assert set(r["kernels"]) == set(km)
    assert abs(sum(k["share"] for k in r["kernels"].values()) - 1.0) < 1e-3
    for name, k in r["kernels"].items():
        assert k["algorithmic_bytes"] == int(kb[name])
        assert abs(k["frac"] - k["achieved_gbs"] / r["peak"]) < 1e-3


def test_clear_bytes_move_from_raster_to_scatter():
    """Pixels outside the raster's tiles are written by the clear in the scatter grid."""
    kb = bench.kernel_bytes(COUNTS)
    everything_in_raster = bench.kernel_bytes(dict(COUNTS, raster_pixels=COUNTS["pixels"]))
    moved = (COUNTS["pixels"] - COUNTS["raster_pixels"]) * 12
    assert kb["scatter"] - everything_in_raster["scatter"] == moved
    assert everything_in_raster["raster"] - kb["raster"] == moved


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "WORLD_SIZE": "2", "RANK": str(rank),
                       "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import bench as b
    import torch.distributed as dist

    world, r, _ = b.dist_setup()
    b.dist_barrier(world)
    q.put((r, b.dist_max(1.5 + r, world)))
    dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = dict(q.get(timeout=10) for _ in range(2))
    assert got == {0: 2.5, 1: 2.5}


def test_reference_arm_under_torchrun_two_ranks():
    env = dict(os.environ, OMP_NUM_THREADS="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl", "reference", "--steps", "1",
           "--warmup", "3"]
    res = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, res.stdout
    out = json.loads(lines[0])
    assert out["impl"] == "reference" and out["n_gpus"] == 2 and out["steps"] == 1 and out["warmup"] == 3
    assert out["value"] > 0 and out["unit"] == "frames/s" and out["higher_is_better"] is True
    assert out["cpu_baseline"]["kind"] == "port" and out["cpu_baseline"]["cores"] >= 1
    assert out["e2e"]["h2d_bytes_per_step"] == 0 and out["gpu_launches"] == 0
