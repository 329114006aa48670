"""The oracle timed on the host's cores — TEST AND CPU-BASELINE INFRASTRUCTURE ONLY.

Used by bench.py's ``cpu_baseline`` leg and its ``--impl reference`` arm, never by the
product.  The reference renders on one thread (main.cpp:87-155), so its throughput on a
many-core host is that of independent processes: ``ProcessRenderer`` starts one spawned
worker process per core, each holding its own copy of the serving workload (built from the
same seeds), and hands out whole requests as workers free up; ``latency`` renders single
frames one at a time on the calling thread (one core).

Workers are started with ``spawn`` (a process forked after the CUDA context exists can
hang), and they import neither the library nor torch: only numpy, the scene generators and
liboracle.so.
"""
from __future__ import annotations

import multiprocessing as mp
import os
import queue
import statistics
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

_W: dict = {}


def _paths() -> None:
    for p in (os.path.join(ROOT, "hana-softwarerenderer_gb300"), HERE):
        if p not in sys.path:
            sys.path.insert(0, p)


def _init(pool_spec, pool_seed: int, ntex: int, tex_size: int, tex_seed: int, nreq: int, req_seed: int) -> None:
    _paths()
    from hsr import scenes

    import oracle

    oracle.lib()
    pool = scenes.mesh_pool(pool_spec, seed=pool_seed)
    tex = scenes.pool_textures(ntex, tex_size, seed=tex_seed)
    reqs = scenes.request_stream(pool, nreq, rate_per_s=1000.0, seed=req_seed, ntex=ntex)
    _W.update(pool=pool, tex=tex, reqs=reqs)


def _render(i: int) -> float:
    from hsr import scenes

    import oracle

    t0 = time.perf_counter()
    oracle.render_frame(scenes.view_frame(_W["reqs"][i], _W["pool"], _W["tex"]))
    return time.perf_counter() - t0


def _worker(q_in, q_out, initargs) -> None:
    _init(*initargs)
    q_out.put(("ready", os.getpid()))
    while True:
        i = q_in.get()
        if i is None:
            return
        try:
            q_out.put((i, _render(i)))
        except Exception as e:  # noqa: BLE001  reported to the parent, which raises it
            q_out.put((i, f"{type(e).__name__}: {e}"))


class ProcessRenderer:
    """`procs` worker processes, each with the serving workload of the given seeds; requests
    go through one queue, so each is taken by whichever worker frees up first."""

    def __init__(self, procs: int, pool_spec, pool_seed: int, ntex: int, tex_size: int, tex_seed: int, nreq: int,
                 req_seed: int):
        self.procs = procs
        ctx = mp.get_context("spawn")
        self.q_in, self.q_out = ctx.Queue(), ctx.Queue()
        initargs = (pool_spec, pool_seed, ntex, tex_size, tex_seed, nreq, req_seed)
        self.workers = [ctx.Process(target=_worker, args=(self.q_in, self.q_out, initargs), daemon=True)
                        for _ in range(procs)]
        for w in self.workers:
            w.start()
        # every worker has built its workload before any timing starts; a worker that died
        # in its set-up is an error, not a wait
        ready = 0
        t0 = time.perf_counter()
        while ready < procs:
            try:
                self.q_out.get(timeout=2)
                ready += 1
            except queue.Empty:
                dead = [w for w in self.workers if not w.is_alive()]
                if dead or time.perf_counter() - t0 > 900:
                    self.close()
                    raise RuntimeError(f"oracle worker processes failed to start ({len(dead)} exited)")

    def _result(self) -> float:
        i, r = self.q_out.get(timeout=900)
        if isinstance(r, str):
            raise RuntimeError(f"oracle worker failed on request {i}: {r}")
        return r

    def render(self, indices) -> tuple:
        """Render the requests; returns (wall seconds, per-request seconds)."""
        indices = list(indices)
        t0 = time.perf_counter()
        for i in indices:
            self.q_in.put(i)
        per = [self._result() for _ in indices]
        return time.perf_counter() - t0, per

    def render_for(self, indices, seconds: float) -> tuple:
        """Render requests in order until `seconds` of wall time have passed (no request starts
        after that); returns (requests rendered, wall seconds)."""
        it = iter(indices)
        t0 = time.perf_counter()
        inflight = 0
        for _ in range(self.procs):
            i = next(it, None)
            if i is None:
                break
            self.q_in.put(i)
            inflight += 1
        done = 0
        while inflight:
            self._result()
            inflight -= 1
            done += 1
            if time.perf_counter() - t0 < seconds:
                i = next(it, None)
                if i is not None:
                    self.q_in.put(i)
                    inflight += 1
        return done, time.perf_counter() - t0

    def close(self) -> None:
        for w in self.workers:
            if w.is_alive():
                self.q_in.put(None)
        for w in self.workers:
            w.join(timeout=30)
            if w.is_alive():
                w.terminate()
                w.join(timeout=5)


def latency(frames: dict, counts: dict) -> dict:
    """One core, one frame at a time: {name: {frames, p50_ms, p99_ms, mean_ms}}."""
    _paths()
    import numpy as np

    import oracle

    out = {}
    for name, fr in frames.items():
        ms = []
        for _ in range(counts[name]):
            t0 = time.perf_counter()
            oracle.render_frame(fr)
            ms.append((time.perf_counter() - t0) * 1e3)
        out[name] = {"frames": len(ms), "p50_ms": round(float(np.percentile(ms, 50)), 3),
                     "p99_ms": round(float(np.percentile(ms, 99)), 3), "mean_ms": round(statistics.mean(ms), 3)}
    return out
