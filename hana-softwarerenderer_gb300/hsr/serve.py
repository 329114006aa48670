"""Resident mesh pool, batched views and the serving loop on top of the C ABI.

- ``ResidentPool`` keeps the meshes and textures of a workload on the device.
- ``ViewBatch`` builds the draws of many views (shadow pass + main pass each) on resident
  targets; they run as one ``hsr_draw_batch`` or as a replayable ``Plan`` (CUDA graph), or
  one view at a time (the plain per-frame path).
- ``serve_batched`` drives an ``hsr_server`` with a request stream at its arrival times;
  ``serve_plain`` renders the same stream one request at a time through the per-frame
  drop-in path (targets created for the request, the two passes drawn, the colour read
  back, the targets released).  Both return per-request latencies measured from each
  request's scheduled arrival.

The reference renders one frame per loop iteration on one thread (main.cpp:87-155,
scene.h:53-99); a request here is one such frame.
"""
from __future__ import annotations

import collections
import time

import numpy as np

from . import (ERR_OUT_OF_MEMORY, Mesh, PinnedArray, Plan, Server, Target, Texture, check, draw_batch, lib,
               make_desc)
from . import scenes

BLACK = (0, 0, 0, 255)
FLT_MAX = float(np.finfo(np.float32).max)


class ResidentPool:
    def __init__(self, pool: list, textures: list):
        self.pool = pool
        self.meshes = [Mesh(p.mesh) for p in pool]
        self.textures = [(Texture(d), Texture(n)) for d, n in textures]

    def release(self) -> None:
        for m in self.meshes:
            m.release()
        for d, n in self.textures:
            d.release()
            n.release()


class ViewBatch:
    """Targets and draw descriptors for a list of views (scenes.View)."""

    def __init__(self, rp: ResidentPool, views: list):
        self.rp = rp
        self.views = views
        self.keep: list = []
        self.mains: list[Target] = []
        self.shadows: list[Target | None] = []
        self.per_view: list[list] = []
        for v in views:
            mesh = rp.meshes[v.mesh]
            d, n = rp.textures[v.tex]
            main = Target(v.width, v.height)
            sh = Target(v.shadow, v.shadow) if v.shadow else None
            descs = []
            if sh is not None:
                descs.append(make_desc(mesh, scenes.SHADOW, v.sd, sh, d, n, clear=(BLACK, FLT_MAX), keep=self.keep))
            descs.append(make_desc(mesh, v.shader, v.sd, main, d, n, shadow_map=sh, clear=(BLACK, FLT_MAX),
                                   keep=self.keep))
            self.mains.append(main)
            self.shadows.append(sh)
            self.per_view.append(descs)
        self.descs = [d for ds in self.per_view for d in ds]

    def draw_all(self) -> None:
        draw_batch(self.descs)

    def draw_each(self) -> None:
        for ds in self.per_view:
            draw_batch(ds)

    def plan(self) -> Plan:
        return Plan(self.descs)

    def download(self, i: int) -> dict:
        return self.mains[i].download()

    def pixels(self) -> int:
        return sum(v.width * v.height + v.shadow * v.shadow for v in self.views)

    def release(self) -> None:
        for t in self.mains + [s for s in self.shadows if s is not None]:
            t.release()


class PinnedRing:
    """Page-locked output buffers carved from one ring in allocation order; a region is
    reused only after the request that owns it has completed.  Allocation and release are
    O(1): regions are handed out and reclaimed first in, first out."""

    def __init__(self, nbytes: int, buffer=None):
        """`buffer`: an object with `.array` (nbytes uint8) and `.release()`; page-locked memory
        from the library when omitted."""
        self.buf = buffer if buffer is not None else PinnedArray((nbytes,), np.uint8)
        self.cap = nbytes
        self.head = 0                                     # next free byte
        self.live: collections.deque = collections.deque()  # [key, start, end, freed] in allocation order
        self.by_key: dict = {}

    def _drop_freed(self) -> None:
        while self.live and self.live[0][3]:
            del self.by_key[self.live.popleft()[0]]

    def _fits(self, n: int) -> int:
        """Start of a free region of n bytes at the head (or the ring's start), or -1."""
        if not self.live:
            return self.head if self.head + n <= self.cap else 0
        s0 = self.live[0][1]
        if self.head > s0:
            if self.head + n <= self.cap:
                return self.head
            return 0 if n <= s0 else -1
        return self.head if self.head + n <= s0 else -1

    def alloc(self, n: int, key, reclaim) -> np.ndarray:
        n = (n + 255) // 256 * 256
        if n > self.cap:
            raise ValueError("request output larger than the pinned ring")
        while True:
            self._drop_freed()
            start = self._fits(n)
            if start >= 0:
                break
            reclaim()  # waits for the oldest outstanding request
        self.head = start + n
        entry = [key, start, start + n, False]
        self.live.append(entry)
        self.by_key[key] = entry
        return self.buf.array[start:start + n]

    def free(self, key) -> None:
        e = self.by_key.get(key)
        if e is not None:
            e[3] = True
        self._drop_freed()

    def release(self) -> None:
        self.buf.release()


def _wait_until(t0: float, ms: float) -> None:
    while True:
        d = ms - (time.perf_counter() - t0) * 1e3
        if d <= 0:
            return
        if d > 1.0:
            time.sleep((d - 0.5) / 1e3)


def serve_batched(rp: ResidentPool, reqs: list, pool_bytes: int = 40 << 30, max_batch: int = 64, slots: int = 2,
                  ring_bytes: int = 1 << 30, keep_outputs: bool = False, server: Server | None = None,
                  ring: "PinnedRing | None" = None) -> dict:
    """Submit `reqs` (scenes.Request) at their arrival times to an hsr_server; return
    per-request latency (done - scheduled arrival) and the run's wall time.  A `server` and
    `ring` passed in are used as they are and stay open (a long-running server across calls);
    otherwise both are made for this call and closed at its end."""
    own = server is None
    srv = server if server is not None else Server(pool_bytes, max_batch, slots)
    if ring is None:
        ring = PinnedRing(ring_bytes)
        own_ring = True
    else:
        own_ring = False
    outstanding: collections.deque = collections.deque()
    status: dict[int, dict] = {}
    outputs: dict[int, np.ndarray] = {}
    t0 = time.perf_counter()
    srv_t0 = srv.now_ms()  # server clock at t0 (ms); request i arrives at srv_t0 + arrival_ms
    tickets = []

    def complete(i: int, st: dict) -> None:
        status[i] = st
        if keep_outputs:
            r = reqs[i]
            outputs[i] = ring_view[i][: r.width * r.height * 4].reshape(r.height, r.width, 4).copy()
        ring.free(i)
        del ring_view[i]

    def reclaim_one():
        i, tk = outstanding.popleft()
        complete(i, srv.wait(tk))

    def reap():
        while outstanding:
            i, tk = outstanding[0]
            st = srv.poll(tk)
            if st is None:
                return
            outstanding.popleft()
            complete(i, st)

    ring_view: dict[int, np.ndarray] = {}
    try:
        for i, r in enumerate(reqs):
            _wait_until(t0, r.arrival_ms)
            reap()
            buf = ring.alloc(r.width * r.height * 4, i, reclaim_one)
            ring_view[i] = buf
            color = buf[: r.width * r.height * 4].reshape(r.height, r.width, 4)
            d, n = rp.textures[r.tex]
            tk = srv.submit(rp.meshes[r.mesh], r.shader, r.sd, r.width, r.height, diffuse=d, normal=n,
                            shadow_size=r.shadow, clear=(BLACK, FLT_MAX), shadow_clear=(BLACK, FLT_MAX),
                            out={"color": color})
            tickets.append(tk)
            outstanding.append((i, tk))
        while outstanding:
            reclaim_one()
        wall = time.perf_counter() - t0
    finally:
        # results still in flight are copied into the ring: wait for them before its memory
        # goes (a server we own finishes its batches when closed; one passed in keeps running)
        if own:
            srv.close()
        else:
            while outstanding:
                i, tk = outstanding.popleft()
                try:
                    srv.wait(tk)
                except Exception:  # noqa: BLE001  the original error is the one to raise
                    pass
        if own_ring:
            ring.release()
    lat = np.array([status[i]["done_ms"] - (srv_t0 + reqs[i].arrival_ms) for i in range(len(reqs))])
    ok = all(status[i]["status"] == 0 for i in range(len(reqs)))
    batches = {status[i]["batch"]: status[i]["batch_requests"] for i in range(len(reqs))}
    return {"latency_ms": lat, "wall_s": wall, "ok": ok, "status": status, "outputs": outputs,
            "batches": len(batches), "mean_batch": float(np.mean(list(batches.values()))) if batches else 0.0}


def render_plain(rp: ResidentPool, r, color_out: np.ndarray | None = None) -> None:
    """One request through the per-frame path: targets created, shadow + main pass in one
    hsr_draw_batch, colour read back, targets released."""
    mesh = rp.meshes[r.mesh]
    d, n = rp.textures[r.tex]
    keep: list = []
    main = Target(r.width, r.height)
    sh = Target(r.shadow, r.shadow) if r.shadow else None
    try:
        descs = []
        if sh is not None:
            descs.append(make_desc(mesh, scenes.SHADOW, r.sd, sh, d, n, clear=(BLACK, FLT_MAX), keep=keep))
        descs.append(make_desc(mesh, r.shader, r.sd, main, d, n, shadow_map=sh, clear=(BLACK, FLT_MAX), keep=keep))
        draw_batch(descs)
        if color_out is not None:
            main.download(color=True, depth=False, prim=False, out={"color": color_out})
    finally:
        main.release()
        if sh is not None:
            sh.release()


def serve_plain(rp: ResidentPool, reqs: list, keep_outputs: bool = False) -> dict:
    """The same stream served serially by the per-frame path (first come, first served)."""
    maxpx = max(r.width * r.height for r in reqs)
    buf = PinnedArray((maxpx * 4,), np.uint8)
    lat = np.empty(len(reqs))
    outputs = {}
    t0 = time.perf_counter()
    try:
        for i, r in enumerate(reqs):
            _wait_until(t0, r.arrival_ms)
            color = buf.array[: r.width * r.height * 4].reshape(r.height, r.width, 4)
            render_plain(rp, r, color)
            lat[i] = (time.perf_counter() - t0) * 1e3 - r.arrival_ms
            if keep_outputs:
                outputs[i] = color.copy()
        wall = time.perf_counter() - t0
    finally:
        buf.release()
    return {"latency_ms": lat, "wall_s": wall, "ok": True, "outputs": outputs}


def latency_summary(res: dict, n: int) -> dict:
    lat = res["latency_ms"]
    return {"frames_per_s": n / res["wall_s"], "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()), "wall_s": res["wall_s"]}


__all__ = ["ResidentPool", "ViewBatch", "PinnedRing", "serve_batched", "serve_plain", "render_plain",
           "latency_summary", "ERR_OUT_OF_MEMORY", "check", "lib"]
