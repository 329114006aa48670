"""CPU: the request loop of hsr.serve.serve_batched (the end-to-end leg of bench.py) against a
stand-in server with the Python Server interface: every request is submitted once with its own
ring region, waited for, and its latency taken from its scheduled arrival; a full ring makes the
loop wait for the oldest request; a server passed in stays open across calls."""
import types

import numpy as np
import pytest

from hsr import scenes
from hsr import serve as hserve


class HostBuffer:
    def __init__(self, n):
        self.array = np.zeros(n, np.uint8)

    def release(self):
        pass


class FakeServer:
    """Completes requests in submission order; each finishes `step_ms` after the previous one
    on its own clock, and writes a marker into the request's colour array."""

    def __init__(self, step_ms=1.0):
        self.t = 1000.0
        self.step = step_ms
        self.queue, self.done, self.closed = [], {}, False
        self.next = 1

    def now_ms(self):
        return self.t

    def submit(self, mesh, shader, sd, width, height, diffuse=None, normal=None, shadow_size=0, clear=None,
               shadow_clear=None, out=None):
        assert not self.closed
        tk = self.next
        self.next += 1
        out["color"][...] = tk & 255
        self.queue.append(tk)
        return tk

    def _finish_one(self):
        tk = self.queue.pop(0)
        self.t += self.step
        self.done[tk] = {"status": 0, "batch": (tk - 1) // 4 + 1, "batch_requests": 4, "submit_ms": 0.0,
                         "launch_ms": 0.0, "done_ms": self.t}

    def poll(self, tk):
        return self.done.get(tk)

    def wait(self, tk):
        while tk not in self.done:
            self._finish_one()
        return self.done[tk]

    def close(self):
        self.closed = True


def requests(n, w=16, h=8):
    sd = np.zeros((), dtype=np.uint8)
    return [scenes.Request(0, 0, scenes.BLINN, w, h, 0, sd, float(i)) for i in range(n)]


RP = types.SimpleNamespace(meshes=[object()], textures=[(object(), object())])


def test_every_request_once_with_latency_from_its_arrival():
    srv, reqs = FakeServer(step_ms=0.5), requests(10)
    ring = hserve.PinnedRing(1 << 16, buffer=HostBuffer(1 << 16))
    res = hserve.serve_batched(RP, reqs, server=srv, ring=ring, keep_outputs=True)
    assert res["ok"] and len(res["status"]) == 10 and not srv.closed
    for i in range(10):
        assert (res["outputs"][i] == (i + 1) & 255).all()  # each request kept its own region
    assert np.all(res["latency_ms"] == np.array([res["status"][i]["done_ms"] - (1000.0 + i) for i in range(10)]))
    assert res["batches"] == 3 and res["wall_s"] > 0
    assert not ring.live  # every region returned


def test_full_ring_waits_for_the_oldest_request():
    srv = FakeServer()
    reqs = requests(12, w=32, h=32)  # 4 KiB of colour each
    ring = hserve.PinnedRing(3 * 4096, buffer=HostBuffer(3 * 4096))
    res = hserve.serve_batched(RP, reqs, server=srv, ring=ring, keep_outputs=True)
    assert res["ok"] and len(res["outputs"]) == 12
    for i in range(12):
        assert (res["outputs"][i] == (i + 1) & 255).all()


def test_server_passed_in_serves_two_calls():
    srv = FakeServer()
    ring = hserve.PinnedRing(1 << 16, buffer=HostBuffer(1 << 16))
    a = hserve.serve_batched(RP, requests(5), server=srv, ring=ring)
    b = hserve.serve_batched(RP, requests(7), server=srv, ring=ring)
    assert a["ok"] and b["ok"] and len(b["status"]) == 7 and not srv.closed
