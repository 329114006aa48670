"""CPU: the server's output ring (hsr.serve.PinnedRing) hands out regions in allocation order,
reuses a region only after its request completed, wraps around at the end, and asks the caller
to reclaim the oldest request when nothing fits."""
import numpy as np
import pytest

from hsr.serve import PinnedRing


class HostBuffer:
    def __init__(self, n):
        self.array = np.zeros(n, np.uint8)
        self.released = False

    def release(self):
        self.released = True


def ring(n=4096):
    return PinnedRing(n, buffer=HostBuffer(n))


def span(r, a):
    start = a.__array_interface__["data"][0] - r.buf.array.__array_interface__["data"][0]
    return start, start + a.size


def test_regions_are_disjoint_and_256_aligned():
    r = ring()
    got = [span(r, r.alloc(n, k, lambda: pytest.fail("no reclaim expected"))) for k, n in enumerate((10, 300, 1))]
    assert got == [(0, 256), (256, 768), (768, 1024)]


def test_wraps_after_the_oldest_frees():
    r = ring(1024)
    r.alloc(512, "a", None)
    r.alloc(256, "b", None)
    r.free("a")
    s, e = span(r, r.alloc(512, "c", None))  # 256 left at the end: wraps to the freed start
    assert (s, e) == (0, 512)


def test_out_of_order_free_waits_for_the_head():
    r = ring(1024)
    r.alloc(512, "a", None)
    r.alloc(512, "b", None)
    r.free("b")  # the head ("a") is still live: nothing can be reused yet
    calls = []

    def reclaim():
        calls.append(1)
        r.free("a")

    s, e = span(r, r.alloc(512, "c", reclaim))
    assert calls == [1] and (s, e) == (0, 512)


def test_full_ring_reclaims_until_it_fits_and_rejects_oversize():
    r = ring(1024)
    for k in range(4):
        r.alloc(256, k, None)
    order = []

    def reclaim():
        k = len(order)
        order.append(k)
        r.free(k)

    r.alloc(600, "big", reclaim)  # needs the three oldest regions
    assert order == [0, 1, 2]
    with pytest.raises(ValueError):
        r.alloc(2048, "too big", reclaim)


def test_release_releases_the_buffer():
    r = ring()
    r.release()
    assert r.buf.released
