"""Host logic of the serving loop on CPU: the scene pool's budget, LRU
eviction and pinning, and the request generator's distributions."""
import numpy as np
import pytest

from radeonrays_sdk_gb300 import rr, serving


class _Buf:
    def __init__(self, n):
        self.n = n

    def numel(self):
        return self.n


class _FakeCtx:
    def geometry_requirements(self, ntri, node_format, bits, nvert, stride):
        return 0, ntri * 100


class _Pool(serving.ScenePool):
    def build(self, scene):
        return _Buf(self.result_bytes(scene))


def _pool(budget, sizes):
    p = _Pool(_FakeCtx(), budget)
    for k, n in enumerate(sizes):
        p.register(k, np.zeros((3 * n, 3), np.float32), np.zeros((n, 3), np.uint32))
    return p


def test_pool_builds_once_and_evicts_lru():
    p = _pool(1000, [3, 4, 5])
    p.acquire(0)
    p.release(0)
    p.acquire(1)
    p.release(1)
    assert p.bytes == 700 and p.builds == 2
    p.acquire(0)  # resident: no build, becomes most recently used
    p.release(0)
    assert p.builds == 2
    p.acquire(2)  # needs 500: evicts scene 1 (least recently used), not 0
    assert 1 not in p.resident and 0 in p.resident and p.evictions == 1
    assert p.bytes == 800
    p.release(2)


def test_pool_never_evicts_pinned():
    p = _pool(1000, [3, 4, 5])
    p.acquire(1)
    p.acquire(2)
    with pytest.raises(MemoryError):
        p.acquire(0)  # 900 pinned + 300 > 1000
    p.release(2)
    p.acquire(0)  # now scene 2 can go
    assert 2 not in p.resident and p.bytes == 700


def test_pool_rejects_scene_larger_than_budget():
    p = _pool(100, [5])
    with pytest.raises(MemoryError):
        p.acquire(0)


def test_request_generator():
    meshes = [(np.random.default_rng(k).random((30, 3)).astype(np.float32), np.zeros((10, 3), np.uint32))
              for k in range(4)]
    reqs = serving.make_requests(meshes, 400, rate_per_s=1000.0, lo_rays=16, hi_rays=4096)
    t = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(t) > 0)
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert 0.7e-3 < gaps.mean() < 1.3e-3  # exponential gaps, mean 1 / rate
    sizes = np.array([r.rays.shape[0] for r in reqs])
    assert sizes.min() >= 16 and sizes.max() <= 4096
    anyq = np.array([r.query == rr.RR_INTERSECT_QUERY_ANY for r in reqs])
    assert 0.2 < anyq.mean() < 0.4
    for r in reqs:
        lo, hi = meshes[r.scene][0].min(axis=0), meshes[r.scene][0].max(axis=0)
        assert np.all(r.rays[:, :3] >= lo - 1e-6) and np.all(r.rays[:, :3] <= hi + 1e-6)
        if r.query == rr.RR_INTERSECT_QUERY_ANY:
            assert np.all((r.rays[:, 7] >= 0.01) & (r.rays[:, 7] <= 0.5))
