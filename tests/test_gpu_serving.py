"""GPU multi-request traversal (rrCudaCmdIntersectBatch) and the serving
loop: every request's hits are bit-identical alone and packed with others,
equal to the oracle, under scene eviction and overlapping launches."""
import numpy as np
import pytest

from gpu_util import INVALID, hits_np, to_dev

pytestmark = pytest.mark.gpu


def _scenes():
    from radeonrays_sdk_gb300 import scenes
    return [scenes.soup(3000, scenes.rng(50, 0)), scenes.heightfield(65, scenes.rng(50, 1)),
            scenes.soup(40000, scenes.rng(50, 2))]


def _alone(ctx, bvh, rays, q, o, traversal=1):
    """The request traced alone by rrCmdIntersect (the plain kernel, or the
    4-wide kernel for the 4-wide launches)."""
    ctx.set_traversal(traversal)
    h = hits_np(ctx.intersect(bvh, to_dev(rays), query=q, output=o))
    ctx.set_traversal(0)
    return h


def test_batch_equals_alone_and_oracle(ctx, orc):
    from radeonrays_sdk_gb300 import scenes
    ms = _scenes()
    bvhs = [ctx.build_geometry(to_dev(v), to_dev(i), node_format=0) for v, i in ms]
    empty = ctx.build_geometry(to_dev(np.zeros((0, 3), np.float32)), to_dev(np.zeros((0, 3), np.uint32)))
    reqs, host = [], []
    spec = [(0, 5000, 0, 0), (1, 1, 1, 0), (2, 77777, 0, 1), (0, 0, 0, 0), (1, 20000, 1, 1), (-1, 300, 0, 0),
            (2, 4096, 1, 0)]
    for k, (s, n, q, o) in enumerate(spec):
        v = ms[max(s, 0)][0]
        rays = scenes.incoherent_rays(n, v.min(axis=0), v.max(axis=0), scenes.rng(51, k))
        if q == 1 and n:
            rays[:, 7] = np.float32(0.2)
        reqs.append((empty if s < 0 else bvhs[s], to_dev(rays), q, o))
        host.append((s, rays, q, o))
    got = [hits_np(h) for h in ctx.intersect_batch(reqs)]
    assert ctx.device_errors() == 0
    for (s, rays, q, o), (bvh, _, _, _), g in zip(host, reqs, got):
        if rays.shape[0] == 0:
            continue
        assert np.array_equal(g, _alone(ctx, bvh, rays, q, o)), (s, q, o)
        if s >= 0:
            v, i = ms[s]
            want = orc.trace(orc.build_mesh(v, i)[0], rays, query=q, output=o)
            assert np.array_equal(g, want), (s, q, o)
        else:
            miss = g[:, 2] if o == 0 else g
            assert np.all(miss == INVALID)


def test_server_results_equal_alone_under_eviction(ctx):
    from radeonrays_sdk_gb300 import serving
    ms = _scenes()
    pool = serving.ScenePool(ctx, budget_bytes=0)
    for k, (v, i) in enumerate(ms):
        pool.register(k, v, i)
    sizes = [pool.result_bytes(k) for k in range(len(ms))]
    # Room for the largest scene plus one of the others: evictions happen.
    pool.budget = max(sizes) + sorted(sizes)[-2]
    reqs = serving.make_requests(ms, 60, rate_per_s=20000.0, lo_rays=64, hi_rays=30000, seed=52)
    server = serving.Server(ctx, pool, slot_rays=1 << 16, slots=3, max_requests=16)
    stats = server.run(reqs)
    assert stats["requests"] == 60 and stats["launches"] >= 2
    assert stats["latency_ms"]["p99"] >= stats["latency_ms"]["p50"] > 0
    assert ctx.device_errors() == 0
    bvhs = {k: pool.build(k) for k in range(len(ms))}
    for r in reqs:  # the pool's scenes have 4-wide nodes: the launches ran the 4-wide kernel
        want = _alone(ctx, bvhs[r.scene], r.rays, r.query, r.output, traversal=4)
        assert np.array_equal(r.hits, want), r.rid


@pytest.mark.parametrize("fmt", [2, 4])  # fp32 and 8-bit 4-wide nodes
def test_batch_bvh4_equals_alone_and_oracle(ctx, orc, fmt):
    """Requests whose geometries all carry 4-wide nodes of one form run the
    4-wide multi-request kernel: each request's hits equal the 4-wide
    kernel's on that request alone, bit for bit, and the oracle's up to
    equal-t ties."""
    from radeonrays_sdk_gb300 import scenes
    from gpu_util import tie_only_mismatch
    ms = _scenes()
    bvhs = [ctx.build_geometry(to_dev(v), to_dev(i), node_format=fmt) for v, i in ms]
    empty = ctx.build_geometry(to_dev(np.zeros((0, 3), np.float32)), to_dev(np.zeros((0, 3), np.uint32)))
    spec = [(0, 5000, 0, 0), (1, 1, 1, 0), (2, 77777, 0, 1), (0, 0, 0, 0), (1, 20000, 1, 1), (-1, 300, 0, 0),
            (2, 4096, 1, 0), (1, 30000, 0, 0)]
    reqs, host = [], []
    for k, (s, n, q, o) in enumerate(spec):
        v = ms[max(s, 0)][0]
        rays = scenes.incoherent_rays(n, v.min(axis=0), v.max(axis=0), scenes.rng(53, k))
        if q == 1 and n:
            rays[:, 7] = np.float32(0.2)
        reqs.append((empty if s < 0 else bvhs[s], to_dev(rays), q, o))
        host.append((s, rays, q, o))
    ctx.set_traversal(0)
    got = [hits_np(h) for h in ctx.intersect_batch(reqs)]
    ctx.set_traversal(1)  # a binary traversal option keeps the reference-order kernel
    plain = [hits_np(h) for h in ctx.intersect_batch(reqs)]
    ctx.set_traversal(0)
    assert ctx.device_errors() == 0
    for (s, rays, q, o), (bvh, _, _, _), g, p in zip(host, reqs, got, plain):
        if rays.shape[0] == 0:
            continue
        assert np.array_equal(g, _alone(ctx, bvh, rays, q, o, traversal=4)), (s, q, o)
        assert np.array_equal(p, _alone(ctx, bvh, rays, q, o, traversal=1)), (s, q, o)
        if s < 0:
            miss = g[:, 2] if o == 0 else g
            assert np.all(miss == INVALID)
            continue
        v, i = ms[s]
        want = orc.trace(orc.build_mesh(v, i)[0], rays, query=q, output=0)
        gf = g if o == 0 else None
        if o == 0:
            assert np.array_equal(gf[:, 2] != INVALID, want[:, 2] != INVALID)
            if q == 0:
                tie_only_mismatch(orc, rays, gf, want, v, i)
        else:
            assert np.array_equal(g != INVALID, want[:, 2] != INVALID)


def test_batch_mixed_4wide_forms_take_the_binary_kernel(ctx):
    """fp32 and 8-bit 4-wide geometries in one launch: the launch runs the
    reference-order kernel, so each request equals the binary kernel alone."""
    from radeonrays_sdk_gb300 import scenes
    ms = _scenes()
    bvhs = [ctx.build_geometry(to_dev(v), to_dev(i), node_format=2 + 2 * (k % 2)) for k, (v, i) in enumerate(ms)]
    reqs, host = [], []
    for k, (v, i) in enumerate(ms):
        rays = scenes.incoherent_rays(3000 + 500 * k, v.min(axis=0), v.max(axis=0), scenes.rng(54, k))
        reqs.append((bvhs[k], to_dev(rays), 0, 0))
        host.append(rays)
    ctx.set_traversal(0)
    got = [hits_np(h) for h in ctx.intersect_batch(reqs)]
    for (bvh, _, _, _), rays, g in zip(reqs, host, got):
        assert np.array_equal(g, _alone(ctx, bvh, rays, 0, 0, traversal=1))
    assert ctx.device_errors() == 0
