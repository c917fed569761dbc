"""GPU on-disk BVH files: a build saved, loaded into another context and
registered (rrCudaRegisterGeometry) traces, feeds a scene build and updates
like the original; registration checks; serving-pool checkpoint and resume."""
import numpy as np
import pytest

from gpu_util import hits_np, to_dev, trace

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fmt", [0, 1])
def test_saved_build_loads_into_another_context(ctx, orc, tmp_path, fmt):
    from radeonrays_sdk_gb300 import bvh_io, rr, scenes
    v, i = scenes.heightfield(97, scenes.rng(92))
    n = i.shape[0]
    res = ctx.build_geometry(to_dev(v), to_dev(i), node_format=fmt)
    p = tmp_path / "hf.rrbvh"
    bvh_io.save_geometry(p, res, n)
    rays = scenes.incoherent_rays(5000, v.min(axis=0), v.max(axis=0), scenes.rng(92, 1))
    want = trace(ctx, res, rays, traversal=1)
    other = rr.Context()
    try:
        buf, n2 = bvh_io.load_geometry(other, p)
        assert n2 == n and np.array_equal(buf.cpu().numpy(), res.cpu().numpy())
        for trav in (0, 1, 3):
            assert np.array_equal(trace(other, buf, rays, traversal=trav), want), trav
        if fmt == 1:
            wide = trace(other, buf, rays, traversal=2)
            assert np.array_equal(wide[:, 2] != 0xFFFFFFFF, want[:, 2] != 0xFFFFFFFF)
        # The loaded buffer is a BLAS like any other, and can be updated.
        scene = other.build_scene([buf], np.eye(3, 4, dtype=np.float32)[None])
        other.set_traversal(1)
        s_hits = hits_np(other.intersect(scene, to_dev(rays)))
        other.set_traversal(0)
        assert np.array_equal(s_hits[:, 2] != 0xFFFFFFFF, want[:, 2] != 0xFFFFFFFF)
        assert np.array_equal(s_hits[:, 3], want[:, 3])
        other.update_geometry(to_dev(v), to_dev(i), buf)
        assert np.array_equal(trace(other, buf, rays, traversal=1), want)
        assert other.device_errors() == 0
    finally:
        other.close()


def test_register_checks_the_trailer(ctx):
    import torch
    from radeonrays_sdk_gb300 import rr, scenes
    v, i = scenes.soup(300, scenes.rng(93))
    res = ctx.build_geometry(to_dev(v), to_dev(i), node_format=0)
    L, c = ctx.L, ctx.ctx
    assert L.rrCudaRegisterGeometry(c, ctx.ptr(res), 300) == rr.RR_SUCCESS
    assert L.rrCudaRegisterGeometry(c, ctx.ptr(res), 299) == rr.RR_ERROR_INVALID_PARAMETER
    junk = torch.zeros_like(res)
    assert L.rrCudaRegisterGeometry(c, ctx.ptr(junk), 300) == rr.RR_ERROR_INVALID_PARAMETER


def test_pool_checkpoint_and_resume(ctx, tmp_path):
    from radeonrays_sdk_gb300 import bvh_io, serving
    from radeonrays_sdk_gb300 import scenes
    ms = [scenes.soup(2000, scenes.rng(94, 0)), scenes.heightfield(33, scenes.rng(94, 1))]
    pool = serving.ScenePool(ctx, budget_bytes=1 << 30)
    for k, (v, i) in enumerate(ms):
        pool.register(k, v, i)
        pool.acquire(k)
        pool.release(k)
    files = bvh_io.save_pool(pool, tmp_path)
    assert len(files) == 2
    fresh = serving.ScenePool(ctx, budget_bytes=1 << 30)
    for k, (v, i) in enumerate(ms):
        fresh.register(k, v, i)
    assert bvh_io.load_pool(fresh, tmp_path) == 2 and fresh.builds == 0
    reqs = serving.make_requests(ms, 12, rate_per_s=1e6, lo_rays=100, hi_rays=3000, seed=95)
    serving.Server(ctx, fresh, slot_rays=1 << 15, slots=2, max_requests=8).run(reqs)
    assert fresh.builds == 0
    for r in reqs:  # the pool's default scenes have 4-wide nodes: the launches ran the 4-wide kernel
        ctx.set_traversal(4)
        want = hits_np(ctx.intersect(pool.resident[r.scene], to_dev(r.rays), query=r.query, output=r.output))
        ctx.set_traversal(0)
        assert np.array_equal(r.hits, want), r.rid
