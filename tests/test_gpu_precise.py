"""The precise triangle test on the GPU (RRCudaTraversalOptions::triangle_test
= RR_CUDA_TRIANGLE_TEST_WATERTIGHT) against its CPU twin in the oracle
(oracle.trace_precise): watertight decision, accurate t and uv, robust box
test.

  * persistent binary kernel (the reference's visit order): RRHit records
    bit-identical to the oracle for every query and output;
  * 4-wide kernel (nearest child first): hit flags identical, primitive ids
    identical except exact equal-t ties, records identical where the
    primitive is the same;
  * rays aimed at shared vertices and edges: no ray leaks through the mesh
    (the reference's test lets several percent through);
  * host-buffer tracing, the option checks and the autotuner keep the mode.
"""
import numpy as np
import pytest

from gpu_util import INVALID, hits_np, tie_only_mismatch, to_dev

pytestmark = pytest.mark.gpu

PERSISTENT, BVH4, WATERTIGHT = 3, 4, 1


def _trace(ctx, bvh, rays, traversal, q=0, o=0):
    ctx.set_traversal(traversal, triangle_test=WATERTIGHT)
    try:
        return hits_np(ctx.intersect(bvh, to_dev(rays), query=q, output=o))
    finally:
        ctx.set_traversal(0)


@pytest.fixture(scope="module")
def hf():
    from radeonrays_sdk_gb300 import scenes
    v, i, rays = scenes.config1(grid=257, nrays=1 << 18)
    occl = rays.copy()
    occl[:, 7] = scenes.rng(130).uniform(0.01, 0.5, rays.shape[0]).astype(np.float32)
    return v, i, rays, occl


@pytest.mark.parametrize("q,o", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_persistent_precise_is_bit_identical_to_oracle(ctx, orc, hf, q, o):
    v, i, rays, occl = hf
    r = occl if q == 1 else rays
    nodes, _, _ = orc.build_mesh(v, i)
    want, _ = orc.trace_precise(nodes, r, query=q, output=o, threads=16)
    bvh = ctx.build_geometry(to_dev(v), to_dev(i))
    got = _trace(ctx, bvh, r, PERSISTENT, q, o)
    assert np.array_equal(got, want)
    assert ctx.device_errors() == 0


def test_bvh4_precise_matches_oracle(ctx, orc, hf):
    v, i, rays, occl = hf
    nodes, _, _ = orc.build_mesh(v, i)
    want, _ = orc.trace_precise(nodes, rays, threads=16)
    for quality in (False, True):
        bvh = ctx.build_geometry(to_dev(v), to_dev(i), quality=quality)
        got = _trace(ctx, bvh, rays, BVH4)
        hit = want[:, 2] != INVALID
        assert np.array_equal(got[:, 2] != INVALID, hit)
        tie_only_mismatch(orc, rays, got, want, v, i, precise=True)
        same = got[:, 3] == want[:, 3]
        assert np.array_equal(got[same & hit], want[same & hit])
        wa, _ = orc.trace_precise(nodes, occl, query=1, threads=16)
        ga = _trace(ctx, bvh, occl, BVH4, q=1)
        assert np.array_equal(ga[:, 2] != INVALID, wa[:, 2] != INVALID)
    assert ctx.device_errors() == 0


def test_precise_is_watertight(ctx, orc):
    from edge_rays import bumpy_grid, edge_rays
    v, i = bumpy_grid()
    rays = edge_rays(v)
    nodes, _, _ = orc.build_mesh(v, i)
    want, _ = orc.trace_precise(nodes, rays, threads=16)
    assert np.all(want[:, 2] != INVALID)
    bvh = ctx.build_geometry(to_dev(v), to_dev(i))
    ctx.set_traversal(1)
    ref = hits_np(ctx.intersect(bvh, to_dev(rays)))
    ctx.set_traversal(0)
    assert (ref[:, 2] == INVALID).sum() > 1000  # the reference's test leaks here
    got = _trace(ctx, bvh, rays, PERSISTENT)
    assert np.array_equal(got, want)
    got4 = _trace(ctx, bvh, rays, BVH4)
    assert np.all(got4[:, 2] != INVALID)
    tie_only_mismatch(orc, rays, got4, want, v, i, precise=True)


def test_precise_host_buffers_equal_device_trace(ctx, hf):
    import torch
    v, i, rays, _ = hf
    bvh = ctx.build_geometry(to_dev(v), to_dev(i))
    rh = torch.from_numpy(rays).pin_memory()
    for trav in (PERSISTENT, BVH4, 0):
        ctx.set_traversal(trav, triangle_test=WATERTIGHT)
        try:
            want = hits_np(ctx.intersect(bvh, to_dev(rays)))
            got = ctx.intersect_host(bvh, rh, chunk_rays=16384).numpy().view(np.uint32)
        finally:
            ctx.set_traversal(0)
        assert np.array_equal(got, want), trav
    assert ctx.device_errors() == 0


def test_precise_option_checks_and_autotune(ctx, orc, hf):
    import ctypes as C
    from radeonrays_sdk_gb300 import rr
    v, i, rays, _ = hf
    for trav in (1, 2):  # plain and 8-wide kernels keep the reference's test
        o = rr.RRCudaTraversalOptions(C.sizeof(rr.RRCudaTraversalOptions), trav, 0, 0, 0, 0, 0, WATERTIGHT)
        assert ctx.L.rrCudaSetTraversalOptions(ctx.ctx, C.byref(o)) == rr.RR_ERROR_INVALID_PARAMETER
    o = rr.RRCudaTraversalOptions(C.sizeof(rr.RRCudaTraversalOptions), 0, 0, 0, 0, 0, 0, 7)
    assert ctx.L.rrCudaSetTraversalOptions(ctx.ctx, C.byref(o)) == rr.RR_ERROR_INVALID_PARAMETER
    bvh = ctx.build_geometry(to_dev(v), to_dev(i))
    scene = ctx.build_scene([bvh], np.eye(3, 4, dtype=np.float32)[None])
    ctx.set_traversal(0, triangle_test=WATERTIGHT)
    try:
        with pytest.raises(rr.RRException) as e:
            ctx.intersect(scene, to_dev(rays[:1000]))
        assert e.value.code == rr.RR_ERROR_NOT_IMPLEMENTED
        choice = ctx.autotune(bvh, to_dev(rays))
        assert choice["traversal"] in (PERSISTENT, BVH4)
        got = hits_np(ctx.intersect(bvh, to_dev(rays)))
        opts = rr.RRCudaTraversalOptions()
        ctx.L.rrCudaGetTraversalOptions(ctx.ctx, C.byref(opts))
        assert opts.triangle_test == WATERTIGHT
    finally:
        ctx.set_traversal(0)
    nodes, _, _ = orc.build_mesh(v, i)
    want, _ = orc.trace_precise(nodes, rays, threads=16)
    assert np.array_equal(got[:, 2] != INVALID, want[:, 2] != INVALID)
    tie_only_mismatch(orc, rays, got, want, v, i, precise=True)
