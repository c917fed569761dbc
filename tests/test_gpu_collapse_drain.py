"""GPU tests of the collapse's drain kernel (k_collapse_drain in wide.cu).

The host launches one level kernel per collapse level for as many levels as a
tree of the batch's size normally has, and one single-block drain that does
any deeper level.  RR_CUDA_COLLAPSE_LEVELS=k makes the host launch only k
level kernels, so the drain does most of an ordinary tree here.  The wide
trees must then have the same structure properties, and trace to the same
hits, as the normal builds: the collapse numbers nodes in a different order,
but every node's children and their slot order are the same.
"""
import numpy as np
import pytest

from gpu_util import INVALID, build, hits_np, to_dev, trace
from test_gpu_bvh4 import check_structure
from test_gpu_bvh4q8 import check_conservative

pytestmark = pytest.mark.gpu

WIDE8, BVH4, BVH4Q8 = 1, 2, 4


@pytest.mark.parametrize("fmt", [BVH4, BVH4Q8, WIDE8])
@pytest.mark.parametrize("levels", [1, 3])
def test_drain_builds_the_same_tree(ctx, monkeypatch, fmt, levels):
    from radeonrays_sdk_gb300 import scenes
    v, i, rays = scenes.config1(grid=257, nrays=1 << 16)
    normal = build(ctx, v, i, node_format=fmt)
    trav = 2 if fmt == WIDE8 else 4
    want = trace(ctx, normal, rays, traversal=trav)
    monkeypatch.setenv("RR_CUDA_COLLAPSE_LEVELS", str(levels))
    drained = build(ctx, v, i, node_format=fmt)
    monkeypatch.delenv("RR_CUDA_COLLAPSE_LEVELS")
    if fmt == BVH4:
        check_structure(drained, v, i)
    elif fmt == BVH4Q8:
        check_conservative(drained, v, i)
    got = trace(ctx, drained, rays, traversal=trav)
    assert np.array_equal(got, want)
    anyr = rays.copy()
    anyr[:, 7] = np.float32(0.05)
    assert np.array_equal(trace(ctx, drained, anyr, query=1, traversal=trav),
                          trace(ctx, normal, anyr, query=1, traversal=trav))
    assert ctx.device_errors() == 0


def test_drain_in_a_fused_build(ctx, monkeypatch):
    """A fused build of uneven meshes with the drain doing levels 2 on:
    every geometry traces as its one-by-one build does."""
    import torch
    from radeonrays_sdk_gb300 import scenes
    meshes, host = [], []
    for k, n in enumerate((1, 2, 7, 300, 5000, 40000)):
        v, i = scenes.soup(n, scenes.rng(71, k))
        host.append((v, i))
        meshes.append((torch.from_numpy(v).cuda(), torch.from_numpy(i.view(np.int32)).cuda()))
    monkeypatch.setenv("RR_CUDA_COLLAPSE_LEVELS", "2")
    fused = ctx.build_geometries(meshes, node_format=BVH4, api="batch")
    torch.cuda.synchronize()
    monkeypatch.delenv("RR_CUDA_COLLAPSE_LEVELS")
    for (v, i), res in zip(host, fused):
        rays = scenes.incoherent_rays(4096, v.min(axis=0), v.max(axis=0), scenes.rng(71, 99))
        alone = build(ctx, v, i, node_format=BVH4)
        if i.shape[0] > 1:
            check_structure(res, v, i)
        got = hits_np(ctx.intersect(res, to_dev(rays)))
        want = hits_np(ctx.intersect(alone, to_dev(rays)))
        assert np.array_equal(got, want)
        assert np.any(got[:, 2] != INVALID) or i.shape[0] < 8
    assert ctx.device_errors() == 0
