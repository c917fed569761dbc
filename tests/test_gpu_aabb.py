"""GPU AABB-list geometry (RR_PRIMITIVE_TYPE_AABB_LIST): build bit-identical
to the oracle (the mesh build over each box's (min, max, max) leaf
vertices), traversal equal to the oracle's box-leaf traversal for every
query/output and kernel, multi-request launches, update and quality build."""
import numpy as np
import pytest

from gpu_util import INVALID, hits_np, nodes_of, to_dev, trace
from test_gpu_build import same_nodes

pytestmark = pytest.mark.gpu


def boxes(n, seed, stride_floats=8):
    from radeonrays_sdk_gb300 import scenes
    g = scenes.rng(110, seed)
    c = g.random((n, 3))
    h = g.uniform(0.0005, 0.02, size=(n, 3))
    b = np.full((n, stride_floats), 7.0, np.float32)  # padding and the w lanes carry junk on purpose
    b[:, 0:3] = c - h
    b[:, 4:7] = c + h
    return b


def rays_for(n, seed):
    from radeonrays_sdk_gb300 import scenes
    return scenes.incoherent_rays(n, (0, 0, 0), (1, 1, 1), scenes.rng(111, seed))


@pytest.mark.parametrize("n,stride", [(1, 8), (2, 8), (100, 8), (5000, 8), (3000, 12)])
def test_aabb_build_and_trace_match_oracle(ctx, orc, n, stride):
    b = boxes(n, n, stride)
    res = ctx.build_aabbs(to_dev(b), stride=4 * stride)
    want_nodes, _, _ = orc.build_aabbs(b[:, :8])
    assert same_nodes(nodes_of(res, n), want_nodes)
    rays = rays_for(8192, n)
    for q in (0, 1):
        r = rays.copy()
        if q == 1:
            r[:, 7] = np.float32(0.05)
        for o in (0, 1):
            want = orc.trace(want_nodes, r, query=q, output=o, box_leaves=True)
            for trav in (0, 1, 3):
                assert np.array_equal(trace(ctx, res, r, query=q, output=o, traversal=trav), want), (q, o, trav)
    # Hit records of box leaves carry uv = (0, 0).
    h = trace(ctx, res, rays)
    hit = h[:, 2] != INVALID
    assert hit.any() and np.all(h[hit, 0] == 0) and np.all(h[hit, 1] == 0)
    assert ctx.device_errors() == 0


def test_aabb_batch_update_and_quality(ctx, orc):
    from radeonrays_sdk_gb300 import rr
    b = boxes(4000, 1)
    res = ctx.build_aabbs(to_dev(b))
    tri_v, tri_i = orc.aabb_vertices(b)
    from radeonrays_sdk_gb300 import scenes
    tv, ti = scenes.soup(2000, scenes.rng(112))
    tri = ctx.build_geometry(to_dev(tv), to_dev(ti), node_format=0)
    r1, r2 = rays_for(3000, 2), rays_for(5000, 3)
    got = ctx.intersect_batch([(res, to_dev(r1), 0, 0), (tri, to_dev(r2), 0, 0), (res, to_dev(r2), 1, 1)])
    nodes, _, _ = orc.build_aabbs(b)
    assert np.array_equal(hits_np(got[0]), orc.trace(nodes, r1, box_leaves=True))
    assert np.array_equal(hits_np(got[1]), orc.trace(orc.build_mesh(tv, ti)[0], r2))
    assert np.array_equal(hits_np(got[2]), orc.trace(nodes, r2, query=1, output=1, box_leaves=True))
    # Update: moved boxes on the same tree.
    b2 = b.copy()
    b2[:, 0:3] *= np.float32(1.25)
    b2[:, 4:7] *= np.float32(1.25)
    ctx.build_aabbs(to_dev(b2), update_of=res)
    v2, i2 = orc.aabb_vertices(b2)
    assert same_nodes(nodes_of(res, 4000), orc.fit(nodes, v2, i2))
    # Quality build: the restructured tree.
    q = ctx.build_aabbs(to_dev(b), quality=True)
    assert same_nodes(nodes_of(q, 4000), orc.restructure(nodes, 4000, 64, 3)[0])
    # Instances of AABB lists are not supported by the two-level kernels.
    with pytest.raises(rr.RRException) as e:
        ctx.build_scene([res], np.eye(3, 4, dtype=np.float32)[None])
    assert e.value.code == rr.RR_ERROR_NOT_IMPLEMENTED
    assert ctx.device_errors() == 0
