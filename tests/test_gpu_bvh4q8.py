"""GPU tests of the quantised 4-wide format (RR_CUDA_NODE_FORMAT_BVH4Q8: 64-byte
nodes, 8-bit child bounds rounded outward against a per-node fp32 origin and
power-of-two scales) and its traversal (RR_CUDA_TRAVERSAL_BVH4).

The decoded child boxes contain the exact child boxes, and every leaf
triangle is re-tested on its exact box with the reference's slab arithmetic
before the reference's triangle test.  Hit/miss flags therefore equal the
reference's for closest and any hit, closest-hit primitives equal it except
equal-t ties, and uv is bit-identical wherever the primitive is the same.
"""
import numpy as np
import pytest

from conftest import MESH_FIXTURES, golden
from gpu_util import INVALID, build, nodes_of, tie_only_mismatch, trace, trailer_of

pytestmark = pytest.mark.gpu

Q8_FORMAT, BVH4 = 4, 4


def q8_nodes(res, n):
    """Decoded quantised nodes: lo, hi (cnt, 3, 4) float64 and child refs."""
    tr = trailer_of(res, n)
    raw = res.cpu().numpy()
    off, cnt = int(tr["wide_nodes_off"]), int(tr["wide_count"])
    a = raw[off: off + 64 * cnt].reshape(cnt, 64)
    p = a[:, 0:12].copy().view(np.float32).astype(np.float64)  # (cnt, 3)
    e = a[:, 12:15].astype(np.int64)
    scale = np.ldexp(1.0, e - 127)  # (cnt, 3)
    ch = a[:, 16:32].copy().view(np.uint32)  # (cnt, 4)
    q = a[:, 32:56].reshape(cnt, 6, 4).astype(np.float64)
    lo = p[:, :, None] + q[:, 0:3, :] * scale[:, :, None]
    hi = p[:, :, None] + q[:, 3:6, :] * scale[:, :, None]
    return lo, hi, ch


def check_conservative(res, v, i):
    """Every binary leaf is referenced once, every 4-wide node but the root
    once, and every decoded leaf box contains its triangle's exact box."""
    n = i.shape[0]
    lo, hi, ch = q8_nodes(res, n)
    leaves = ch[(ch != INVALID) & (ch >= 0x80000000)] & 0x7FFFFFFF
    assert np.array_equal(np.sort(leaves), np.arange(n - 1, 2 * n - 1))
    inner = ch[(ch != INVALID) & (ch < 0x80000000)]
    assert np.array_equal(np.sort(inner), np.arange(1, lo.shape[0]))
    nodes = nodes_of(res, n)
    tri = v[i.astype(np.int64)].astype(np.float64)
    prim = nodes["child1"][n - 1:]
    k, s = np.nonzero((ch != INVALID) & (ch >= 0x80000000))
    t = tri[prim[(ch[k, s] & 0x7FFFFFFF).astype(np.int64) - (n - 1)]]
    assert np.all(lo[k, :, s] <= t.min(axis=1)) and np.all(hi[k, :, s] >= t.max(axis=1))


def compare(orc, rays, got, want, v, i, near_ulp=0):
    assert np.array_equal(got[:, 2] != INVALID, want[:, 2] != INVALID)
    ties = tie_only_mismatch(orc, rays, got, want, v, i, near_ulp=near_ulp)
    same = got[:, 3] == want[:, 3]
    hit = want[:, 2] != INVALID
    assert np.array_equal(got[same & hit], want[same & hit])
    return ties


@pytest.mark.parametrize("name", MESH_FIXTURES)
def test_bvh4q8_on_fixtures(ctx, orc, name):
    g = golden(name)
    res = build(ctx, g["vertices"], g["indices"], node_format=Q8_FORMAT)
    n = g["indices"].shape[0]
    if n > 1:
        check_conservative(res, g["vertices"], g["indices"].reshape(-1, 3))
    got = trace(ctx, res, g["rays"], query=0, output=0, traversal=BVH4)
    compare(orc, g["rays"], got, g["hits_q0_o0"], g["vertices"], g["indices"])
    anyh = trace(ctx, res, g["rays"], query=1, output=0, traversal=BVH4)
    assert np.array_equal(anyh[:, 2] != INVALID, g["hits_q1_o0"][:, 2] != INVALID)
    auto = trace(ctx, res, g["rays"], query=0, output=0, traversal=0)  # AUTO runs the 4-wide kernel here
    assert np.array_equal(auto, got)
    assert ctx.device_errors() == 0


def test_bvh4q8_soup_heightfield_quality_and_update(ctx, orc):
    from gpu_util import to_dev
    from radeonrays_sdk_gb300 import scenes
    v, i, rays = scenes.config0()
    res = build(ctx, v, i, node_format=Q8_FORMAT)
    check_conservative(res, v, i)
    nodes, _, _ = orc.build_mesh(v, i)
    compare(orc, rays, trace(ctx, res, rays, traversal=BVH4), orc.trace(nodes, rays, threads=16), v, i)
    v, i, rays = scenes.config1(grid=257, nrays=1 << 18)
    for quality in (False, True):
        res = ctx.build_geometry(to_dev(v), to_dev(i), node_format=Q8_FORMAT, quality=quality)
        check_conservative(res, v, i)
        qn = nodes_of(res, i.shape[0])  # the reference's order on the same (possibly restructured) tree
        want = orc.trace(qn, rays, threads=16)
        compare(orc, rays, trace(ctx, res, rays, traversal=BVH4), want, v, i)
        anyr = rays.copy()
        anyr[:, 7] = np.float32(0.05)
        wa = orc.trace(qn, anyr, query=1, threads=16)
        assert np.array_equal(trace(ctx, res, anyr, query=1, traversal=BVH4)[:, 2] != INVALID, wa[:, 2] != INVALID)
    # An update re-collapses the quantised nodes over the moved vertices.
    v2 = (v * np.float32(1.02)).astype(np.float32)
    ctx.update_geometry(to_dev(v2), to_dev(i), res)
    check_conservative(res, v2, i)
    want = orc.trace(orc.fit(nodes_of(res, i.shape[0]), v2, i), rays, threads=16)
    compare(orc, rays, trace(ctx, res, rays, traversal=BVH4), want, v2, i)
    assert ctx.device_errors() == 0


def test_bvh4q8_precise_mode(ctx, orc):
    """With the precise test the 4-wide kernel decodes each quantised plane
    with outward rounding and runs the robust box test, so no box the exact
    ray segment touches is culled: hits equal the oracle twin's (binary
    nodes, reference order) except exact equal-t ties, and the persistent
    binary kernel over the same buffer is bit-identical to the twin."""
    from gpu_util import hits_np, to_dev
    from radeonrays_sdk_gb300 import scenes
    v, i, rays = scenes.config1(grid=129, nrays=1 << 16)
    res = build(ctx, v, i, node_format=Q8_FORMAT)
    nodes, _, _ = orc.build_mesh(v, i)
    want, _ = orc.trace_precise(nodes, rays, threads=16)
    got = {}
    for trav in (0, 3, 4):
        ctx.set_traversal(trav, triangle_test=1)
        got[trav] = hits_np(ctx.intersect(res, to_dev(rays)))
        ctx.set_traversal(0)
    assert np.array_equal(got[3], want)
    assert np.array_equal(got[0], got[4])  # AUTO runs the 4-wide kernel
    assert np.array_equal(got[4][:, 2] != INVALID, want[:, 2] != INVALID)
    tie_only_mismatch(orc, rays, got[4], want, v, i, precise=True)
    same = got[4][:, 3] == want[:, 3]
    assert np.array_equal(got[4][same], want[same])
    # Any hit: the same occlusion flags.
    occl = rays.copy()
    occl[:, 7] = np.float32(0.05)
    wa, _ = orc.trace_precise(nodes, occl, query=1, threads=16)
    ctx.set_traversal(4, triangle_test=1)
    ga = hits_np(ctx.intersect(res, to_dev(occl), query=1))
    ctx.set_traversal(0)
    assert np.array_equal(ga[:, 2] != INVALID, wa[:, 2] != INVALID)
    assert ctx.device_errors() == 0


def test_default_build_is_bvh4q8_and_auto_runs_the_4wide_kernel(ctx, orc):
    """A build with null RRBuildOptions (what a drop-in client passes) makes
    8-bit 4-wide nodes, and the default traversal option runs the 4-wide
    kernel on them: hit flags are the reference's."""
    import ctypes as C
    import torch
    from gpu_util import to_dev
    from radeonrays_sdk_gb300 import rr, scenes
    v, i, rays = scenes.config1(grid=129, nrays=1 << 15)
    n = i.shape[0]
    vd, idd = to_dev(v), to_dev(i)
    bi, mesh = ctx._build_input(ctx.ptr(vd), v.shape[0], 12, ctx.ptr(idd), n, False)
    req = rr.RRMemoryRequirements()
    rr.check(ctx.L.rrGetGeometryBuildMemoryRequirements(ctx.ctx, C.byref(bi), None, C.byref(req)), "requirements")
    assert req.result_buffer_size == ctx.geometry_requirements(n, rr.RR_CUDA_NODE_FORMAT_BVH4Q8, 30, v.shape[0], 12)[1]
    scratch = torch.empty(req.temporary_build_buffer_size, dtype=torch.uint8, device="cuda")
    res = torch.empty(req.result_buffer_size, dtype=torch.uint8, device="cuda")
    cs = ctx.command_stream()
    rr.check(ctx.L.rrCmdBuildGeometry(ctx.ctx, rr.RR_BUILD_OPERATION_BUILD, C.byref(bi), None, ctx.ptr(scratch),
                                      ctx.ptr(res), cs), "rrCmdBuildGeometry")
    ctx.submit(cs)
    ctx.release_stream(cs)
    assert trailer_of(res, n)["node_format"] == Q8_FORMAT
    check_conservative(res, v, i)
    nodes, _, _ = orc.build_mesh(v, i)
    want = orc.trace(nodes, rays, threads=16)
    got = trace(ctx, res, rays, traversal=0)
    assert np.array_equal(got, trace(ctx, res, rays, traversal=BVH4))
    compare(orc, rays, got, want, v, i)
    assert ctx.device_errors() == 0
