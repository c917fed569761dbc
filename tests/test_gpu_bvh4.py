"""GPU tests of the 4-wide fp32 format (RR_CUDA_NODE_FORMAT_BVH4) and its
traversal (RR_CUDA_TRAVERSAL_BVH4) against the oracle's plain traversal.

The 4-wide nodes keep exact child boxes and the reference's slab and
triangle arithmetic, but visit children nearest first: hit/miss flags equal
the reference's for closest and any hit, closest-hit primitives equal it
except exact equal-t ties, and uv is bit-identical wherever the primitive is
the same.  (The binary nodes of a BVH4 buffer are compared with the oracle's
in test_gpu_build.py.)"""
import numpy as np
import pytest

from conftest import MESH_FIXTURES, golden
from gpu_util import INVALID, build, hits_np, nodes_of, tie_only_mismatch, to_dev, trace, trailer_of

pytestmark = pytest.mark.gpu

BVH4_FORMAT, BVH4 = 2, 4


def bvh4_nodes(res, n):
    tr = trailer_of(res, n)
    raw = res.cpu().numpy()
    off, cnt = int(tr["wide_nodes_off"]), int(tr["wide_count"])
    a = raw[off: off + 128 * cnt].view(np.uint32).reshape(cnt, 32)
    lo = a[:, 0:12].view(np.float32).reshape(cnt, 3, 4)
    hi = a[:, 12:24].view(np.float32).reshape(cnt, 3, 4)
    return lo, hi, a[:, 24:28]


def check_structure(res, v, i):
    """Every binary leaf is referenced once; every 4-wide node but the root
    once; every child box contains its subtree's triangles exactly (the
    leaf boxes are the triangles' boxes)."""
    n = i.shape[0]
    lo, hi, ch = bvh4_nodes(res, n)
    leaves = ch[(ch != INVALID) & (ch >= 0x80000000)] & 0x7FFFFFFF
    assert np.array_equal(np.sort(leaves), np.arange(n - 1, 2 * n - 1))
    inner = ch[(ch != INVALID) & (ch < 0x80000000)]
    assert np.array_equal(np.sort(inner), np.arange(1, lo.shape[0]))
    nodes = nodes_of(res, n)
    tri = v[i.astype(np.int64)]  # (n, 3, 3)
    prim = nodes["child1"][n - 1:]  # binary leaf -> primitive
    k, s = np.nonzero((ch != INVALID) & (ch >= 0x80000000))
    t = tri[prim[(ch[k, s] & 0x7FFFFFFF).astype(np.int64) - (n - 1)]]
    assert np.array_equal(lo[k, :, s], t.min(axis=1)) and np.array_equal(hi[k, :, s], t.max(axis=1))


def compare(orc, rays, got, want, v, i):
    assert np.array_equal(got[:, 2] != INVALID, want[:, 2] != INVALID)
    ties = tie_only_mismatch(orc, rays, got, want, v, i)
    same = got[:, 3] == want[:, 3]
    hit = want[:, 2] != INVALID
    assert np.array_equal(got[same & hit], want[same & hit])
    return ties


@pytest.mark.parametrize("name", MESH_FIXTURES)
def test_bvh4_on_fixtures(ctx, orc, name):
    g = golden(name)
    res = build(ctx, g["vertices"], g["indices"], node_format=BVH4_FORMAT)
    n = g["indices"].shape[0]
    if n > 1:
        check_structure(res, g["vertices"], g["indices"].reshape(-1, 3))
    got = trace(ctx, res, g["rays"], query=0, output=0, traversal=BVH4)
    compare(orc, g["rays"], got, g["hits_q0_o0"], g["vertices"], g["indices"])
    anyh = trace(ctx, res, g["rays"], query=1, output=0, traversal=BVH4)
    assert np.array_equal(anyh[:, 2] != INVALID, g["hits_q1_o0"][:, 2] != INVALID)
    inst = trace(ctx, res, g["rays"], query=0, output=1, traversal=BVH4)
    assert np.array_equal(inst, got[:, 3] * (got[:, 2] != INVALID) + INVALID * (got[:, 2] == INVALID))
    assert ctx.device_errors() == 0


def test_bvh4_soup_pinhole_and_heightfield(ctx, orc):
    from radeonrays_sdk_gb300 import scenes
    v, i, rays = scenes.config0()
    res = build(ctx, v, i, node_format=BVH4_FORMAT)
    check_structure(res, v, i)
    nodes, _, _ = orc.build_mesh(v, i)
    want = orc.trace(nodes, rays, threads=16)
    assert compare(orc, rays, trace(ctx, res, rays, traversal=BVH4), want, v, i) <= 16
    v, i, rays = scenes.config1(grid=257, nrays=1 << 18)
    res = build(ctx, v, i, node_format=BVH4_FORMAT)
    check_structure(res, v, i)
    nodes, _, _ = orc.build_mesh(v, i)
    want = orc.trace(nodes, rays, threads=16)
    compare(orc, rays, trace(ctx, res, rays, traversal=BVH4), want, v, i)
    anyr = rays.copy()
    anyr[:, 7] = np.float32(0.05)
    want = orc.trace(nodes, anyr, query=1, threads=16)
    got = trace(ctx, res, anyr, query=1, traversal=BVH4)
    assert np.array_equal(got[:, 2] != INVALID, want[:, 2] != INVALID)
    assert ctx.device_errors() == 0


def test_bvh4_quality_build_and_autotuner(ctx, orc):
    """The restructured (quality) tree collapses the same way; the autotuner
    includes the 4-wide kernel for BVH4 buffers, and whatever it picks keeps
    the hits."""
    from gpu_util import to_dev
    from radeonrays_sdk_gb300 import scenes
    v, i, rays = scenes.config1(grid=257, nrays=1 << 18)
    res = ctx.build_geometry(to_dev(v), to_dev(i), node_format=BVH4_FORMAT, quality=True)
    check_structure(res, v, i)
    plain = trace(ctx, res, rays, traversal=1)
    got = trace(ctx, res, rays, traversal=BVH4)
    compare(orc, rays, got, plain, v, i)
    rd = to_dev(rays)
    tuned = ctx.autotune(res, rd)
    assert tuned["traversal"] in (1, 3, 4)
    assert tuned["blocks_per_sm"] in (0, 4, 6) and tuned["short_stack"] in (0, 12, 24)
    h = ctx.intersect(res, rd).cpu().numpy().view(np.uint32)
    compare(orc, rays, h, plain, v, i)
    ctx.set_traversal(0)
    assert ctx.device_errors() == 0


def test_bvh4_deep_stacks_spill_and_refill(ctx, orc):
    """30,000 triangles crowded into a 0.02-wide cube: every box along a ray
    is hit, so the 16-entry short stack spills to the scratch and refills
    many times per ray.  Hits must still equal the plain traversal's."""
    from radeonrays_sdk_gb300 import scenes
    g = scenes.rng(63)
    c = np.float32(0.5) + (g.random((30000, 1, 3), dtype=np.float32) - np.float32(0.5)) * np.float32(0.02)
    v = (c + (g.random((30000, 3, 3), dtype=np.float32) - np.float32(0.5)) * np.float32(0.01)).reshape(-1, 3)
    i = np.arange(90000, dtype=np.uint32).reshape(-1, 3)
    rays = scenes.incoherent_rays(20000, (0.49, 0.49, 0.49), (0.51, 0.51, 0.51), scenes.rng(63, 1))
    res = build(ctx, v, i, node_format=BVH4_FORMAT)
    check_structure(res, v, i)
    nodes, _, _ = orc.build_mesh(v, i)
    want = orc.trace(nodes, rays, threads=16)
    compare(orc, rays, trace(ctx, res, rays, traversal=BVH4), want, v, i)
    anyw = orc.trace(nodes, rays, query=1, threads=16)
    got = trace(ctx, res, rays, query=1, traversal=BVH4)
    assert np.array_equal(got[:, 2] != INVALID, anyw[:, 2] != INVALID)
    assert ctx.device_errors() == 0


def test_bvh4_stack_depth_and_launch_shape_keep_hits(ctx, orc):
    """The short-stack depth (12..32 entries) and the resident blocks per SM
    are launch parameters the autotuner picks: they change where entries
    live and how rays are spread over the SMs, never the visit order, so
    hits are bit-identical to the default launch on the deep-stack mesh
    (which spills at every depth).  Depths outside 12..32 are rejected."""
    from gpu_util import to_dev
    from radeonrays_sdk_gb300 import rr, scenes
    g = scenes.rng(64)
    c = np.float32(0.5) + (g.random((20000, 1, 3), dtype=np.float32) - np.float32(0.5)) * np.float32(0.02)
    v = (c + (g.random((20000, 3, 3), dtype=np.float32) - np.float32(0.5)) * np.float32(0.01)).reshape(-1, 3)
    i = np.arange(60000, dtype=np.uint32).reshape(-1, 3)
    rays = scenes.incoherent_rays(20000, (0.49, 0.49, 0.49), (0.51, 0.51, 0.51), scenes.rng(64, 1))
    res = build(ctx, v, i, node_format=BVH4_FORMAT)
    rd = to_dev(rays)
    for query in (0, 1):
        base = trace(ctx, res, rays, query=query, traversal=BVH4)
        for bps, depth in ((0, 12), (0, 24), (0, 32), (4, 0), (6, 20)):
            ctx.set_traversal(BVH4, 0, bps, short_stack=depth)
            got = ctx.intersect(res, rd, query=query).cpu().numpy().view(np.uint32)
            ctx.set_traversal(0)
            assert np.array_equal(got, base), (query, bps, depth)
    nodes, _, _ = orc.build_mesh(v, i)
    compare(orc, rays, trace(ctx, res, rays, traversal=BVH4), orc.trace(nodes, rays, threads=16), v, i)
    for bad in (1, 11, 33, 64):
        with pytest.raises(rr.RRException):
            ctx.set_traversal(BVH4, short_stack=bad)
    ctx.set_traversal(0)
    assert ctx.device_errors() == 0


def test_node_format_autotuner_and_auto_builds(ctx, orc, tmp_path, monkeypatch):
    """rrCudaAutotuneNodeFormat builds the mesh in the three wide formats, tunes the
    traversal of each, and remembers the faster width for the mesh's size
    class; builds with RR_CUDA_NODE_FORMAT_AUTO then use it, from the context
    and, through RR_CUDA_TUNE_CACHE, in a fresh one."""
    from radeonrays_sdk_gb300 import rr, scenes
    monkeypatch.setenv("RR_CUDA_TUNE_CACHE", str(tmp_path / "tune.tsv"))
    v, i, rays = scenes.config1(grid=257, nrays=1 << 18)
    with rr.Context() as c:
        fmt = c.autotune_node_format(to_dev(v), to_dev(i), to_dev(rays))
        assert fmt in (rr.RR_CUDA_NODE_FORMAT_BVH4, rr.RR_CUDA_NODE_FORMAT_BVH4Q8, rr.RR_CUDA_NODE_FORMAT_WIDE8)
        res = c.build_geometry(to_dev(v), to_dev(i), node_format=rr.RR_CUDA_NODE_FORMAT_AUTO)
        assert trailer_of(res, i.shape[0])["node_format"] == fmt
        nodes, _, _ = orc.build_mesh(v, i)
        want = orc.trace(nodes, rays, threads=16)
        got = hits_np(c.intersect(res, to_dev(rays)))
        assert np.array_equal(got[:, 2] != INVALID, want[:, 2] != INVALID)
        assert c.device_errors() == 0
    assert "fmt|" in (tmp_path / "tune.tsv").read_text()
    with rr.Context() as c2:  # a fresh context reads the choice from the cache file
        res2 = c2.build_geometry(to_dev(v), to_dev(i), node_format=rr.RR_CUDA_NODE_FORMAT_AUTO)
        assert trailer_of(res2, i.shape[0])["node_format"] == fmt
