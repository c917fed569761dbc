"""GPU fused multi-geometry build (rrCudaCmdBuildGeometries, and consecutive
rrCmdBuildGeometry calls fused inside one command stream): every geometry's
binary nodes bit-identical to the oracle's build of it alone, wide trees that
trace like separately built ones, overlap handling, and a scene over fused
BLASes against the oracle's two-level traversal."""
import ctypes as C

import numpy as np
import pytest

from gpu_util import INVALID, hits_np, nodes_of, to_dev, trailer_of
from test_gpu_build import same_nodes

pytestmark = pytest.mark.gpu

# Uneven sizes around the sort tile (4,096 keys) and the chunk (256) edges.
SIZES = [0, 1, 2, 3, 7, 64, 255, 256, 257, 1000, 4095, 4096, 4097, 20000, 70001]


def meshes_for(sizes, seed):
    from radeonrays_sdk_gb300 import scenes
    out = []
    for k, n in enumerate(sizes):
        if n == 0:
            out.append((np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32)))
        else:
            out.append(scenes.soup(n, scenes.rng(40 + seed, k)))
    return out


def dev_meshes(ms):
    return [(to_dev(v), to_dev(i)) for v, i in ms]


def ord_bounds(v, i):
    """Mesh box of the referenced vertices in the order-preserving uint
    encoding of the trailer: [lo.x, lo.y, lo.z, 0, hi.x, hi.y, hi.z, 0]."""
    vv = v[i.reshape(-1).astype(np.int64)]

    def enc(f):
        u = np.asarray(f, np.float32).view(np.uint32).astype(np.uint64)
        return ((u ^ (((0x100000000 - (u >> 31)) & 0xFFFFFFFF) | 0x80000000)) & 0xFFFFFFFF).astype(np.uint32)

    e = enc(vv)
    out = np.zeros(8, np.uint32)
    out[0:3] = e.min(axis=0)
    out[4:7] = e.max(axis=0)
    return out


@pytest.mark.parametrize("api", ["batch", "record"])
@pytest.mark.parametrize("fmt", [0, 1])
def test_fused_build_matches_oracle(ctx, orc, api, fmt):
    ms = meshes_for(SIZES, 0)
    res = ctx.build_geometries(dev_meshes(ms), node_format=fmt, api=api)
    assert ctx.device_errors() == 0
    for (v, i), r in zip(ms, res):
        n = i.shape[0]
        tr = trailer_of(r, n)
        assert tr["magic"] == 0x52524742 and tr["leaf_count"] == n and tr["node_format"] == fmt
        if n == 0:
            continue
        nodes, _, _ = orc.build_mesh(v, i)
        assert same_nodes(nodes_of(r, n), nodes), n
        assert np.array_equal(tr["bounds"], ord_bounds(v, i)), n
        if fmt == 1:
            assert tr["wide_count"] >= 1 and tr["wide_tri_count"] == n


def test_fused_build_63bit(ctx, orc):
    ms = meshes_for([5, 3000, 9000], 1)
    res = ctx.build_geometries(dev_meshes(ms), node_format=0, morton_bits=63)
    for (v, i), r in zip(ms, res):
        nodes, _, _ = orc.build_mesh(v, i, bits=63)
        assert same_nodes(nodes_of(r, i.shape[0]), nodes)


def test_fused_equals_separate_and_traces_alike(ctx, orc):
    """Log-uniform sizes (a scaled copy of the 2,048-BLAS workload): fused and
    one-by-one builds give the same binary nodes and the same wide-path hits."""
    from radeonrays_sdk_gb300 import scenes
    g = scenes.rng(41)
    sizes = np.rint(np.exp(g.uniform(np.log(64), np.log(16384), size=96))).astype(int).tolist()
    ms = meshes_for(sizes, 2)
    dm = dev_meshes(ms)
    fused = ctx.build_geometries(dm, node_format=1, api="batch")
    sep = ctx.build_geometries(dm, node_format=1, api="separate")
    rays = scenes.incoherent_rays(4096, (0, 0, 0), (1, 1, 1), scenes.rng(41, 1))
    rd = to_dev(rays)
    for k in range(0, len(ms), 7):
        v, i = ms[k]
        n = i.shape[0]
        assert np.array_equal(nodes_of(fused[k], n).view(np.uint32), nodes_of(sep[k], n).view(np.uint32))
        a = hits_np(ctx.intersect(fused[k], rd))
        b = hits_np(ctx.intersect(sep[k], rd))
        assert np.array_equal(a, b), k
        want = orc.trace(orc.build_mesh(v, i)[0], rays)
        assert np.array_equal(a[:, 2] != INVALID, want[:, 2] != INVALID)
    assert ctx.device_errors() == 0


def test_record_with_shared_scratch_is_not_fused_wrongly(ctx, orc):
    """Builds recorded into one command stream that share a scratch buffer
    must still each be correct (the fusion splits at the shared buffer)."""
    import torch
    ms = meshes_for([3000, 5000, 70], 3)
    s_max = max(ctx.geometry_requirements(i.shape[0])[0] for _, i in ms)
    shared = torch.empty(s_max, dtype=torch.uint8, device="cuda")
    # Recorded builds read their inputs at submission: keep them alive until then.
    dm = dev_meshes(ms)
    cs = ctx.command_stream()
    res = [ctx.build_geometry(v, i, node_format=1, stream=cs, scratch=shared) for v, i in dm]
    ctx.submit(cs)
    ctx.release_stream(cs)
    for (v, i), r in zip(ms, res):
        assert same_nodes(nodes_of(r, i.shape[0]), orc.build_mesh(v, i)[0])


def test_batch_rejects_overlapping_buffers(ctx):
    import torch
    from radeonrays_sdk_gb300 import rr
    ms = meshes_for([100, 200], 4)
    dm = dev_meshes(ms)
    opts, keep = ctx._options(1, 30)
    reqs = [ctx.geometry_requirements(i.shape[0]) for _, i in ms]
    scratch = torch.empty(max(s for s, _ in reqs), dtype=torch.uint8, device="cuda")
    results = [torch.empty(r, dtype=torch.uint8, device="cuda") for _, r in reqs]
    inputs = [ctx._build_input(ctx.ptr(v), v.shape[0], 12, ctx.ptr(i), i.shape[0], False) for v, i in dm]
    arr = (rr.RRGeometryBuildInput * 2)(*[b for b, _ in inputs])
    sp = (C.c_void_p * 2)(ctx.ptr(scratch).value, ctx.ptr(scratch).value)
    rp = (C.c_void_p * 2)(ctx.ptr(results[0]).value, ctx.ptr(results[1]).value)
    cs = ctx.command_stream()
    code = ctx.L.rrCudaCmdBuildGeometries(ctx.ctx, 2, arr, C.byref(opts), sp, rp, cs)
    ctx.release_stream(cs)
    assert code == rr.RR_ERROR_INVALID_PARAMETER


def test_scene_over_fused_blas(ctx, orc):
    from radeonrays_sdk_gb300 import scenes
    blas_np, M, rays = scenes.config2(n_blas=24, lo_tris=16, hi_tris=3000, nrays=20000)
    fused = ctx.build_geometries(dev_meshes(blas_np), node_format=1)
    scene = ctx.build_scene(fused, M)
    onodes = [orc.build_mesh(v, i)[0] for v, i in blas_np]
    tlas, xf = orc.build_scene(onodes, [i.shape[0] for _, i in blas_np], M)
    want = orc.trace_scene(tlas, xf, onodes, rays)
    ctx.set_traversal(1)
    plain = hits_np(ctx.intersect(scene, to_dev(rays)))
    ctx.set_traversal(0)
    assert np.array_equal(plain, want)
    chosen = hits_np(ctx.intersect(scene, to_dev(rays)))
    assert np.array_equal(chosen[:, 2] != INVALID, want[:, 2] != INVALID)
    assert ctx.device_errors() == 0
