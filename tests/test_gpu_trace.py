"""GPU traversal parity through rrCmdIntersect.

Plain (binary) kernel: bit-identical RRHit records to the oracle for every
query/output variant.  Wide (chosen) kernel: closest-hit primitive ids equal
the plain path's except exact equal-t ties; uv bit-identical wherever the
primitive is the same; hit/miss flags identical for closest and any hit."""
import ctypes as C

import numpy as np
import pytest

from conftest import MESH_FIXTURES, golden
from gpu_util import INVALID, build, tie_only_mismatch, to_dev, trace

pytestmark = pytest.mark.gpu

BINARY, WIDE, PERSISTENT = 1, 2, 3


@pytest.mark.parametrize("name", MESH_FIXTURES)
@pytest.mark.parametrize("trav", [BINARY, PERSISTENT])
def test_binary_trace_bit_exact_on_fixtures(ctx, orc, name, trav):
    """Both binary-node kernels (one thread per ray, and persistent refill)
    visit nodes in the reference order: bit-identical records."""
    g = golden(name)
    res = build(ctx, g["vertices"], g["indices"], node_format=1)
    for q in (0, 1):
        for o in (0, 1):
            got = trace(ctx, res, g["rays"], query=q, output=o, traversal=trav)
            assert np.array_equal(got, g[f"hits_q{q}_o{o}"]), (q, o)
    assert ctx.device_errors() == 0


@pytest.mark.parametrize("name", MESH_FIXTURES)
def test_wide_trace_matches_plain_on_fixtures(ctx, orc, name):
    g = golden(name)
    res = build(ctx, g["vertices"], g["indices"], node_format=1)
    plain = g["hits_q0_o0"]
    wide = trace(ctx, res, g["rays"], query=0, output=0, traversal=WIDE)
    assert np.array_equal(wide[:, 2] != INVALID, plain[:, 2] != INVALID)
    tie_only_mismatch(orc, g["rays"], wide, plain, g["vertices"], g["indices"])
    same = wide[:, 3] == plain[:, 3]
    assert np.array_equal(wide[same], plain[same])
    anyw = trace(ctx, res, g["rays"], query=1, output=0, traversal=WIDE)
    assert np.array_equal(anyw[:, 2] != INVALID, g["hits_q1_o0"][:, 2] != INVALID)
    inst = trace(ctx, res, g["rays"], query=0, output=1, traversal=WIDE)
    assert np.array_equal(inst, wide[:, 3] * (wide[:, 2] != INVALID) + INVALID * (wide[:, 2] == INVALID))
    assert ctx.device_errors() == 0


def test_config0_plain_and_wide(ctx, orc):
    """65,536-triangle soup, 1024 x 1024 primary rays (full config)."""
    from radeonrays_sdk_gb300 import scenes
    v, i, rays = scenes.config0()
    res = build(ctx, v, i, node_format=1)
    nodes, _, _ = orc.build_mesh(v, i)
    want = orc.trace(nodes, rays, threads=16)
    plain = trace(ctx, res, rays, traversal=BINARY)
    assert np.array_equal(plain, want)
    assert np.array_equal(trace(ctx, res, rays, traversal=PERSISTENT), want)
    wide = trace(ctx, res, rays, traversal=WIDE)
    assert np.array_equal(wide[:, 2] != INVALID, want[:, 2] != INVALID)
    ties = tie_only_mismatch(orc, rays, wide, want, v, i)
    assert ties <= 16
    same = wide[:, 3] == want[:, 3]
    assert np.array_equal(wide[same], want[same])


def test_heightfield_incoherent_plain_and_wide(ctx, orc):
    from radeonrays_sdk_gb300 import scenes
    v, i, rays = scenes.config1(grid=257, nrays=1 << 18)
    res = build(ctx, v, i, node_format=1)
    nodes, _, _ = orc.build_mesh(v, i)
    for q in (0, 1):
        want = orc.trace(nodes, rays, query=q, threads=16)
        assert np.array_equal(trace(ctx, res, rays, query=q, traversal=BINARY), want)
        assert np.array_equal(trace(ctx, res, rays, query=q, traversal=PERSISTENT), want)
    want = orc.trace(nodes, rays, threads=16)
    wide = trace(ctx, res, rays, traversal=WIDE)
    assert np.array_equal(wide[:, 2] != INVALID, want[:, 2] != INVALID)
    tie_only_mismatch(orc, rays, wide, want, v, i)
    assert ctx.device_errors() == 0


def test_any_hit_occlusion_rays(ctx, orc):
    """Config-1 style any-hit: tmax ~ U[0.01, 0.5]."""
    from radeonrays_sdk_gb300 import scenes
    v, i, rays = scenes.config1(grid=129, nrays=1 << 16, any_hit=True)
    res = build(ctx, v, i, node_format=1)
    nodes, _, _ = orc.build_mesh(v, i)
    want = orc.trace(nodes, rays, query=1, output=1)
    assert np.array_equal(trace(ctx, res, rays, query=1, output=1, traversal=BINARY), want)
    wide = trace(ctx, res, rays, query=1, output=1, traversal=WIDE)
    assert np.array_equal(wide != INVALID, want != INVALID)


def test_miss_writes_only_inst_id_and_indirect_count(ctx, orc):
    import torch
    g = golden("height17")
    res = build(ctx, g["vertices"], g["indices"])
    rays = to_dev(g["rays"])
    R = rays.shape[0]
    want = g["hits_q0_o0"]
    for trav in (BINARY, WIDE):
        ctx.set_traversal(trav)
        hits = torch.full((R, 4), 0x11223344, dtype=torch.int32, device="cuda")
        ctx.intersect(res, rays, hits=hits)
        h = hits.cpu().numpy().view(np.uint32)
        miss = want[:, 2] == INVALID
        assert np.all(h[miss, 2] == INVALID) and np.all(h[miss][:, [0, 1, 3]] == 0x11223344)
        # indirect count: only the first k rays are traced
        k = 777
        hits = torch.full((R, 4), 0x11223344, dtype=torch.int32, device="cuda")
        cnt = torch.tensor([k], dtype=torch.int32, device="cuda")
        ctx.intersect(res, rays, hits=hits, indirect=cnt)
        h = hits.cpu().numpy().view(np.uint32)
        assert np.all(h[k:] == 0x11223344)
        assert np.array_equal(h[:k, 2] != INVALID, want[:k, 2] != INVALID)
    ctx.set_traversal(0)


def test_command_stream_replay_and_external_stream(ctx, orc):
    """A recorded command stream replays (as a CUDA graph) with the same
    result; an external CUDA stream enqueues immediately."""
    import torch
    from radeonrays_sdk_gb300 import rr
    g = golden("soup256")
    res = build(ctx, g["vertices"], g["indices"])
    rays = to_dev(g["rays"])
    R = rays.shape[0]
    hits = torch.zeros((R, 4), dtype=torch.int32, device="cuda")
    scratch = torch.empty(ctx.trace_scratch_bytes(R), dtype=torch.uint8, device="cuda")
    cs = ctx.command_stream()
    ctx.cmd_intersect(res, rays, R, hits, scratch, cs)
    ctx.cmd_intersect(res, rays, R, hits, scratch, cs)  # two ops -> captured as a graph
    ctx.submit(cs)
    first = hits.cpu().numpy().copy()
    hits.zero_()
    ctx.submit(cs)
    assert np.array_equal(hits.cpu().numpy(), first)
    ctx.release_stream(cs)
    s = torch.cuda.Stream()
    ext = ctx.external_stream(s)
    hits2 = torch.zeros_like(hits)
    ctx.cmd_intersect(res, rays, R, hits2, scratch, ext)
    s.synchronize()
    assert np.array_equal(hits2.cpu().numpy(), first)
    assert ctx.L.rrReleaseExternalCommandStream(ctx.ctx, ext) == rr.RR_SUCCESS


def test_wait_event_timeout_is_bounded(ctx):
    """rrWaitEvent gives up after the configured timeout instead of waiting
    forever (reference vlk/device.cpp:249-272 waits forever); a later wait
    with the default timeout completes."""
    import torch
    from radeonrays_sdk_gb300 import rr, scenes
    v, i, rays = scenes.config1(grid=513, nrays=1 << 22)
    res = build(ctx, v, i)
    rays_d = to_dev(rays)
    R = rays.shape[0]
    hits = torch.empty((R, 4), dtype=torch.int32, device="cuda")
    scratch = torch.empty(ctx.trace_scratch_bytes(R), dtype=torch.uint8, device="cuda")
    cs = ctx.command_stream()
    for _ in range(16):  # tens of milliseconds of queued work against a 0 ms limit
        ctx.cmd_intersect(res, rays_d, R, hits, scratch, cs)
    ev = ctx.submit(cs, wait=False)
    assert ctx.L.rrCudaSetWaitTimeout(ctx.ctx, 0) == rr.RR_SUCCESS
    first = ctx.L.rrWaitEvent(ctx.ctx, ev)
    assert ctx.L.rrCudaSetWaitTimeout(ctx.ctx, 600000) == rr.RR_SUCCESS
    assert ctx.L.rrWaitEvent(ctx.ctx, ev) == rr.RR_SUCCESS
    assert first == rr.RR_ERROR_INTERNAL
    ctx.L.rrReleaseEvent(ctx.ctx, ev)
    ctx.release_stream(cs)


def test_argument_errors_with_context(ctx):
    from radeonrays_sdk_gb300 import rr
    L = ctx.L
    mesh = rr.RRTriangleMeshPrimitive(None, 0, 12, None, 10, rr.RR_INDEX_TYPE_UINT32)
    bi = rr.RRGeometryBuildInput(7, 1, C.pointer(mesh))  # no such primitive type
    cs = ctx.command_stream()
    fake = C.c_void_p(0x1000)
    assert L.rrCmdBuildGeometry(ctx.ctx, 1, C.byref(bi), None, fake, fake, cs) == rr.RR_ERROR_NOT_IMPLEMENTED
    boxes = rr.RRAABBListPrimitive(None, 10, 12)  # box stride below 32 bytes
    bi = rr.RRGeometryBuildInput(rr.RR_PRIMITIVE_TYPE_AABB_LIST, 1,
                                 C.cast(C.pointer(boxes), C.POINTER(rr.RRTriangleMeshPrimitive)))
    assert L.rrCmdBuildGeometry(ctx.ctx, 1, C.byref(bi), None, fake, fake, cs) == rr.RR_ERROR_INVALID_PARAMETER
    bi = rr.RRGeometryBuildInput(rr.RR_PRIMITIVE_TYPE_TRIANGLE_MESH, 1, C.pointer(mesh))
    assert L.rrCmdBuildGeometry(ctx.ctx, 1, C.byref(bi), None, fake, fake, cs) == rr.RR_ERROR_INVALID_PARAMETER
    assert L.rrCmdBuildGeometry(ctx.ctx, rr.RR_BUILD_OPERATION_UPDATE, C.byref(bi), None, fake, fake, cs) in (
        rr.RR_ERROR_NOT_IMPLEMENTED, rr.RR_ERROR_INVALID_PARAMETER)
    bad_opts = rr.RRCudaBuildOptions(4, 7, 30, 0)
    o = rr.RRBuildOptions(0, C.cast(C.pointer(bad_opts), C.c_void_p))
    req = rr.RRMemoryRequirements()
    assert L.rrGetGeometryBuildMemoryRequirements(ctx.ctx, C.byref(bi), C.byref(o), C.byref(req)) == \
        rr.RR_ERROR_INVALID_PARAMETER
    assert L.rrCmdIntersect(ctx.ctx, fake, 5, fake, 1, None, 0, fake, fake, cs) == rr.RR_ERROR_INVALID_PARAMETER
    ctx.release_stream(cs)


def test_autotuner_selects_a_kernel_and_results_stay_exact(ctx, orc, tmp_path, monkeypatch):
    """rrCudaAutotuneTraversal times the candidate kernels, sets the fastest on
    the context and caches it; the tuned path keeps the parity bar."""
    from radeonrays_sdk_gb300 import scenes
    monkeypatch.setenv("RR_CUDA_TUNE_CACHE", str(tmp_path / "tune.tsv"))
    v, i, rays = scenes.config1(grid=257, nrays=1 << 18)
    res = build(ctx, v, i, node_format=1)
    rays_d = to_dev(rays)
    choice = ctx.autotune(res, rays_d)
    assert choice["traversal"] in (BINARY, WIDE, PERSISTENT)  # a WIDE8 buffer: no 4-wide candidate
    assert (tmp_path / "tune.tsv").exists()
    nodes, _, _ = orc.build_mesh(v, i)
    want = orc.trace(nodes, rays, threads=16)
    got = hits_np_of(ctx.intersect(res, rays_d))
    assert np.array_equal(got[:, 2] != INVALID, want[:, 2] != INVALID)
    tie_only_mismatch(orc, rays, got, want, v, i)
    assert ctx.autotune(res, rays_d) == choice  # served from the cache
    ctx.set_traversal(0)


def hits_np_of(t):
    return t.cpu().numpy().view(np.uint32)
