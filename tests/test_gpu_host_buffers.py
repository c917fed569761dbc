"""GPU host-buffer tracing (rrCudaCmdIntersectHostBuffers): chunks pipelined
over the context's side streams give exactly the hits of rrCmdIntersect on
device buffers, for every chunking, query and output."""
import numpy as np
import pytest

from gpu_util import INVALID, hits_np, to_dev

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,chunk", [(100, 0), (30000, 0), (70000, 5000), (70001, 4096), (200000, 0)])
@pytest.mark.parametrize("q,o", [(0, 0), (1, 0), (0, 1)])
def test_host_buffers_equal_device_trace(ctx, orc, n, chunk, q, o):
    import torch
    from radeonrays_sdk_gb300 import scenes
    v, i = scenes.heightfield(129, scenes.rng(60))
    bvh = ctx.build_geometry(to_dev(v), to_dev(i))
    rays = scenes.incoherent_rays(n, v.min(axis=0), v.max(axis=0), scenes.rng(60, n))
    if q == 1:
        rays[:, 7] = np.float32(0.3)
    want = hits_np(ctx.intersect(bvh, to_dev(rays), query=q, output=o))
    got = ctx.intersect_host(bvh, torch.from_numpy(rays).pin_memory(), query=q, output=o, chunk_rays=chunk)
    assert np.array_equal(got.numpy().view(np.uint32), want)
    assert ctx.device_errors() == 0


# The streamed plan (one persistent launch over all rays while the copies
# run; 2^16 rays or more) against device tracing: ragged last chunks, many
# small chunks, a single chunk, AABB-list and empty geometry; and the chunked
# plan it falls back to (graph capture, RR_CUDA_STREAM_RAYS=0) on the same rays.
def _heightfield_case(n, seed):
    from radeonrays_sdk_gb300 import scenes
    v, i = scenes.heightfield(257, scenes.rng(61))
    rays = scenes.incoherent_rays(n, v.min(axis=0), v.max(axis=0), scenes.rng(61, seed))
    return v, i, rays


@pytest.mark.parametrize("n,chunk", [(65536, 0), (1_000_003, 0), (300_001, 4096), (524_288, 65536)])
@pytest.mark.parametrize("q,o", [(0, 0), (1, 1)])
def test_streamed_host_trace_equals_device_trace(ctx, n, chunk, q, o):
    import torch
    v, i, rays = _heightfield_case(n, n)
    if q == 1:
        rays[:, 7] = np.float32(0.05)
    bvh = ctx.build_geometry(to_dev(v), to_dev(i), quality=True)
    ctx.set_traversal(3)  # the persistent binary kernel's streamed variant (the 4-wide one: test below)
    try:
        want = hits_np(ctx.intersect(bvh, to_dev(rays), query=q, output=o))
        got = ctx.intersect_host(bvh, torch.from_numpy(rays).pin_memory(), query=q, output=o, chunk_rays=chunk)
    finally:
        ctx.set_traversal(0)
    assert np.array_equal(got.numpy().view(np.uint32), want)
    assert ctx.device_errors() == 0


def test_streamed_host_trace_aabbs_and_empty(ctx):
    import torch
    from radeonrays_sdk_gb300 import scenes
    g = scenes.rng(62)
    lo = g.random((5000, 3), dtype=np.float32)
    boxes = np.zeros((5000, 8), np.float32)
    boxes[:, 0:3] = lo
    boxes[:, 4:7] = lo + np.float32(0.01)
    aabb = ctx.build_aabbs(torch.from_numpy(boxes).cuda())
    rays = scenes.incoherent_rays(100_000, (0, 0, 0), (1, 1, 1), scenes.rng(62, 1))
    want = hits_np(ctx.intersect(aabb, to_dev(rays)))
    got = ctx.intersect_host(aabb, torch.from_numpy(rays).pin_memory())
    assert np.array_equal(got.numpy().view(np.uint32), want)
    empty = ctx.build_geometry(torch.zeros((3, 3), dtype=torch.float32, device="cuda"),
                               torch.zeros((0, 3), dtype=torch.int32, device="cuda"))
    got = ctx.intersect_host(empty, torch.from_numpy(rays).pin_memory()).numpy().view(np.uint32)
    assert np.all(got[:, 2] == INVALID)
    assert ctx.device_errors() == 0


def test_streamed_and_chunked_plans_agree(ctx, monkeypatch):
    """Two host-buffer traces recorded into one command stream are captured
    into a CUDA graph, where the chunked plan runs; a context made with
    RR_CUDA_STREAM_RAYS=0 always runs it.  Both equal the streamed plan."""
    import ctypes as C
    import torch
    from radeonrays_sdk_gb300 import rr
    v, i, rays = _heightfield_case(300_000, 7)
    bvh = ctx.build_geometry(to_dev(v), to_dev(i))
    rh = torch.from_numpy(rays).pin_memory()
    streamed = ctx.intersect_host(bvh, rh).numpy().view(np.uint32).copy()
    R = rays.shape[0]
    outs = [torch.full((R, 4), -1, dtype=torch.int32).pin_memory() for _ in range(2)]
    stag = [(torch.empty((R, 8), dtype=torch.float32, device="cuda"),
             torch.full((R, 4), -1, dtype=torch.int32, device="cuda"),  # a miss writes only inst_id
             torch.empty(ctx.trace_scratch_bytes(R), dtype=torch.uint8, device="cuda")) for _ in range(2)]
    cs = ctx.command_stream()
    for k in range(2):
        rr.check(ctx.L.rrCudaCmdIntersectHostBuffers(ctx.ctx, ctx.ptr(bvh), 0, C.c_void_p(rh.data_ptr()), R, 0,
                                                     C.c_void_p(outs[k].data_ptr()), ctx.ptr(stag[k][0]),
                                                     ctx.ptr(stag[k][1]), ctx.ptr(stag[k][2]), 0, cs), "record")
    ctx.submit(cs)
    ctx.release_stream(cs)
    for k in range(2):
        assert np.array_equal(outs[k].numpy().view(np.uint32), streamed)
    monkeypatch.setenv("RR_CUDA_STREAM_RAYS", "0")
    with rr.Context() as c2:
        b2 = c2.build_geometry(to_dev(v), to_dev(i))
        chunked = c2.intersect_host(b2, rh).numpy().view(np.uint32)
        assert c2.device_errors() == 0
    assert np.array_equal(chunked, streamed)
    assert ctx.device_errors() == 0


@pytest.mark.parametrize("q,o", [(0, 0), (1, 1)])
def test_streamed_host_trace_bvh4(ctx, q, o):
    """The 4-wide kernel's streamed variant gives the hits of its device run."""
    import torch
    v, i, rays = _heightfield_case(300_001, 11)
    if q == 1:
        rays[:, 7] = np.float32(0.05)
    bvh = ctx.build_geometry(to_dev(v), to_dev(i), node_format=2)
    ctx.set_traversal(4)
    try:
        want = hits_np(ctx.intersect(bvh, to_dev(rays), query=q, output=o))
        got = ctx.intersect_host(bvh, torch.from_numpy(rays).pin_memory(), query=q, output=o, chunk_rays=16384)
    finally:
        ctx.set_traversal(0)
    assert np.array_equal(got.numpy().view(np.uint32), want)
    assert ctx.device_errors() == 0


def _late_count(sc, R, chunk):
    """The late-list count of the streamed plan that last used scratch `sc`: its words sit at the end of the
    scratch (arrival flags, one per chunk; done counters, one per part of eight chunks; the give-up flag; the
    count)."""
    shift = 17
    if chunk:
        shift = 12
        while shift < 24 and (2 << shift) <= chunk:
            shift += 1
    chunks = -(-R // (1 << shift))
    parts = -(-R // (1 << (shift + 3)))
    wbytes = -(-(chunks + parts + 2) * 4 // 256) * 256
    woff = (sc.numel() - wbytes) // 256 * 256
    w = sc[woff:woff + wbytes].cpu().numpy().view(np.uint32)
    return int(w[chunks + parts + 1])


@pytest.mark.parametrize("trav,fmt", [(3, 0), (4, 4)])
@pytest.mark.parametrize("q,o", [(0, 0), (1, 1)])
def test_streamed_late_list(ctx, trav, fmt, q, o):
    """Small parts (32,768 rays) and a full grid in flight: warps publish parts while some of their rays are still
    traced, and every ray in flight when the rays run out is late-listed.  Those rays' hits reach the host through
    the late scatter after the parts' copies; every hit equals the device trace's."""
    import torch
    R, chunk = 400_003, 4096
    v, i, rays = _heightfield_case(R, 13)
    if q == 1:
        rays[:, 7] = np.float32(0.05)
    bvh = ctx.build_geometry(to_dev(v), to_dev(i), node_format=fmt, quality=True)
    full = o == 0
    staging = (torch.empty((R, 8), dtype=torch.float32, device="cuda"),
               torch.full((R, 4) if full else (R,), -1, dtype=torch.int32, device="cuda"),
               torch.empty(ctx.trace_scratch_bytes(R), dtype=torch.uint8, device="cuda"))
    ctx.set_traversal(trav)
    try:
        want = hits_np(ctx.intersect(bvh, to_dev(rays), query=q, output=o))
        for _ in range(2):
            got = ctx.intersect_host(bvh, torch.from_numpy(rays).pin_memory(), query=q, output=o, chunk_rays=chunk,
                                     staging=staging)
            torch.cuda.synchronize()
            assert np.array_equal(got.numpy().view(np.uint32), want)
            late = _late_count(staging[2], R, chunk)
            assert 0 < late < R
    finally:
        ctx.set_traversal(0)
    assert ctx.device_errors() == 0


def test_pageable_hit_buffer_takes_the_chunked_plan(ctx):
    """The late scatter writes the host hit buffer from a kernel; a pageable buffer, which it cannot write, takes
    the chunked plan, with the same hits."""
    import torch
    R = 300_001
    v, i, rays = _heightfield_case(R, 14)
    bvh = ctx.build_geometry(to_dev(v), to_dev(i), node_format=4)
    want = hits_np(ctx.intersect(bvh, to_dev(rays)))
    got = ctx.intersect_host(bvh, torch.from_numpy(rays).pin_memory(), chunk_rays=65536, pinned_hits=False)
    assert np.array_equal(got.numpy().view(np.uint32), want)
    assert ctx.device_errors() == 0
