"""Failure detection on the GPU, with no fault provoked.

Every device-side wait of the build is bounded and every traversal checks
its node indices and stack depth; each stop sets a bit of the context's
device error word (rrCudaGetDeviceErrors) instead of trapping.  The
reference waits forever (vlk/device.cpp:249-272) and writes past its stack.
These tests make each stop happen on purpose and read the bit back:

  * WAIT_TIMEOUT, onesweep look-back: a sort tile that never publishes its
    digit counts (rrCudaSetWaitLimits test hook) makes later tiles run out of
    polls; they count the earlier keys themselves, so the build stays exact;
  * WAIT_TIMEOUT, streamed host-buffer trace: the last chunk's arrival flag
    is never raised; the warps that wait for it give up and finish their rays
    as misses, and every copy still completes;
  * NODE_RANGE: a result buffer whose child index points past its node array;
  * STACK_OVERFLOW: a tree 400 levels deep whose every node defers a child.

Each case is followed by a clean run on the same context: the error word
reads back 0 and the results are the normal ones.
"""
import numpy as np
import pytest

from gpu_util import INVALID, hits_np, nodes_of, to_dev, trailer_of

pytestmark = pytest.mark.gpu

WAIT_TIMEOUT, NODE_RANGE, STACK_OVERFLOW = 16, 8, 1


def test_sort_lookback_timeout_is_reported_and_build_stays_exact(ctx, orc):
    from radeonrays_sdk_gb300 import scenes
    v, i = scenes.soup(100_000, scenes.rng(120))  # 25 sort tiles of 4096 keys
    want, _, _ = orc.build_mesh(v, i)
    assert ctx.device_errors() == 0
    ctx.set_wait_limits(lookback_polls=2000, hold_sort_tile=3)
    try:
        res = ctx.build_geometry(to_dev(v), to_dev(i), node_format=0)
        assert ctx.device_errors() & WAIT_TIMEOUT
    finally:
        ctx.set_wait_limits()
    got = nodes_of(res, 100_000)
    assert np.array_equal(got.view(np.uint32).reshape(-1, 16), want.view(np.uint32).reshape(-1, 16))
    res2 = ctx.build_geometry(to_dev(v), to_dev(i), node_format=0)
    assert ctx.device_errors() == 0
    assert np.array_equal(nodes_of(res2, 100_000).view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("traversal", [3, 4])
def test_streamed_arrival_timeout_is_reported(ctx, traversal):
    import torch
    from radeonrays_sdk_gb300 import scenes
    v, i = scenes.heightfield(257, scenes.rng(121))
    n, chunk = 300_000, 16_384
    rays = scenes.incoherent_rays(n, v.min(axis=0), v.max(axis=0), scenes.rng(121, 1))
    bvh = ctx.build_geometry(to_dev(v), to_dev(i))
    rh = torch.from_numpy(rays).pin_memory()
    ctx.set_traversal(traversal)
    try:
        want = hits_np(ctx.intersect(bvh, to_dev(rays)))
        last = (n - 1) // chunk
        ctx.set_wait_limits(arrival_polls=20_000, drop_arrival_chunk=last)
        try:
            got = ctx.intersect_host(bvh, rh, chunk_rays=chunk).numpy().view(np.uint32)
            assert ctx.device_errors() & WAIT_TIMEOUT
        finally:
            ctx.set_wait_limits()
        # Rays of the withheld chunk that a waiting warp gave up on are misses;
        # every other ray is traced normally.  A claim spans at most 32 rays.
        same = np.all(got == want, axis=1)
        assert np.all(same | (got[:, 2] == INVALID))
        assert np.all(same[: last * chunk - 32])
        assert not np.all(same[last * chunk:])
        again = ctx.intersect_host(bvh, rh, chunk_rays=chunk).numpy().view(np.uint32)
        assert np.array_equal(again, want)
        assert ctx.device_errors() == 0
    finally:
        ctx.set_traversal(0)


def _registered_copy(ctx, res, n):
    """A copy of a result buffer, registered like a loaded one."""
    from radeonrays_sdk_gb300 import rr
    buf = res.clone()
    import torch
    torch.cuda.synchronize()
    rr.check(ctx.L.rrCudaRegisterGeometry(ctx.ctx, ctx.ptr(buf), n), "rrCudaRegisterGeometry")
    return buf


def test_node_range_is_reported(ctx):
    import torch
    from radeonrays_sdk_gb300 import scenes
    v, i = scenes.heightfield(65, scenes.rng(122))
    n = i.shape[0]
    rays = scenes.incoherent_rays(20_000, v.min(axis=0), v.max(axis=0), scenes.rng(122, 1))
    rd = to_dev(rays)
    # Binary nodes: the root's child0 points past the 2n - 1 nodes.
    res = ctx.build_geometry(to_dev(v), to_dev(i), node_format=0)
    bad = _registered_copy(ctx, res, n)
    root = bad[:64].view(torch.int32)
    root[3] = 2 * n + 7
    for trav in (1, 3):
        ctx.set_traversal(trav)
        ctx.intersect(bad, rd)
        assert ctx.device_errors() & NODE_RANGE, trav
        ctx.intersect(res, rd)
        assert ctx.device_errors() == 0, trav
    # 4-wide nodes (fp32: child words at byte 96 of a 128-byte node; 8-bit:
    # at byte 16 of a 64-byte node): an internal reference past the 4-wide
    # array, and a leaf reference past the binary leaves.
    for fmt, coff in ((2, 96), (4, 16)):
        res4 = ctx.build_geometry(to_dev(v), to_dev(i), node_format=fmt)
        off = int(trailer_of(res4, n)["wide_nodes_off"])
        for ref in (0x7FFFFFF0, 0x80000000 | (2 * n + 5)):
            bad4 = _registered_copy(ctx, res4, n)
            child = bad4[off + coff: off + coff + 16].view(torch.int32)
            child[:] = torch.tensor(np.array([ref] * 4, np.uint32).view(np.int32), device="cuda")
            ctx.set_traversal(4)
            ctx.intersect(bad4, rd)
            assert ctx.device_errors() & NODE_RANGE, (fmt, hex(ref))
            ctx.intersect(res4, rd)
            assert ctx.device_errors() == 0
    ctx.set_traversal(0)


def test_stack_overflow_is_reported(ctx):
    """A caterpillar tree: internal node k has the next internal node as
    child0 and a leaf as child1, every box is the unit cube, so a ray that
    enters the cube visits child0 first and defers a leaf at every level."""
    import torch
    from radeonrays_sdk_gb300 import rr, scenes
    n = 400
    v, i = scenes.soup(n, scenes.rng(123))
    res = ctx.build_geometry(to_dev(v), to_dev(i), node_format=0)
    nodes = np.zeros(2 * n - 1, rr.NODE_DTYPE)
    inner = np.arange(n - 1)
    nodes["a0"][inner] = 0.0
    nodes["a1"][inner] = 1.0
    nodes["b0"][inner] = 0.0
    nodes["b1"][inner] = 1.0
    nodes["child0"][inner] = np.where(inner + 1 <= n - 2, inner + 1, 2 * n - 2)
    nodes["child1"][inner] = n - 1 + inner
    nodes["update"][inner] = 1
    leaves = np.arange(n - 1, 2 * n - 1)
    nodes["child0"][leaves] = INVALID
    nodes["child1"][leaves] = np.arange(n)
    nodes["a0"][leaves] = (10.0, 10.0, 10.0)  # triangles far outside the cube: every leaf test misses
    nodes["a1"][leaves] = (10.0, 11.0, 10.0)
    nodes["b0"][leaves] = (11.0, 10.0, 10.0)
    nodes["parent"] = INVALID
    bad = _registered_copy(ctx, res, n)
    raw = torch.from_numpy(nodes.view(np.uint8).copy()).cuda()
    bad[: raw.numel()] = raw
    rays = np.zeros((256, 8), np.float32)
    rays[:, 0:3] = (0.5, 0.5, -1.0)
    rays[:, 4:7] = (0.0, 0.0, 1.0)
    rays[:, 7] = 1e30
    for trav in (1, 3):
        ctx.set_traversal(trav)
        h = hits_np(ctx.intersect(bad, to_dev(rays)))
        assert ctx.device_errors() & STACK_OVERFLOW, trav
        assert np.all(h[:, 2] == INVALID)
        ctx.intersect(res, to_dev(rays))
        assert ctx.device_errors() == 0
    ctx.set_traversal(0)
