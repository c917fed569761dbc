"""GPU host-buffer tracing (rrCudaCmdIntersectHostBuffers): chunks pipelined
over the context's side streams give exactly the hits of rrCmdIntersect on
device buffers, for every chunking, query and output."""
import numpy as np
import pytest

from gpu_util import hits_np, to_dev

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
