"""rrCudaIntersectNoAlloc: tracing without any device allocation.

Some callers cannot call cudaMalloc when they trace rays (a latency-bound
serving loop, where cudaMalloc may block and synchronise the device, or a host
whose device memory is owned by another allocator).  This entry point takes
only their BVH, rays and hit buffer and keeps its traversal scratch in a fixed
device array inside librr.so.  The test checks it through the C-ABI against
rrCmdIntersect's plain traversal (the same kernel, so bit-identical hits) on
two calls in a row, and that oversized batches are refused.

The file is collected last so that a failure here does not hide any other
test's result; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_no_alloc_intersect_matches_rr_cmd_intersect(rrlib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from radeonrays_sdk_gb300 import rr, scenes

    v, i = scenes.heightfield(129, scenes.rng(60))
    rays = scenes.incoherent_rays(50_000, v.min(0), v.max(0), scenes.rng(60, 1))
    with rr.Context() as ctx:
        bvh = ctx.build_geometry(torch.from_numpy(v).cuda(), torch.from_numpy(i.view(np.int32)).cuda())
        rays_d = torch.from_numpy(rays).cuda()
        ctx.set_traversal(rr.RR_CUDA_TRAVERSAL_BINARY)
        for query, output, shape in ((rr.RR_INTERSECT_QUERY_CLOSEST, rr.RR_INTERSECT_QUERY_OUTPUT_FULL_HIT, (50_000, 4)),
                                     (rr.RR_INTERSECT_QUERY_ANY, rr.RR_INTERSECT_QUERY_OUTPUT_INSTANCE_ID, (50_000,))):
            want = ctx.intersect(bvh, rays_d, query=query, output=output).cpu().numpy()
            stream = torch.cuda.Stream()
            for _ in range(2):  # two calls in a row share (and must clear) the fixed scratch
                hits = torch.full(shape, -1, dtype=torch.int32, device="cuda")
                code = ctx.L.rrCudaIntersectNoAlloc(C.c_void_p(bvh.data_ptr()), query, C.c_void_p(rays_d.data_ptr()),
                                                    rays.shape[0], output, C.c_void_p(hits.data_ptr()),
                                                    C.c_void_p(stream.cuda_stream))
                assert code == rr.RR_SUCCESS
                stream.synchronize()
                assert np.array_equal(hits.cpu().numpy(), want)
        big = torch.empty((131_073, 8), dtype=torch.float32, device="cuda")
        out = torch.empty((131_073, 4), dtype=torch.int32, device="cuda")
        assert ctx.L.rrCudaIntersectNoAlloc(C.c_void_p(bvh.data_ptr()), 0, C.c_void_p(big.data_ptr()), 131_073, 0,
                                            C.c_void_p(out.data_ptr()), None) == rr.RR_ERROR_INVALID_PARAMETER
