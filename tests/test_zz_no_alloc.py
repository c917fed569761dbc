"""rrCudaIntersectNoAlloc: tracing without any device allocation.

Some callers cannot call cudaMalloc when they trace rays (a latency-bound
serving loop, where cudaMalloc may block and synchronise the device, or a host
whose device memory is owned by another allocator).  This entry point takes
only their BVH, rays and hit buffer and keeps its traversal scratch in a fixed
device array inside librr.so.  The test checks it through the C-ABI against
rrCmdIntersect's plain traversal (the same kernel, so bit-identical hits) and
against the CPU oracle, on two calls in a row; that its device error word
reads back clean after normal calls and reports a node-range stop; and that
oversized batches are refused.

The file is collected last so that a failure here does not hide any other
test's result; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _errors(L, stream):
    from radeonrays_sdk_gb300 import rr
    bits = C.c_uint32(0xDEAD)
    assert L.rrCudaGetNoAllocDeviceErrors(C.c_void_p(stream.cuda_stream), C.byref(bits)) == rr.RR_SUCCESS
    return bits.value


def test_no_alloc_intersect_matches_rr_cmd_intersect(rrlib, orc):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from radeonrays_sdk_gb300 import rr, scenes

    v, i = scenes.heightfield(129, scenes.rng(60))
    n_tri = i.shape[0]
    rays = scenes.incoherent_rays(50_000, v.min(0), v.max(0), scenes.rng(60, 1))
    nodes, _, _ = orc.build_mesh(v, i)
    with rr.Context() as ctx:
        bvh = ctx.build_geometry(torch.from_numpy(v).cuda(), torch.from_numpy(i.view(np.int32)).cuda())
        rays_d = torch.from_numpy(rays).cuda()
        ctx.set_traversal(rr.RR_CUDA_TRAVERSAL_BINARY)
        stream = torch.cuda.Stream()
        assert _errors(ctx.L, stream) == 0  # clears anything an earlier process step left
        for query, output, shape in ((rr.RR_INTERSECT_QUERY_CLOSEST, rr.RR_INTERSECT_QUERY_OUTPUT_FULL_HIT, (50_000, 4)),
                                     (rr.RR_INTERSECT_QUERY_ANY, rr.RR_INTERSECT_QUERY_OUTPUT_INSTANCE_ID, (50_000,))):
            want = ctx.intersect(bvh, rays_d, query=query, output=output).cpu().numpy()
            oracle_hits = orc.trace(nodes, rays, query=query, output=output)
            assert np.array_equal(want.view(np.uint32), oracle_hits)
            for _ in range(2):  # two calls in a row share the fixed scratch
                hits = torch.full(shape, -1, dtype=torch.int32, device="cuda")
                code = ctx.L.rrCudaIntersectNoAlloc(C.c_void_p(bvh.data_ptr()), n_tri, query,
                                                    C.c_void_p(rays_d.data_ptr()), rays.shape[0], output,
                                                    C.c_void_p(hits.data_ptr()), C.c_void_p(stream.cuda_stream))
                assert code == rr.RR_SUCCESS
                stream.synchronize()
                got = hits.cpu().numpy()
                assert np.array_equal(got, want)
                assert np.array_equal(got.view(np.uint32), oracle_hits)
                assert _errors(ctx.L, stream) == 0
        # A triangle count that is too small bounds the node indices below the
        # real tree: the rays that reach past it stop, and the error word says so.
        hits = torch.full((50_000, 4), -1, dtype=torch.int32, device="cuda")
        assert ctx.L.rrCudaIntersectNoAlloc(C.c_void_p(bvh.data_ptr()), n_tri // 4, rr.RR_INTERSECT_QUERY_CLOSEST,
                                            C.c_void_p(rays_d.data_ptr()), rays.shape[0],
                                            rr.RR_INTERSECT_QUERY_OUTPUT_FULL_HIT, C.c_void_p(hits.data_ptr()),
                                            C.c_void_p(stream.cuda_stream)) == rr.RR_SUCCESS
        assert _errors(ctx.L, stream) & rr.RR_CUDA_DEVICE_ERROR_NODE_RANGE
        assert _errors(ctx.L, stream) == 0  # read and cleared
        big = torch.empty((131_073, 8), dtype=torch.float32, device="cuda")
        out = torch.empty((131_073, 4), dtype=torch.int32, device="cuda")
        assert ctx.L.rrCudaIntersectNoAlloc(C.c_void_p(bvh.data_ptr()), n_tri, 0, C.c_void_p(big.data_ptr()),
                                            131_073, 0, C.c_void_p(out.data_ptr()), None) == \
            rr.RR_ERROR_INVALID_PARAMETER
