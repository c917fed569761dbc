"""CPU tests of the C-ABI library: it loads, exports every entry point the
headers declare, and the host-side argument checks return the reference's
error codes (radeonrays.cpp) without touching a GPU."""
import ctypes as C
import re

import pytest

from conftest import ROOT


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        names |= set(re.findall(r"RR_API\s+RRError\s+(\w+)\s*\(", h.read_text()))
    return names


def test_library_exports_every_declared_symbol(rrlib):
    from radeonrays_sdk_gb300 import rr
    names = declared_symbols()
    assert len(names) >= 28
    for n in names:
        assert hasattr(rrlib, n), n
    assert names <= set(rr.PROTOTYPES), names - set(rr.PROTOTYPES)


def test_reference_spellings_kept(rrlib):
    text = (ROOT / "include" / "radeonrays.h").read_text()
    assert "rrSumbitCommandStream" in text and "RR_INAVLID_VALUE" in text
    assert hasattr(rrlib, "rrSumbitCommandStream")


def test_create_context_argument_checks(rrlib):
    from radeonrays_sdk_gb300 import rr
    ctx = C.c_void_p()
    assert rrlib.rrCreateContext(rr.RR_API_VERSION, rr.RR_API_CUDA, None) == rr.RR_ERROR_INVALID_PARAMETER
    assert rrlib.rrCreateContext(rr.RR_API_VERSION, rr.RR_API_VK, C.byref(ctx)) == rr.RR_ERROR_UNSUPPORTED_API
    assert rrlib.rrCreateContext(rr.RR_API_VERSION, rr.RR_API_DX, C.byref(ctx)) == rr.RR_ERROR_UNSUPPORTED_API
    assert rrlib.rrDestroyContext(None) == rr.RR_ERROR_INVALID_PARAMETER


def test_null_arguments_rejected(rrlib):
    from radeonrays_sdk_gb300 import rr
    E = rr.RR_ERROR_INVALID_PARAMETER
    fake = C.c_void_p(0x1000)  # never dereferenced: every call below fails its null checks first
    assert rrlib.rrCmdBuildGeometry(None, 1, None, None, None, None, None) == E
    assert rrlib.rrCmdBuildGeometry(fake, 1, None, None, None, None, fake) == E
    assert rrlib.rrCmdBuildScene(fake, None, None, None, None, fake) == E
    assert rrlib.rrCmdIntersect(fake, None, 0, fake, 1, None, 0, fake, fake, fake) == E
    assert rrlib.rrCmdIntersect(fake, fake, 0, fake, 1, None, 0, fake, None, fake) == E
    assert rrlib.rrGetTraceMemoryRequirements(None, 1, None) == E
    sz = C.c_size_t()
    assert rrlib.rrGetTraceMemoryRequirements(fake, 0, C.byref(sz)) == E  # radeonrays.cpp:741-745
    assert rrlib.rrAllocateCommandStream(fake, None) == E
    assert rrlib.rrSumbitCommandStream(fake, fake, None, None) == E
    assert rrlib.rrWaitEvent(fake, None) == E
    assert rrlib.rrReleaseEvent(None, fake) == E
    assert rrlib.rrReleaseDevicePtr(fake, None) == E
    assert rrlib.rrGetDevicePtrFromCudaPtr(fake, None, 0, None) == E
    assert rrlib.rrSetLogLevel(99) == E
    assert rrlib.rrSetLogFile(None) == E


def test_memory_requirements_host_logic(rrlib, tmp_path):
    """Sizes come from the host layout code only (no device access)."""
    from radeonrays_sdk_gb300 import rr
    fake = C.c_void_p(0x1000)
    mesh = rr.RRTriangleMeshPrimitive(None, 0, 12, None, 1000, rr.RR_INDEX_TYPE_UINT32)
    bi = rr.RRGeometryBuildInput(rr.RR_PRIMITIVE_TYPE_TRIANGLE_MESH, 1, C.pointer(mesh))
    req = rr.RRMemoryRequirements()
    assert rrlib.rrGetGeometryBuildMemoryRequirements(fake, C.byref(bi), None, C.byref(req)) == rr.RR_SUCCESS
    plain_opts = rr.RRCudaBuildOptions(C.sizeof(rr.RRCudaBuildOptions), rr.RR_CUDA_NODE_FORMAT_BINARY, 30, 0)
    opts = rr.RRBuildOptions(1, C.cast(C.pointer(plain_opts), C.c_void_p))
    req_b = rr.RRMemoryRequirements()
    assert rrlib.rrGetGeometryBuildMemoryRequirements(fake, C.byref(bi), C.byref(opts), C.byref(req_b)) == 0
    nodes = (2 * 1000 - 1) * 64
    assert req_b.result_buffer_size == (nodes + 255) // 256 * 256 + 256
    # Default (null options): binary nodes + trailer + quantised 4-wide nodes
    # of 64 B, capacity (n-1)//3 + n//3 + 1, 256-byte aligned; BVH4 has 128 B.
    cap4 = (1000 - 1) // 3 + 1000 // 3 + 1
    assert req.result_buffer_size == ((nodes + 255) // 256 * 256 + 256 + cap4 * 64 + 255) // 256 * 256
    f4_opts = rr.RRCudaBuildOptions(C.sizeof(rr.RRCudaBuildOptions), rr.RR_CUDA_NODE_FORMAT_BVH4, 30, 0)
    opts4 = rr.RRBuildOptions(1, C.cast(C.pointer(f4_opts), C.c_void_p))
    req_4 = rr.RRMemoryRequirements()
    assert rrlib.rrGetGeometryBuildMemoryRequirements(fake, C.byref(bi), C.byref(opts4), C.byref(req_4)) == 0
    assert req_4.result_buffer_size == ((nodes + 255) // 256 * 256 + 256 + cap4 * 128 + 255) // 256 * 256
    w8_opts = rr.RRCudaBuildOptions(C.sizeof(rr.RRCudaBuildOptions), rr.RR_CUDA_NODE_FORMAT_WIDE8, 30, 0)
    opts8 = rr.RRBuildOptions(1, C.cast(C.pointer(w8_opts), C.c_void_p))
    req_8 = rr.RRMemoryRequirements()
    assert rrlib.rrGetGeometryBuildMemoryRequirements(fake, C.byref(bi), C.byref(opts8), C.byref(req_8)) == 0
    assert req_8.result_buffer_size > req.result_buffer_size > req_b.result_buffer_size
    # AUTO (the node-format tuner's choice) is sized for either width.
    auto_opts = rr.RRCudaBuildOptions(C.sizeof(rr.RRCudaBuildOptions), rr.RR_CUDA_NODE_FORMAT_AUTO, 30, 0)
    optsa = rr.RRBuildOptions(1, C.cast(C.pointer(auto_opts), C.c_void_p))
    req_a = rr.RRMemoryRequirements()
    assert rrlib.rrGetGeometryBuildMemoryRequirements(fake, C.byref(bi), C.byref(optsa), C.byref(req_a)) == 0
    q8_opts = rr.RRCudaBuildOptions(C.sizeof(rr.RRCudaBuildOptions), rr.RR_CUDA_NODE_FORMAT_BVH4Q8, 30, 0)
    optsq = rr.RRBuildOptions(1, C.cast(C.pointer(q8_opts), C.c_void_p))
    req_q = rr.RRMemoryRequirements()
    assert rrlib.rrGetGeometryBuildMemoryRequirements(fake, C.byref(bi), C.byref(optsq), C.byref(req_q)) == 0
    cap4 = (1000 - 1) // 3 + 1000 // 3 + 1  # 64-byte quantised 4-wide nodes
    assert req_q.result_buffer_size == ((nodes + 255) // 256 * 256 + 256 + cap4 * 64 + 255) // 256 * 256
    assert req_q.result_buffer_size == req.result_buffer_size  # the default is BVH4Q8
    assert req_a.result_buffer_size == max(req_4.result_buffer_size, req_8.result_buffer_size,
                                           req_q.result_buffer_size)
    assert req_a.temporary_build_buffer_size == max(req.temporary_build_buffer_size,
                                                    req_8.temporary_build_buffer_size,
                                                    req_q.temporary_build_buffer_size)
    # An unknown node format is rejected.
    bad_opts = rr.RRCudaBuildOptions(C.sizeof(rr.RRCudaBuildOptions), 5, 30, 0)
    optsx = rr.RRBuildOptions(1, C.cast(C.pointer(bad_opts), C.c_void_p))
    assert rrlib.rrGetGeometryBuildMemoryRequirements(fake, C.byref(bi), C.byref(optsx), C.byref(req_8)) == \
        rr.RR_ERROR_INVALID_PARAMETER
    # An update needs scratch only to collapse the wide nodes again.
    assert req_b.temporary_update_buffer_size == 0
    assert 0 < req.temporary_update_buffer_size < req.temporary_build_buffer_size
    # Unsupported primitive type / bad input.
    # AABB lists: sized like a binary-node build of that many leaves; a box
    # stride below 32 bytes is rejected; an unknown primitive type is not implemented.
    boxes = rr.RRAABBListPrimitive(None, 1000, 32)
    bi2 = rr.RRGeometryBuildInput(rr.RR_PRIMITIVE_TYPE_AABB_LIST, 1,
                                  C.cast(C.pointer(boxes), C.POINTER(rr.RRTriangleMeshPrimitive)))
    req_a = rr.RRMemoryRequirements()
    assert rrlib.rrGetGeometryBuildMemoryRequirements(fake, C.byref(bi2), None, C.byref(req_a)) == rr.RR_SUCCESS
    assert req_a.result_buffer_size == req_b.result_buffer_size
    boxes.aabb_stride = 16
    assert rrlib.rrGetGeometryBuildMemoryRequirements(fake, C.byref(bi2), None, C.byref(req_a)) == \
        rr.RR_ERROR_INVALID_PARAMETER
    bi5 = rr.RRGeometryBuildInput(7, 1, C.pointer(mesh))
    assert rrlib.rrGetGeometryBuildMemoryRequirements(fake, C.byref(bi5), None, C.byref(req)) == \
        rr.RR_ERROR_NOT_IMPLEMENTED
    bi3 = rr.RRGeometryBuildInput(rr.RR_PRIMITIVE_TYPE_TRIANGLE_MESH, 2, C.pointer(mesh))
    assert rrlib.rrGetGeometryBuildMemoryRequirements(fake, C.byref(bi3), None, C.byref(req)) == \
        rr.RR_ERROR_INVALID_PARAMETER
    bad = rr.RRTriangleMeshPrimitive(None, 0, 10, None, 10, rr.RR_INDEX_TYPE_UINT32)
    bi4 = rr.RRGeometryBuildInput(rr.RR_PRIMITIVE_TYPE_TRIANGLE_MESH, 1, C.pointer(bad))
    assert rrlib.rrGetGeometryBuildMemoryRequirements(fake, C.byref(bi4), None, C.byref(req)) == \
        rr.RR_ERROR_INVALID_PARAMETER
    # Trace scratch: 256 bytes per ray (reference geometry_trace.cpp:169), at least 4096 rays' worth.
    sz = C.c_size_t()
    assert rrlib.rrGetTraceMemoryRequirements(fake, 1 << 20, C.byref(sz)) == 0
    assert sz.value == 256 + (1 << 20) * 256
    # Scene sizes: nodes + [inverse, forward] transforms + trailer + instance records.
    sbi = rr.RRSceneBuildInput(None, 2048)
    assert rrlib.rrGetSceneBuildMemoryRequirements(fake, C.byref(sbi), None, C.byref(req)) == 0
    assert req.result_buffer_size >= (2 * 2048 - 1) * 64 + 2 * 2048 * 48 + 256 + 2048 * 32


def test_log_controls(rrlib, tmp_path):
    from radeonrays_sdk_gb300 import rr
    assert rrlib.rrSetLogLevel(rr.RR_LOG_LEVEL_ERROR) == 0
    assert rrlib.rrSetLogFile(str(tmp_path / "rr.log").encode()) == 0
    assert rrlib.rrSetLogLevel(rr.RR_LOG_LEVEL_WARN) == 0


def test_no_alloc_argument_checks(rrlib):
    """rrCudaIntersectNoAlloc and its error reader reject bad arguments before
    any device call; an empty batch is a successful no-op."""
    from radeonrays_sdk_gb300 import rr
    E = rr.RR_ERROR_INVALID_PARAMETER
    fake = C.c_void_p(0x1000)  # never dereferenced: every call below returns before touching a device
    f = rrlib.rrCudaIntersectNoAlloc
    CL, FULL = rr.RR_INTERSECT_QUERY_CLOSEST, rr.RR_INTERSECT_QUERY_OUTPUT_FULL_HIT
    assert f(None, 10, CL, fake, 1, FULL, fake, None) == E
    assert f(fake, 10, CL, None, 1, FULL, fake, None) == E
    assert f(fake, 10, CL, fake, 1, FULL, None, None) == E
    assert f(fake, 10, 7, fake, 1, FULL, fake, None) == E
    assert f(fake, 10, CL, fake, 1, 9, fake, None) == E
    assert f(fake, 0x80000000, CL, fake, 1, FULL, fake, None) == E  # 2N - 1 nodes would not fit 32 bits
    assert f(fake, 10, CL, fake, 131_073, FULL, fake, None) == E    # beyond the fixed scratch
    assert f(fake, 10, CL, fake, 0, FULL, fake, None) == rr.RR_SUCCESS
    assert f(fake, 10, rr.RR_INTERSECT_QUERY_ANY, fake, 0, rr.RR_INTERSECT_QUERY_OUTPUT_INSTANCE_ID, fake,
             None) == rr.RR_SUCCESS
    assert rrlib.rrCudaGetNoAllocDeviceErrors(None, None) == E
