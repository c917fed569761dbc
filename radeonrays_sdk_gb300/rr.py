"""ctypes binding of librr.so (the C-ABI in include/radeonrays.h and
include/radeonrays_cuda.h) plus a thin convenience layer used by the tests,
the benchmark and the serving loop.

The binding mirrors the C API one to one (same names, same argument order,
errors raised as RRException carrying the RRError code).  Device memory for
inputs and outputs is allocated with PyTorch (plumbing only); every compute
step runs in librr.so's CUDA kernels.  There is no fallback: if librr.so is
missing or cannot load, `lib()` raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "librr.so"

# ---- enums (include/radeonrays.h) --------------------------------------
RR_SUCCESS = 0
RR_ERROR_NOT_IMPLEMENTED = 1
RR_ERROR_INTERNAL = 2
RR_ERROR_OUT_OF_HOST_MEMORY = 3
RR_ERROR_OUT_OF_DEVICE_MEMORY = 4
RR_ERROR_INVALID_API_VERSION = 5
RR_ERROR_INVALID_PARAMETER = 6
RR_ERROR_UNSUPPORTED_API = 7
RR_ERROR_UNSUPPORTED_INTEROP = 8
ERROR_NAMES = {v: k for k, v in list(globals().items()) if k.startswith("RR_ERROR_") or k == "RR_SUCCESS"}

RR_API_VERSION = 0 * 1000000 + 1 * 1000 + 1
RR_API_DX, RR_API_VK, RR_API_CUDA = 1, 2, 3
RR_INVALID = 0xFFFFFFFF
RR_BUILD_OPERATION_BUILD, RR_BUILD_OPERATION_UPDATE = 1, 2
RR_BUILD_FLAG_BITS_PREFER_FAST_BUILD, RR_BUILD_FLAG_BITS_ALLOW_UPDATE = 1, 2
RR_PRIMITIVE_TYPE_TRIANGLE_MESH, RR_PRIMITIVE_TYPE_AABB_LIST = 0, 1
RR_INDEX_TYPE_UINT32, RR_INDEX_TYPE_UINT16 = 0, 1
RR_INTERSECT_QUERY_CLOSEST, RR_INTERSECT_QUERY_ANY = 0, 1
RR_INTERSECT_QUERY_OUTPUT_FULL_HIT, RR_INTERSECT_QUERY_OUTPUT_INSTANCE_ID = 0, 1
RR_LOG_LEVEL_DEBUG, RR_LOG_LEVEL_INFO, RR_LOG_LEVEL_WARN, RR_LOG_LEVEL_ERROR, RR_LOG_LEVEL_OFF = 1, 2, 3, 4, 5
RR_CUDA_NODE_FORMAT_BINARY, RR_CUDA_NODE_FORMAT_WIDE8, RR_CUDA_NODE_FORMAT_BVH4, RR_CUDA_NODE_FORMAT_AUTO = 0, 1, 2, 3
RR_CUDA_NODE_FORMAT_BVH4Q8 = 4
RR_CUDA_TRAVERSAL_AUTO, RR_CUDA_TRAVERSAL_BINARY, RR_CUDA_TRAVERSAL_WIDE = 0, 1, 2
RR_CUDA_TRAVERSAL_BINARY_PERSISTENT, RR_CUDA_TRAVERSAL_BVH4 = 3, 4
RR_CUDA_TRIANGLE_TEST_REFERENCE, RR_CUDA_TRIANGLE_TEST_WATERTIGHT = 0, 1
RR_CUDA_DEVICE_ERROR_STACK_OVERFLOW = 1
RR_CUDA_DEVICE_ERROR_BAD_BUFFER = 2
RR_CUDA_DEVICE_ERROR_COLLAPSE_DEPTH = 4
RR_CUDA_DEVICE_ERROR_NODE_RANGE = 8
RR_CUDA_DEVICE_ERROR_WAIT_TIMEOUT = 16

# numpy views of the ABI records
RAY_DTYPE = np.dtype([("origin", "<f4", 3), ("min_t", "<f4"), ("direction", "<f4", 3), ("max_t", "<f4")])
HIT_DTYPE = np.dtype([("uv", "<f4", 2), ("inst_id", "<u4"), ("prim_id", "<u4")])
NODE_DTYPE = np.dtype([("a0", "<f4", 3), ("child0", "<u4"), ("a1", "<f4", 3), ("child1", "<u4"),
                       ("b0", "<f4", 3), ("parent", "<u4"), ("b1", "<f4", 3), ("update", "<u4")])
assert RAY_DTYPE.itemsize == 32 and HIT_DTYPE.itemsize == 16 and NODE_DTYPE.itemsize == 64

# Trailer layout offsets (csrc/rr_internal.h struct Trailer).
TRAILER_DTYPE = np.dtype([("magic", "<u4"), ("version", "<u4"), ("kind", "<u4"), ("node_format", "<u4"),
                          ("leaf_count", "<u4"), ("node_count", "<u4"), ("wide_count", "<u4"),
                          ("wide_tri_count", "<u4"), ("wide_nodes_off", "<u8"), ("wide_tris_off", "<u8"),
                          ("wide_capacity", "<u8"), ("tri_capacity", "<u8"), ("bounds", "<u4", 8),
                          ("morton_bits", "<u4"), ("pad", "<u4", 3), ("xforms_off", "<u8"), ("inst_off", "<u8"),
                          ("reserved", "<u8", 16)])
assert TRAILER_DTYPE.itemsize == 256


class RRException(RuntimeError):
    def __init__(self, code: int, where: str):
        super().__init__(f"{where} failed: {ERROR_NAMES.get(code, code)}")
        self.code = code


# ---- ABI structures --------------------------------------------------------
class RRTriangleMeshPrimitive(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("vertex_count", C.c_uint32), ("vertex_stride", C.c_uint32),
                ("triangle_indices", C.c_void_p), ("triangle_count", C.c_uint32), ("index_type", C.c_int)]


class RRAABBListPrimitive(C.Structure):
    _fields_ = [("aabbs", C.c_void_p), ("aabb_count", C.c_uint32), ("aabb_stride", C.c_uint32)]


class RRGeometryBuildInput(C.Structure):
    # The third field is a union of primitive pointers (radeonrays.h:215-226):
    # for RR_PRIMITIVE_TYPE_AABB_LIST pass C.cast(pointer(RRAABBListPrimitive), ...).
    _fields_ = [("primitive_type", C.c_int), ("primitive_count", C.c_uint32),
                ("triangle_mesh_primitives", C.POINTER(RRTriangleMeshPrimitive))]


class RRBuildOptions(C.Structure):
    _fields_ = [("build_flags", C.c_uint32), ("backend_specific_info", C.c_void_p)]


class RRCudaBuildOptions(C.Structure):
    _fields_ = [("struct_size", C.c_uint32), ("node_format", C.c_uint32), ("morton_bits", C.c_uint32),
                ("reserved", C.c_uint32)]


class RRMemoryRequirements(C.Structure):
    _fields_ = [("temporary_build_buffer_size", C.c_size_t), ("temporary_update_buffer_size", C.c_size_t),
                ("result_buffer_size", C.c_size_t)]


class RRInstance(C.Structure):
    _fields_ = [("geometry", C.c_void_p), ("transform", (C.c_float * 4) * 3)]


class RRSceneBuildInput(C.Structure):
    _fields_ = [("instances", C.POINTER(RRInstance)), ("instance_count", C.c_uint32)]


class RRCudaTraversalOptions(C.Structure):
    _fields_ = [("struct_size", C.c_uint32), ("traversal", C.c_uint32), ("block_size", C.c_uint32),
                ("blocks_per_sm", C.c_uint32), ("collect_stats", C.c_uint32), ("ray_order", C.c_uint32),
                ("short_stack", C.c_uint32), ("triangle_test", C.c_uint32)]


class RRCudaWaitLimits(C.Structure):
    _fields_ = [("struct_size", C.c_uint32), ("lookback_polls", C.c_uint32), ("arrival_polls", C.c_uint32),
                ("test_hold_sort_tile", C.c_uint32), ("test_drop_arrival_chunk", C.c_uint32)]


class RRCudaTraversalStats(C.Structure):
    _fields_ = [("rays", C.c_uint64), ("node_fetches", C.c_uint64), ("triangle_fetches", C.c_uint64),
                ("node_bytes", C.c_uint64), ("triangle_bytes", C.c_uint64)]


class RRCudaIntersectRequest(C.Structure):
    _fields_ = [("geometry", C.c_void_p), ("query", C.c_int), ("output", C.c_int), ("rays", C.c_void_p),
                ("ray_count", C.c_uint32), ("hits", C.c_void_p)]


assert C.sizeof(RRGeometryBuildInput) == 16 and C.sizeof(RRInstance) == 56 and C.sizeof(RRMemoryRequirements) == 24
assert C.sizeof(RRCudaIntersectRequest) == 40


class RRCudaHostIntersectRequest(C.Structure):
    _fields_ = [("geometry", C.c_void_p), ("query", C.c_int), ("output", C.c_int), ("host_rays", C.c_void_p),
                ("ray_count", C.c_uint32), ("host_hits", C.c_void_p)]


assert C.sizeof(RRCudaHostIntersectRequest) == 40

# Every symbol the headers declare, with its ctypes prototype.
_P = C.c_void_p
_PP = C.POINTER(C.c_void_p)
PROTOTYPES = {
    "rrCreateContext": [C.c_uint32, C.c_int, _PP],
    "rrDestroyContext": [_P],
    "rrSetLogLevel": [C.c_int],
    "rrSetLogFile": [C.c_char_p],
    "rrCmdBuildGeometry": [_P, C.c_int, C.POINTER(RRGeometryBuildInput), C.POINTER(RRBuildOptions), _P, _P, _P],
    "rrGetGeometryBuildMemoryRequirements": [_P, C.POINTER(RRGeometryBuildInput), C.POINTER(RRBuildOptions),
                                             C.POINTER(RRMemoryRequirements)],
    "rrCmdBuildScene": [_P, C.POINTER(RRSceneBuildInput), C.POINTER(RRBuildOptions), _P, _P, _P],
    "rrGetSceneBuildMemoryRequirements": [_P, C.POINTER(RRSceneBuildInput), C.POINTER(RRBuildOptions),
                                          C.POINTER(RRMemoryRequirements)],
    "rrCmdIntersect": [_P, _P, C.c_int, _P, C.c_uint32, _P, C.c_int, _P, _P, _P],
    "rrGetTraceMemoryRequirements": [_P, C.c_uint32, C.POINTER(C.c_size_t)],
    "rrAllocateCommandStream": [_P, _PP],
    "rrReleaseCommandStream": [_P, _P],
    "rrSumbitCommandStream": [_P, _P, _P, _PP],
    "rrReleaseEvent": [_P, _P],
    "rrWaitEvent": [_P, _P],
    "rrReleaseDevicePtr": [_P, _P],
    "rrReleaseExternalCommandStream": [_P, _P],
    "rrGetDevicePtrFromCudaPtr": [_P, _P, C.c_size_t, _PP],
    "rrGetCudaPtrFromDevicePtr": [_P, _P, _PP],
    "rrGetCommandStreamFromCudaStream": [_P, _P, _PP],
    "rrAllocateDeviceBuffer": [_P, C.c_size_t, _PP],
    "rrMapDevicePtr": [_P, _P, _PP],
    "rrUnmapDevicePtr": [_P, _P, _PP],
    "rrCudaSetTraversalOptions": [_P, C.POINTER(RRCudaTraversalOptions)],
    "rrCudaGetTraversalOptions": [_P, C.POINTER(RRCudaTraversalOptions)],
    "rrCudaGetDeviceErrors": [_P, C.POINTER(C.c_uint32)],
    "rrCudaGetTraversalStats": [_P, C.POINTER(RRCudaTraversalStats)],
    "rrCudaSetWaitTimeout": [_P, C.c_uint32],
    "rrCudaSetWaitLimits": [_P, C.POINTER(RRCudaWaitLimits)],
    "rrCudaIntersectNoAlloc": [_P, C.c_uint32, C.c_int, _P, C.c_uint32, C.c_int, _P, _P],
    "rrCudaGetNoAllocDeviceErrors": [_P, C.POINTER(C.c_uint32)],
    "rrCudaAutotuneTraversal": [_P, _P, C.c_int, _P, C.c_uint32, C.c_int, _P, _P,
                                C.POINTER(RRCudaTraversalOptions)],
    "rrCudaAutotuneNodeFormat": [_P, C.POINTER(RRGeometryBuildInput), C.POINTER(RRBuildOptions), C.c_int, _P,
                                 C.c_uint32, C.c_int, _P, _P, C.POINTER(C.c_uint32)],
    "rrCudaCmdBuildGeometries": [_P, C.c_uint32, C.POINTER(RRGeometryBuildInput), C.POINTER(RRBuildOptions), _PP,
                                 _PP, _P],
    "rrCudaGetIntersectBatchMemoryRequirements": [_P, C.c_uint32, C.c_uint32, C.POINTER(C.c_size_t)],
    "rrCudaCmdIntersectHostBuffers": [_P, _P, C.c_int, _P, C.c_uint32, C.c_int, _P, _P, _P, _P, C.c_uint32, _P],
    "rrCudaRegisterGeometry": [_P, _P, C.c_uint32],
    "rrCudaCmdIntersectBatchHost": [_P, C.c_uint32, C.POINTER(RRCudaHostIntersectRequest), _P, _P, _P, _P],
    "rrCudaCmdIntersectBatch": [_P, C.c_uint32, C.POINTER(RRCudaIntersectRequest), _P, _P],
}

_LIB = None


def lib(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load librr.so (built by radeonrays_sdk_gb300.build) and bind every entry point."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: run radeonrays_sdk_gb300.build.build() (no CPU fallback exists)")
    L = C.CDLL(str(p))
    for name, args in PROTOTYPES.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = C.c_int
    if path is None:
        _LIB = L
    return L


def check(code: int, where: str) -> None:
    if code != RR_SUCCESS:
        raise RRException(code, where)


# ---- convenience layer -----------------------------------------------------
def _torch():
    import torch  # noqa: WPS433 (plumbing: device memory and streams)
    return torch


class Context:
    """One RRContext on the current CUDA device, with helpers that allocate
    device buffers through PyTorch and call the C-ABI."""

    def __init__(self):
        self.L = lib()
        self.ctx = C.c_void_p()
        check(self.L.rrCreateContext(RR_API_VERSION, RR_API_CUDA, C.byref(self.ctx)), "rrCreateContext")
        self._ptrs = []

    # -- handles
    def ptr(self, t, offset: int = 0) -> C.c_void_p:
        addr = t if isinstance(t, int) else t.data_ptr()
        h = C.c_void_p()
        check(self.L.rrGetDevicePtrFromCudaPtr(self.ctx, C.c_void_p(addr), offset, C.byref(h)), "rrGetDevicePtrFromCudaPtr")
        self._ptrs.append(h)
        return h

    def command_stream(self) -> C.c_void_p:
        s = C.c_void_p()
        check(self.L.rrAllocateCommandStream(self.ctx, C.byref(s)), "rrAllocateCommandStream")
        return s

    def external_stream(self, cuda_stream) -> C.c_void_p:
        s = C.c_void_p()
        handle = cuda_stream.cuda_stream if hasattr(cuda_stream, "cuda_stream") else int(cuda_stream)
        check(self.L.rrGetCommandStreamFromCudaStream(self.ctx, C.c_void_p(handle), C.byref(s)),
              "rrGetCommandStreamFromCudaStream")
        return s

    def submit(self, stream, wait: bool = True, wait_event=None):
        ev = C.c_void_p()
        check(self.L.rrSumbitCommandStream(self.ctx, stream, wait_event, C.byref(ev)), "rrSumbitCommandStream")
        if wait:
            check(self.L.rrWaitEvent(self.ctx, ev), "rrWaitEvent")
            check(self.L.rrReleaseEvent(self.ctx, ev), "rrReleaseEvent")
            return None
        return ev

    def release_stream(self, s):
        check(self.L.rrReleaseCommandStream(self.ctx, s), "rrReleaseCommandStream")

    # -- geometry
    @staticmethod
    def _build_input(vptr, nvert, stride, iptr, ntri, index16):
        mesh = RRTriangleMeshPrimitive(vptr, nvert, stride, iptr, ntri,
                                       RR_INDEX_TYPE_UINT16 if index16 else RR_INDEX_TYPE_UINT32)
        bi = RRGeometryBuildInput(RR_PRIMITIVE_TYPE_TRIANGLE_MESH, 1, C.pointer(mesh))
        return bi, mesh

    @staticmethod
    def _options(node_format=RR_CUDA_NODE_FORMAT_BVH4Q8, morton_bits=30, quality=False):
        """quality=True clears RR_BUILD_FLAG_BITS_PREFER_FAST_BUILD: the build adds the treelet restructure."""
        cuda_opts = RRCudaBuildOptions(C.sizeof(RRCudaBuildOptions), node_format, morton_bits, 0)
        flags = 0 if quality else RR_BUILD_FLAG_BITS_PREFER_FAST_BUILD
        opts = RRBuildOptions(flags, C.cast(C.pointer(cuda_opts), C.c_void_p))
        return opts, cuda_opts

    def geometry_requirements(self, ntri, node_format=RR_CUDA_NODE_FORMAT_BVH4Q8, morton_bits=30, nvert=0, stride=12,
                              index16=False):
        bi, mesh = self._build_input(None, nvert, stride, None, ntri, index16)
        opts, keep = self._options(node_format, morton_bits)
        req = RRMemoryRequirements()
        check(self.L.rrGetGeometryBuildMemoryRequirements(self.ctx, C.byref(bi), C.byref(opts), C.byref(req)),
              "rrGetGeometryBuildMemoryRequirements")
        return req.temporary_build_buffer_size, req.result_buffer_size

    def build_geometry(self, vertices, indices, node_format=RR_CUDA_NODE_FORMAT_BVH4Q8, morton_bits=30,
                       stride=None, stream=None, scratch=None, result=None, quality=False):
        """vertices: cuda float32 tensor (V, k>=3) or flat; indices: cuda int32/int16 (T, 3).
        quality=True: build flags without PREFER_FAST_BUILD (treelet restructure)."""
        torch = _torch()
        index16 = indices.dtype == torch.int16
        ntri = indices.numel() // 3
        stride = stride if stride is not None else (vertices.shape[-1] * 4 if vertices.dim() == 2 else 12)
        nvert = vertices.numel() * 4 // stride
        s_bytes, r_bytes = self.geometry_requirements(ntri, node_format, morton_bits, nvert, stride, index16)
        dev = vertices.device
        if scratch is None:
            scratch = torch.empty(max(s_bytes, 256), dtype=torch.uint8, device=dev)
        if result is None:
            result = torch.empty(r_bytes, dtype=torch.uint8, device=dev)
        bi, mesh = self._build_input(self.ptr(vertices) if ntri else None, nvert, stride,
                                     self.ptr(indices) if ntri else None, ntri, index16)
        opts, keep = self._options(node_format, morton_bits, quality)
        own = stream is None
        cs = self.command_stream() if own else stream
        check(self.L.rrCmdBuildGeometry(self.ctx, RR_BUILD_OPERATION_BUILD, C.byref(bi), C.byref(opts),
                                        self.ptr(scratch), self.ptr(result), cs), "rrCmdBuildGeometry")
        if own:
            self.submit(cs)
            self.release_stream(cs)
        return result

    def _aabb_input(self, boxes, stride):
        n = boxes.numel() * 4 // stride if boxes.numel() else 0
        prim = RRAABBListPrimitive(self.ptr(boxes) if n else None, n, stride)
        bi = RRGeometryBuildInput(RR_PRIMITIVE_TYPE_AABB_LIST, 1,
                                  C.cast(C.pointer(prim), C.POINTER(RRTriangleMeshPrimitive)))
        return bi, prim, n

    def build_aabbs(self, boxes, stride=32, quality=False, stream=None, update_of=None):
        """Build (or, with update_of = an earlier result, update) an AABB list: `boxes` is a cuda float32
        tensor of (min.x, min.y, min.z, _, max.x, max.y, max.z, _) records `stride` bytes apart."""
        torch = _torch()
        bi, prim, n = self._aabb_input(boxes, stride)
        opts, keep = self._options(RR_CUDA_NODE_FORMAT_BINARY, 30, quality)
        req = RRMemoryRequirements()
        check(self.L.rrGetGeometryBuildMemoryRequirements(self.ctx, C.byref(bi), C.byref(opts), C.byref(req)),
              "rrGetGeometryBuildMemoryRequirements")
        op = RR_BUILD_OPERATION_UPDATE if update_of is not None else RR_BUILD_OPERATION_BUILD
        s_bytes = req.temporary_update_buffer_size if update_of is not None else req.temporary_build_buffer_size
        scratch = torch.empty(max(s_bytes, 256), dtype=torch.uint8, device="cuda")
        result = update_of if update_of is not None else torch.empty(req.result_buffer_size, dtype=torch.uint8,
                                                                      device="cuda")
        own = stream is None
        cs = self.command_stream() if own else stream
        check(self.L.rrCmdBuildGeometry(self.ctx, op, C.byref(bi), C.byref(opts), self.ptr(scratch),
                                        self.ptr(result), cs), "rrCmdBuildGeometry(aabb list)")
        if own:
            self.submit(cs)
            self.release_stream(cs)
        else:
            self._keep = (scratch, bi, prim)
        return result

    def update_geometry(self, vertices, indices, result, stream=None, scratch=None):
        """RR_BUILD_OPERATION_UPDATE of `result` (built on this context from a mesh with the same triangle
        count) with new vertex positions: leaves take the new vertices, boxes are refitted, wide nodes are
        collapsed again."""
        torch = _torch()
        ntri = indices.numel() // 3
        nvert = vertices.numel() // 3
        bi, mesh = self._build_input(self.ptr(vertices) if ntri else None, nvert, 12,
                                     self.ptr(indices) if ntri else None, ntri, indices.dtype == torch.int16)
        req = RRMemoryRequirements()
        opts, keep = self._options()
        check(self.L.rrGetGeometryBuildMemoryRequirements(self.ctx, C.byref(bi), C.byref(opts), C.byref(req)),
              "rrGetGeometryBuildMemoryRequirements")
        if scratch is None and req.temporary_update_buffer_size:
            scratch = torch.empty(req.temporary_update_buffer_size, dtype=torch.uint8, device=vertices.device)
        own = stream is None
        cs = self.command_stream() if own else stream
        check(self.L.rrCmdBuildGeometry(self.ctx, RR_BUILD_OPERATION_UPDATE, C.byref(bi), C.byref(opts),
                                        self.ptr(scratch) if scratch is not None else None, self.ptr(result), cs),
              "rrCmdBuildGeometry(update)")
        if own:
            self.submit(cs)
            self.release_stream(cs)
        return result

    def build_geometries(self, meshes, node_format=RR_CUDA_NODE_FORMAT_BVH4Q8, morton_bits=30, stream=None,
                         api="batch", quality=False):
        """Build many meshes [(vertices (V, 3) float32, indices (T, 3) int32), ...] (cuda tensors).

        api "batch": one rrCudaCmdBuildGeometries call (one fused build);
        "record": one rrCmdBuildGeometry per mesh on an internal command
        stream (fused when the stream is submitted); "separate": one
        rrCmdBuildGeometry per mesh on an external stream (each runs alone).
        Scratch and results are slices of two device buffers at 256-byte
        offsets.  Returns the list of result tensors (views)."""
        torch = _torch()
        n = len(meshes)
        opts, keep = self._options(node_format, morton_bits, quality)
        reqs, inputs = [], []
        for v, i in meshes:
            ntri = i.numel() // 3
            bi, mesh = self._build_input(self.ptr(v) if ntri else None, v.numel() // 3, 12,
                                         self.ptr(i) if ntri else None, ntri, False)
            inputs.append((bi, mesh))
            req = RRMemoryRequirements()
            check(self.L.rrGetGeometryBuildMemoryRequirements(self.ctx, C.byref(bi), C.byref(opts), C.byref(req)),
                  "rrGetGeometryBuildMemoryRequirements")
            reqs.append((req.temporary_build_buffer_size, req.result_buffer_size))
        al = lambda x: (x + 255) // 256 * 256  # noqa: E731
        s_off = np.cumsum([0] + [al(s) for s, _ in reqs])
        r_off = np.cumsum([0] + [al(r) for _, r in reqs])
        dev = meshes[0][0].device if n else torch.device("cuda")
        scratch = torch.empty(max(int(s_off[-1]), 256), dtype=torch.uint8, device=dev)
        result = torch.empty(max(int(r_off[-1]), 256), dtype=torch.uint8, device=dev)
        s_ptrs = [self.ptr(scratch, int(s_off[k])) for k in range(n)]
        r_ptrs = [self.ptr(result, int(r_off[k])) for k in range(n)]
        if api == "separate":
            cs = self.external_stream(torch.cuda.current_stream(dev))
            for k in range(n):
                check(self.L.rrCmdBuildGeometry(self.ctx, RR_BUILD_OPERATION_BUILD, C.byref(inputs[k][0]),
                                                C.byref(opts), s_ptrs[k], r_ptrs[k], cs), "rrCmdBuildGeometry")
            torch.cuda.current_stream(dev).synchronize()
            check(self.L.rrReleaseExternalCommandStream(self.ctx, cs), "rrReleaseExternalCommandStream")
        else:
            own = stream is None
            cs = self.command_stream() if own else stream
            if api == "batch":
                arr = (RRGeometryBuildInput * max(n, 1))(*[b for b, _ in inputs])
                sp = (C.c_void_p * max(n, 1))(*[p.value for p in s_ptrs])
                rp = (C.c_void_p * max(n, 1))(*[p.value for p in r_ptrs])
                check(self.L.rrCudaCmdBuildGeometries(self.ctx, n, arr, C.byref(opts), sp, rp, cs),
                      "rrCudaCmdBuildGeometries")
            else:
                for k in range(n):
                    check(self.L.rrCmdBuildGeometry(self.ctx, RR_BUILD_OPERATION_BUILD, C.byref(inputs[k][0]),
                                                    C.byref(opts), s_ptrs[k], r_ptrs[k], cs), "rrCmdBuildGeometry")
            if own:
                self.submit(cs)
                self.release_stream(cs)
        self._keep = (scratch, inputs)
        return [result[int(r_off[k]): int(r_off[k]) + reqs[k][1]] for k in range(n)]

    def scene_build_input(self, geometries, transforms):
        """The RRSceneBuildInput of `geometries` (result tensors) placed by
        `transforms` ((I, 3, 4) object->world); keep the returned instance
        array alive while the input is in use."""
        n = len(geometries)
        inst = (RRInstance * max(n, 1))()
        tf = np.asarray(transforms, dtype=np.float32).reshape(n, 3, 4) if n else np.zeros((0, 3, 4), np.float32)
        rec = np.zeros(max(n, 1), dtype=np.dtype([("geometry", "<u8"), ("transform", "<f4", (3, 4))]))
        assert rec.itemsize == C.sizeof(RRInstance)
        rec["geometry"][:n] = [self.ptr(g).value or 0 for g in geometries]
        rec["transform"][:n] = tf
        C.memmove(inst, rec.ctypes.data, rec.nbytes)
        return RRSceneBuildInput(inst, n), inst

    def build_scene(self, geometries, transforms, stream=None):
        """geometries: list of result tensors; transforms: (I, 3, 4) float array (object->world)."""
        torch = _torch()
        n = len(geometries)
        sbi, inst = self.scene_build_input(geometries, transforms)
        req = RRMemoryRequirements()
        check(self.L.rrGetSceneBuildMemoryRequirements(self.ctx, C.byref(sbi), None, C.byref(req)),
              "rrGetSceneBuildMemoryRequirements")
        dev = geometries[0].device if n else torch.device("cuda")
        scratch = torch.empty(max(req.temporary_build_buffer_size, 256), dtype=torch.uint8, device=dev)
        result = torch.empty(req.result_buffer_size, dtype=torch.uint8, device=dev)
        own = stream is None
        cs = self.command_stream() if own else stream
        check(self.L.rrCmdBuildScene(self.ctx, C.byref(sbi), None, self.ptr(scratch), self.ptr(result), cs),
              "rrCmdBuildScene")
        if own:
            self.submit(cs)
            self.release_stream(cs)
        return result

    def trace_scratch_bytes(self, ray_count: int) -> int:
        sz = C.c_size_t()
        check(self.L.rrGetTraceMemoryRequirements(self.ctx, ray_count, C.byref(sz)), "rrGetTraceMemoryRequirements")
        return sz.value

    def cmd_intersect(self, bvh, rays, ray_count, hits, scratch, stream, query=RR_INTERSECT_QUERY_CLOSEST,
                      output=RR_INTERSECT_QUERY_OUTPUT_FULL_HIT, indirect=None):
        check(self.L.rrCmdIntersect(self.ctx, self.ptr(bvh), query, self.ptr(rays), ray_count,
                                    self.ptr(indirect) if indirect is not None else None, output, self.ptr(hits),
                                    self.ptr(scratch), stream), "rrCmdIntersect")

    def intersect(self, bvh, rays, query=RR_INTERSECT_QUERY_CLOSEST, output=RR_INTERSECT_QUERY_OUTPUT_FULL_HIT,
                  hits=None, indirect=None, fill=0xFF):
        """rays: cuda float32 tensor (R, 8).  Returns the hits tensor (R, 4) int32/float32 bits or (R,) uint32."""
        torch = _torch()
        R = rays.shape[0]
        if hits is None:
            hits = torch.full((R, 4) if output == RR_INTERSECT_QUERY_OUTPUT_FULL_HIT else (R,), -1 if fill == 0xFF else 0,
                              dtype=torch.int32, device=rays.device)
        scratch = torch.empty(self.trace_scratch_bytes(max(R, 1)), dtype=torch.uint8, device=rays.device)
        cs = self.command_stream()
        self.cmd_intersect(bvh, rays, R, hits, scratch, cs, query, output, indirect)
        self.submit(cs)
        self.release_stream(cs)
        return hits

    def intersect_host(self, bvh, rays_host, query=RR_INTERSECT_QUERY_CLOSEST, output=RR_INTERSECT_QUERY_OUTPUT_FULL_HIT,
                       chunk_rays=0, staging=None, pinned_hits=True):
        """rays_host: CPU float32 tensor (R, 8), pinned for copy/compute overlap.  Returns the hits as a CPU
        int32 tensor ((R, 4) or (R,)) through one rrCudaCmdIntersectHostBuffers call.  `staging` may pass
        (rays_dev, hits_dev, scratch) to reuse device buffers; pinned_hits=False returns the hits in pageable
        memory."""
        torch = _torch()
        R = rays_host.shape[0]
        full = output == RR_INTERSECT_QUERY_OUTPUT_FULL_HIT
        hits_host = torch.full((R, 4) if full else (R,), -1, dtype=torch.int32)
        if pinned_hits:
            hits_host = hits_host.pin_memory()
        if staging is None:
            staging = (torch.empty((R, 8), dtype=torch.float32, device="cuda"),
                       torch.full((R, 4) if full else (R,), -1, dtype=torch.int32, device="cuda"),
                       torch.empty(self.trace_scratch_bytes(R), dtype=torch.uint8, device="cuda"))
        rd, hd, sc = staging
        cs = self.command_stream()
        check(self.L.rrCudaCmdIntersectHostBuffers(self.ctx, self.ptr(bvh), query, C.c_void_p(rays_host.data_ptr()), R,
                                                   output, C.c_void_p(hits_host.data_ptr()), self.ptr(rd),
                                                   self.ptr(hd), self.ptr(sc), chunk_rays, cs),
              "rrCudaCmdIntersectHostBuffers")
        self.submit(cs)
        self.release_stream(cs)
        return hits_host

    # -- many requests in one launch
    def batch_scratch_bytes(self, request_count: int, total_rays: int) -> int:
        n = C.c_size_t()
        check(self.L.rrCudaGetIntersectBatchMemoryRequirements(self.ctx, request_count, total_rays, C.byref(n)),
              "rrCudaGetIntersectBatchMemoryRequirements")
        return n.value

    def cmd_intersect_batch(self, reqs, scratch, stream):
        """reqs: [(bvh tensor, rays tensor (R, 8) or (ptr, R), hits tensor or ptr, query, output), ...] with
        device tensors or raw device addresses; records one rrCudaCmdIntersectBatch."""
        n = len(reqs)
        arr = (RRCudaIntersectRequest * n)()
        for k, (bvh, rays, hits, q, o) in enumerate(reqs):
            if isinstance(rays, tuple):
                rays_ptr, count = rays
            else:
                rays_ptr, count = rays, rays.shape[0]
            arr[k] = RRCudaIntersectRequest(self.ptr(bvh), q, o, self.ptr(rays_ptr) if count else None, count,
                                            self.ptr(hits) if count else None)
        check(self.L.rrCudaCmdIntersectBatch(self.ctx, n, arr, self.ptr(scratch), stream), "rrCudaCmdIntersectBatch")

    def intersect_batch(self, reqs):
        """reqs: [(bvh, rays (R, 8) cuda tensor, query, output), ...] -> list of hit tensors (one launch)."""
        torch = _torch()
        hits = []
        full = []
        for bvh, rays, q, o in reqs:
            R = rays.shape[0]
            h = torch.full((R, 4) if o == RR_INTERSECT_QUERY_OUTPUT_FULL_HIT else (R,), -1, dtype=torch.int32,
                           device=rays.device)
            hits.append(h)
            full.append((bvh, rays, h, q, o))
        total = sum(r.shape[0] for _, r, _, _ in reqs)
        scratch = torch.empty(self.batch_scratch_bytes(len(reqs), total), dtype=torch.uint8, device="cuda")
        cs = self.command_stream()
        self.cmd_intersect_batch(full, scratch, cs)
        self.submit(cs)
        self.release_stream(cs)
        return hits

    # -- options and diagnostics
    def set_traversal(self, traversal=RR_CUDA_TRAVERSAL_AUTO, block_size=0, blocks_per_sm=0, collect_stats=0,
                      ray_order=0, short_stack=0, triangle_test=RR_CUDA_TRIANGLE_TEST_REFERENCE):
        o = RRCudaTraversalOptions(C.sizeof(RRCudaTraversalOptions), traversal, block_size, blocks_per_sm,
                                   collect_stats, ray_order, short_stack, triangle_test)
        check(self.L.rrCudaSetTraversalOptions(self.ctx, C.byref(o)), "rrCudaSetTraversalOptions")

    def autotune(self, bvh, rays, query=RR_INTERSECT_QUERY_CLOSEST, output=RR_INTERSECT_QUERY_OUTPUT_FULL_HIT,
                 hits=None, scratch=None) -> dict:
        """Time the applicable traversal kernels on `rays` and select the
        fastest for this context (rrCudaAutotuneTraversal)."""
        torch = _torch()
        R = rays.shape[0]
        if hits is None:
            hits = torch.empty((R, 4) if output == RR_INTERSECT_QUERY_OUTPUT_FULL_HIT else (R,), dtype=torch.int32,
                               device=rays.device)
        if scratch is None:
            scratch = torch.empty(self.trace_scratch_bytes(R), dtype=torch.uint8, device=rays.device)
        o = RRCudaTraversalOptions()
        check(self.L.rrCudaAutotuneTraversal(self.ctx, self.ptr(bvh), query, self.ptr(rays), R, output,
                                             self.ptr(hits), self.ptr(scratch), C.byref(o)),
              "rrCudaAutotuneTraversal")
        return {"traversal": o.traversal, "ray_order": o.ray_order, "blocks_per_sm": o.blocks_per_sm,
                "short_stack": o.short_stack}

    def autotune_node_format(self, vertices, indices, rays, query=RR_INTERSECT_QUERY_CLOSEST,
                             output=RR_INTERSECT_QUERY_OUTPUT_FULL_HIT, quality=False) -> int:
        """rrCudaAutotuneNodeFormat: build the mesh in the 4-wide and the 8-wide
        format, tune the traversal of each on `rays`, remember the faster width
        for meshes of this size (RR_CUDA_NODE_FORMAT_AUTO builds use it) and
        return it."""
        torch = _torch()
        ntri = indices.numel() // 3
        bi, mesh = self._build_input(self.ptr(vertices), vertices.numel() // 3, 12, self.ptr(indices), ntri,
                                     indices.dtype == torch.int16)
        opts, keep = self._options(RR_CUDA_NODE_FORMAT_AUTO, 30, quality)
        R = rays.shape[0]
        hits = torch.empty((R, 4) if output == RR_INTERSECT_QUERY_OUTPUT_FULL_HIT else (R,), dtype=torch.int32,
                           device=rays.device)
        scratch = torch.empty(self.trace_scratch_bytes(R), dtype=torch.uint8, device=rays.device)
        fmt = C.c_uint32()
        check(self.L.rrCudaAutotuneNodeFormat(self.ctx, C.byref(bi), C.byref(opts), query, self.ptr(rays), R, output,
                                              self.ptr(hits), self.ptr(scratch), C.byref(fmt)),
              "rrCudaAutotuneNodeFormat")
        return fmt.value

    def set_wait_limits(self, lookback_polls=0, arrival_polls=0, hold_sort_tile=RR_INVALID,
                        drop_arrival_chunk=RR_INVALID):
        """Limits of the bounded device waits, and the test hooks that make
        them run out (rrCudaSetWaitLimits); no arguments restore the defaults."""
        w = RRCudaWaitLimits(C.sizeof(RRCudaWaitLimits), lookback_polls, arrival_polls, hold_sort_tile,
                             drop_arrival_chunk)
        check(self.L.rrCudaSetWaitLimits(self.ctx, C.byref(w)), "rrCudaSetWaitLimits")

    def device_errors(self) -> int:
        v = C.c_uint32()
        check(self.L.rrCudaGetDeviceErrors(self.ctx, C.byref(v)), "rrCudaGetDeviceErrors")
        return v.value

    def stats(self) -> dict:
        s = RRCudaTraversalStats()
        check(self.L.rrCudaGetTraversalStats(self.ctx, C.byref(s)), "rrCudaGetTraversalStats")
        return {"rays": s.rays, "node_fetches": s.node_fetches, "triangle_fetches": s.triangle_fetches}

    def close(self):
        if self.ctx:
            for h in self._ptrs:
                self.L.rrReleaseDevicePtr(self.ctx, h)
            self._ptrs.clear()
            check(self.L.rrDestroyContext(self.ctx), "rrDestroyContext")
            self.ctx = C.c_void_p()

    def release_ptrs(self):
        for h in self._ptrs:
            self.L.rrReleaseDevicePtr(self.ctx, h)
        self._ptrs.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def read_trailer(result_u8_cpu: np.ndarray, leaf_count: int, scene: bool = False) -> np.ndarray:
    """Decode the trailer of a result buffer copied to the host."""
    if scene:
        nodes = 0 if leaf_count == 0 else (2 * leaf_count - 1) * 64
        off = (nodes + 2 * leaf_count * 48 + 255) // 256 * 256
    else:
        nodes = 0 if leaf_count == 0 else (2 * leaf_count - 1) * 64
        off = (nodes + 255) // 256 * 256
    return np.frombuffer(result_u8_cpu[off:off + 256].tobytes(), dtype=TRAILER_DTYPE)[0]
