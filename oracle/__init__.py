"""Python view of the CPU oracle (liboracle.so) and of the harness around the
reference's own CPU traversal (_ref/librr_ref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product (radeonrays_sdk_gb300).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REF = HERE / "_ref" / "librr_ref.so"
# The reference checkout, named only by the environment (no default): where it
# is unset, the harness around the reference's own traversal is not built and
# the checks that need it skip.
_REF_ROOT = os.environ.get("RR_REFERENCE_DIR")
REF_DIR = Path(_REF_ROOT) / "bvh_analyzer" if _REF_ROOT else None

NODE_DTYPE = np.dtype([("a0", "<f4", 3), ("child0", "<u4"), ("a1", "<f4", 3), ("child1", "<u4"),
                       ("b0", "<f4", 3), ("parent", "<u4"), ("b1", "<f4", 3), ("update", "<u4")])
INVALID = 0xFFFFFFFF

_lib = None
_ref = None


def build() -> None:
    """Compile liboracle.so (and _ref/librr_ref.so where the reference checkout exists)."""
    args = ["make", "-s", "-C", str(HERE)]
    if REF_DIR is not None:
        args.append(f"REF_DIR={REF_DIR}")
    subprocess.run(args, check=True)


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        _lib = C.CDLL(str(LIB))
        for name in ("rro_mesh_aabb", "rro_morton", "rro_sort32", "rro_sort64", "rro_emit", "rro_fit",
                     "rro_build_mesh", "rro_trace", "rro_build_scene", "rro_trace_scene", "rro_fp64_hit",
                     "rro_trace_t", "rro_tri_test", "rro_trace_leaves", "rro_trace_precise",
                     "rro_tri_test_precise"):
            getattr(_lib, name).restype = None
    return _lib


def ref_lib():
    """The reference's bvh_analyzer traversal, or None where it was not built."""
    global _ref
    if _ref is None and REF.exists():
        _ref = C.CDLL(str(REF))
        _ref.rrref_trace.restype = C.c_double
        _ref.rrref_trace.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint32, C.c_int, C.c_void_p,
                                     C.c_int]
        _ref.rrref_validate.restype = C.c_int
        _ref.rrref_validate.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.POINTER(C.c_float)]
    return _ref


def _mesh(vertices, indices):
    v = np.ascontiguousarray(vertices, dtype=np.float32)
    idx16 = indices.dtype == np.uint16
    i = np.ascontiguousarray(indices, dtype=np.uint16 if idx16 else np.uint32)
    stride = v.shape[1] * 4 if v.ndim == 2 else 12
    return v, i, stride, int(idx16)


def mesh_aabb(vertices, indices):
    v, i, stride, i16 = _mesh(vertices, indices)
    out = np.zeros(8, dtype=np.uint32)
    lib().rro_mesh_aabb(_p(v), C.c_uint32(stride), _p(i), C.c_int(i16), C.c_uint32(i.size // 3), _p(out))
    return out


def morton(vertices, indices, aabb, bits=30):
    v, i, stride, i16 = _mesh(vertices, indices)
    n = i.size // 3
    codes = np.zeros(n, dtype=np.uint64 if bits == 63 else np.uint32)
    lib().rro_morton(_p(v), C.c_uint32(stride), _p(i), C.c_int(i16), C.c_uint32(n), _p(aabb), C.c_int(bits), _p(codes))
    return codes


def sort(codes):
    n = codes.size
    sc = np.zeros_like(codes)
    si = np.zeros(n, dtype=np.uint32)
    fn = lib().rro_sort64 if codes.dtype == np.uint64 else lib().rro_sort32
    fn(_p(np.ascontiguousarray(codes)), C.c_uint32(n), _p(sc), _p(si))
    return sc, si


def fit(nodes, vertices, indices):
    """Refit of an existing tree with new vertex positions (the update path,
    lbvh_fit_aabb_mesh.comp with UPDATE_KERNEL): every leaf takes the vertices
    of its primitive (child1), then boxes are rebuilt bottom-up.  Returns a copy."""
    v, i, stride, i16 = _mesh(vertices, indices)
    n = i.size // 3
    out = np.array(nodes, dtype=NODE_DTYPE, copy=True)
    if n:
        lib().rro_fit(_p(v), C.c_uint32(stride), _p(i), C.c_int(i16), C.c_uint32(n), _p(out))
    return out


def restructure(nodes, n, min_prims=64, passes=3):
    """Treelet restructure of a built tree (rro_restructure).  Returns
    (new nodes, number of treelets changed)."""
    out = np.array(nodes, dtype=NODE_DTYPE, copy=True)
    f = lib().rro_restructure
    f.restype = C.c_uint32
    changed = f(_p(out), C.c_uint32(n), C.c_uint32(min_prims), C.c_int(passes)) if n >= 3 else 0
    return out, int(changed)


def build_mesh(vertices, indices, bits=30, threads=8):
    """Full LBVH build.  Returns (nodes, sorted_idx, sorted_codes)."""
    v, i, stride, i16 = _mesh(vertices, indices)
    n = i.size // 3
    nodes = np.zeros(max(2 * n - 1, 0), dtype=NODE_DTYPE)
    sidx = np.zeros(n, dtype=np.uint32)
    scodes = np.zeros(n, dtype=np.uint64 if bits == 63 else np.uint32)
    if n:
        lib().rro_build_mesh(_p(v), C.c_uint32(stride), _p(i), C.c_int(i16), C.c_uint32(n), C.c_int(bits), _p(nodes),
                             _p(sidx), _p(scodes), C.c_int(threads))
    return nodes, sidx, scodes


def trace(nodes, rays, query=0, output=0, threads=8, hits=None, fetches=False, box_leaves=False):
    """isect.comp semantics.  Full output: (R, 4) uint32 view of RRHit
    (pre-filled with 0xFFFFFFFF unless `hits` is given); instance output: (R,) uint32.
    box_leaves: the tree of an AABB list (leaf = box, hit at the slab entry distance, uv = 0)."""
    R = rays.shape[0]
    r = np.ascontiguousarray(rays, dtype=np.float32)
    if hits is None:
        hits = np.full((R, 4) if output == 0 else (R,), INVALID, dtype=np.uint32)
    f = np.zeros(R, dtype=np.uint64) if fetches else None
    lib().rro_trace_leaves(_p(nodes), C.c_uint32(nodes.size), _p(r), C.c_uint32(R), C.c_int(query),
                           C.c_int(output), _p(hits), _p(f), C.c_int(threads), C.c_int(1 if box_leaves else 0))
    return (hits, f) if fetches else hits


def trace_precise(nodes, rays, query=0, output=0, threads=8):
    """The precise triangle test's traversal (watertight decision, accurate t
    and uv, robust box test) in the reference's visit order: the twin of the
    kernels' RR_CUDA_TRIANGLE_TEST_WATERTIGHT mode.  Returns (hits, t) with t
    the fp32 distance of each closest (any: first) hit, +inf on a miss."""
    R = rays.shape[0]
    hits = np.full((R, 4) if output == 0 else (R,), INVALID, dtype=np.uint32)
    t = np.full(R, np.inf, dtype=np.float32)
    lib().rro_trace_precise(_p(nodes), C.c_uint32(nodes.size), _p(np.ascontiguousarray(rays, np.float32)),
                            C.c_uint32(R), C.c_int(query), C.c_int(output), _p(hits), _p(t), C.c_int(threads))
    return hits, t


def tri_test_precise(rays, tri9):
    R = rays.shape[0]
    out = np.zeros((R, 3), dtype=np.float32)
    lib().rro_tri_test_precise(_p(np.ascontiguousarray(rays, np.float32)), _p(np.ascontiguousarray(tri9, np.float32)),
                               C.c_uint32(R), _p(out))
    return out


def aabb_vertices(boxes):
    """An AABB list (n, 2, 4) or (n, 8) float32 [(min.xyz, _), (max.xyz, _)] as
    the three leaf vertices the build stores for each box: (min, max, max)."""
    b = np.asarray(boxes, dtype=np.float32).reshape(-1, 8)
    lo, hi = b[:, 0:3], b[:, 4:7]
    v = np.stack([lo, hi, hi], axis=1).reshape(-1, 3)
    i = np.arange(v.shape[0], dtype=np.uint32).reshape(-1, 3)
    return np.ascontiguousarray(v), i


def build_aabbs(boxes, bits=30, threads=8):
    """LBVH build of an AABB list: the mesh build over each box's (min, max,
    max) leaf vertices -- same bounds (box min/max), same Morton input (box
    centre) and the leaf layout the GPU writes.  Returns (nodes, sorted_idx, sorted_codes)."""
    v, i = aabb_vertices(boxes)
    return build_mesh(v, i, bits=bits, threads=threads)


def trace_t(nodes, rays, threads=8):
    R = rays.shape[0]
    out = np.zeros(R, dtype=np.float32)
    lib().rro_trace_t(_p(nodes), C.c_uint32(nodes.size), _p(np.ascontiguousarray(rays, np.float32)), C.c_uint32(R),
                      _p(out), C.c_int(threads))
    return out


def fp64_hit(rays, tri9, valid):
    R = rays.shape[0]
    out = np.zeros((R, 3), dtype=np.float64)
    lib().rro_fp64_hit(_p(np.ascontiguousarray(rays, np.float32)), _p(np.ascontiguousarray(tri9, np.float32)),
                       _p(np.ascontiguousarray(valid, np.uint32)), C.c_uint32(R), _p(out))
    return out


def tri_test(rays, tri9):
    R = rays.shape[0]
    out = np.zeros((R, 3), dtype=np.float32)
    lib().rro_tri_test(_p(np.ascontiguousarray(rays, np.float32)), _p(np.ascontiguousarray(tri9, np.float32)),
                       C.c_uint32(R), _p(out))
    return out


def build_scene(blas_nodes, blas_leaf_counts, transforms):
    n = len(blas_nodes)
    roots = (C.c_void_p * max(n, 1))()
    keep = []
    for k, nd in enumerate(blas_nodes):
        if nd is None or nd.size == 0:
            dummy = np.zeros(1, dtype=NODE_DTYPE)
            keep.append(dummy)
            roots[k] = dummy.ctypes.data
        else:
            roots[k] = nd.ctypes.data
    counts = np.ascontiguousarray(blas_leaf_counts, dtype=np.uint32)
    tf = np.ascontiguousarray(transforms, dtype=np.float32).reshape(n, 12)
    nodes = np.zeros(max(2 * n - 1, 0), dtype=NODE_DTYPE)
    xf = np.zeros((n, 24), dtype=np.float32)
    if n:
        lib().rro_build_scene(roots, _p(counts), _p(tf), C.c_uint32(n), _p(nodes), _p(xf))
    return nodes, xf


def trace_scene(tlas, xforms, blas_nodes, rays, query=0, output=0, threads=8):
    R = rays.shape[0]
    n = len(blas_nodes)
    ptrs = (C.c_void_p * max(n, 1))()
    for k, nd in enumerate(blas_nodes):
        ptrs[k] = nd.ctypes.data if (nd is not None and nd.size) else None
    hits = np.full((R, 4) if output == 0 else (R,), INVALID, dtype=np.uint32)
    lib().rro_trace_scene(_p(tlas), _p(np.ascontiguousarray(xforms, np.float32)), ptrs,
                          _p(np.ascontiguousarray(rays, np.float32)), C.c_uint32(R), C.c_int(query), C.c_int(output),
                          _p(hits), C.c_int(threads))
    return hits


def ref_trace(nodes, rays, any_hit=False, threads=8):
    """bvh_analyzer's BvhIntersect over `nodes` (Vulkan layout).  Returns
    ((R, 4) uint32 hits, seconds of the ray loop)."""
    L = ref_lib()
    if L is None:
        raise RuntimeError("reference harness not built (reference checkout absent)")
    n = (nodes.size + 1) // 2
    R = rays.shape[0]
    hits = np.zeros((R, 4), dtype=np.uint32)
    secs = L.rrref_trace(_p(nodes), n - 1, n, _p(np.ascontiguousarray(rays, np.float32)), R, int(any_hit), _p(hits),
                         threads)
    return hits, secs


def ref_validate(nodes):
    L = ref_lib()
    if L is None:
        raise RuntimeError("reference harness not built (reference checkout absent)")
    n = (nodes.size + 1) // 2
    sah = C.c_float()
    ok = L.rrref_validate(_p(nodes), n - 1, n, C.byref(sah))
    return bool(ok), float(sah.value)
