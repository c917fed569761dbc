"""Helpers shared by the GPU tests: move numpy inputs to the device, build
through the C-ABI, read result buffers back."""
import numpy as np

INVALID = 0xFFFFFFFF


def to_dev(a):
    import torch
    a = np.ascontiguousarray(a)
    if a.dtype == np.uint32:
        a = a.view(np.int32)
    elif a.dtype == np.uint16:
        a = a.view(np.int16)
    return torch.from_numpy(a).cuda()


def build(ctx, vertices, indices, node_format=1, morton_bits=30):
    from radeonrays_sdk_gb300 import rr
    return ctx.build_geometry(to_dev(vertices), to_dev(indices), node_format=node_format, morton_bits=morton_bits)


def nodes_of(result, n):
    from radeonrays_sdk_gb300 import rr
    raw = result[: max(2 * n - 1, 0) * 64].cpu().numpy()
    return raw.view(rr.NODE_DTYPE)


def trailer_of(result, n, scene=False):
    from radeonrays_sdk_gb300 import rr
    return rr.read_trailer(result.cpu().numpy(), n, scene=scene)


def hits_np(h):
    return h.cpu().numpy().view(np.uint32)


def trace(ctx, bvh, rays, query=0, output=0, traversal=0):
    ctx.set_traversal(traversal)
    h = ctx.intersect(bvh, to_dev(rays), query=query, output=output)
    ctx.set_traversal(0)
    return hits_np(h)


def tie_only_mismatch(orc, rays, a, b, vertices, indices, precise=False, near_ulp=0):
    """Rays where closest-hit primitives a and b differ must be ties: both
    triangles hit at the same fp32 distance (by the reference's triangle
    test, or the precise one).  near_ulp > 0 also admits distances within
    that many ulp: the reference's fp32 slab test can cull a triangle whose
    box entry rounds past the closest t found so far, so two visit orders
    can keep different triangles when their distances differ by an ulp."""
    diff = np.where(a[:, 3] != b[:, 3])[0]
    if diff.size == 0:
        return 0
    assert np.all(a[diff, 2] != INVALID) and np.all(b[diff, 2] != INVALID)
    idx = indices.astype(np.int64).reshape(-1, 3)
    test = orc.tri_test_precise if precise else orc.tri_test
    ta = test(rays[diff], vertices[idx[a[diff, 3]]].reshape(-1, 9))[:, 0]
    tb = test(rays[diff], vertices[idx[b[diff, 3]]].reshape(-1, 9))[:, 0]
    if near_ulp == 0:
        assert np.array_equal(ta, tb), (diff[:8], ta[:8], tb[:8])
    else:
        gap = np.abs(ta.astype(np.float64) - tb) / np.spacing(np.maximum(np.abs(ta), np.abs(tb))).astype(np.float64)
        assert np.all(gap <= near_ulp), (diff[gap > near_ulp][:8], ta[gap > near_ulp][:8], tb[gap > near_ulp][:8])
    return diff.size
