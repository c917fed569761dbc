"""GPU RR_BUILD_OPERATION_UPDATE: new vertex positions on an existing tree.
Binary nodes bit-identical to the oracle's refit of the same topology,
traversal of the updated tree equal to the oracle's, 8-wide nodes collapsed
again, 4-wide nodes (either form) requantised in place with their topology,
argument checks."""
import numpy as np
import pytest

from gpu_util import INVALID, hits_np, nodes_of, tie_only_mismatch, to_dev, trace, trailer_of
from test_gpu_build import same_nodes

pytestmark = pytest.mark.gpu


def _bvh4_children(res, n, fmt):
    """The child references of the buffer's 4-wide nodes (fp32: 128-byte nodes, references at byte 96; 8-bit:
    64-byte nodes, references at byte 16)."""
    tr = trailer_of(res, n)
    size, off = (128, 96) if fmt == 2 else (64, 16)
    raw = res.cpu().numpy().view(np.uint8)
    base = int(tr["wide_nodes_off"])
    cnt = int(tr["wide_count"])
    nodes = raw[base: base + cnt * size].reshape(cnt, size)
    return nodes[:, off: off + 16].copy().view(np.uint32)


def _moved(v, seed):
    g = np.random.default_rng(seed)
    return (v * np.float32(1.5) + g.normal(0, 0.003, size=v.shape).astype(np.float32)).astype(np.float32)


@pytest.mark.parametrize("fmt", [0, 1, 2, 4])
@pytest.mark.parametrize("n", [1, 2, 3, 1000, 40000])
def test_update_matches_oracle_refit(ctx, orc, fmt, n):
    from radeonrays_sdk_gb300 import scenes
    v, i = scenes.soup(n, scenes.rng(70, n))
    res = ctx.build_geometry(to_dev(v), to_dev(i), node_format=fmt)
    old = nodes_of(res, n).copy()
    before4 = _bvh4_children(res, n, fmt) if fmt in (2, 4) and n > 3 else None
    v2 = _moved(v, n)
    ctx.update_geometry(to_dev(v2), to_dev(i), res)
    want = orc.fit(orc.build_mesh(v, i)[0], v2, i)
    got = nodes_of(res, n)
    assert same_nodes(got, want)
    # Topology unchanged, boxes changed.
    assert np.array_equal(got["child0"], old["child0"]) and np.array_equal(got["child1"], old["child1"])
    assert ctx.device_errors() == 0
    if fmt == 1:
        tr = trailer_of(res, n)
        assert tr["wide_tri_count"] == n and tr["wide_count"] >= 1
    rays = scenes.incoherent_rays(4096, v2.min(axis=0), v2.max(axis=0), scenes.rng(70, 1))
    ref = orc.trace(want, rays)
    assert np.array_equal(trace(ctx, res, rays, traversal=1), ref)
    assert np.array_equal(trace(ctx, res, rays, traversal=3), ref)
    if fmt in (1, 2, 4):
        # The wide nodes follow the new boxes: 8-wide collapsed again, 4-wide
        # requantised with their topology.  Hit flags are the reference's and
        # primitive ids differ only at equal-t ties.
        wide = trace(ctx, res, rays, traversal=2 if fmt == 1 else 4)
        assert np.array_equal(wide[:, 2] != INVALID, ref[:, 2] != INVALID)
        tie_only_mismatch(orc, rays, wide, ref, v2, i)
    if fmt in (2, 4) and n > 3:
        # The 4-wide topology is kept: child references unchanged.
        assert np.array_equal(_bvh4_children(res, n, fmt), before4)


def test_update_twice_back_to_original(ctx, orc):
    """Updating back to the original positions restores the built tree."""
    from radeonrays_sdk_gb300 import scenes
    v, i = scenes.heightfield(65, scenes.rng(71))
    n = i.shape[0]
    res = ctx.build_geometry(to_dev(v), to_dev(i), node_format=1)
    built = nodes_of(res, n).copy()
    ctx.update_geometry(to_dev(_moved(v, 3)), to_dev(i), res)
    ctx.update_geometry(to_dev(v), to_dev(i), res)
    assert same_nodes(nodes_of(res, n), built)
    rays = scenes.incoherent_rays(2048, v.min(axis=0), v.max(axis=0), scenes.rng(71, 1))
    assert np.array_equal(trace(ctx, res, rays, traversal=1), orc.trace(orc.build_mesh(v, i)[0], rays))


def test_update_argument_checks(ctx):
    from radeonrays_sdk_gb300 import rr, scenes
    v, i = scenes.soup(100, scenes.rng(72))
    res = ctx.build_geometry(to_dev(v), to_dev(i), node_format=0)
    v3, i3 = scenes.soup(101, scenes.rng(73))
    with pytest.raises(rr.RRException) as e:
        ctx.update_geometry(to_dev(v3), to_dev(i3), res)  # triangle count differs
    assert e.value.code == rr.RR_ERROR_INVALID_PARAMETER
    import torch
    stranger = torch.zeros(res.numel(), dtype=torch.uint8, device="cuda")
    with pytest.raises(rr.RRException) as e:
        ctx.update_geometry(to_dev(v), to_dev(i), stranger)  # never built on this context
    assert e.value.code == rr.RR_ERROR_INVALID_PARAMETER
