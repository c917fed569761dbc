"""GPU quality build (build flags without RR_BUILD_FLAG_BITS_PREFER_FAST_BUILD):
the treelet restructure gives binary nodes bit-identical to the oracle's
deterministic restatement (rro_restructure), for single and fused builds;
traversal of the restructured tree equals the oracle's on it and finds the
same hits as the fast build (primitive ids up to exact equal-t ties)."""
import numpy as np
import pytest

from gpu_util import INVALID, nodes_of, tie_only_mismatch, to_dev, trace
from test_gpu_build import same_nodes

pytestmark = pytest.mark.gpu


def _oracle_quality(orc, v, i):
    nodes, _, _ = orc.build_mesh(v, i)
    out, _ = orc.restructure(nodes, i.shape[0], 64, 3)
    return out


@pytest.mark.parametrize("n", [1, 2, 3, 100, 5000, 70000])
def test_quality_build_matches_oracle(ctx, orc, n):
    from radeonrays_sdk_gb300 import scenes
    v, i = scenes.soup(n, scenes.rng(100, n))
    res = ctx.build_geometry(to_dev(v), to_dev(i), node_format=1, quality=True)
    assert same_nodes(nodes_of(res, n), _oracle_quality(orc, v, i))
    assert ctx.device_errors() == 0


def test_quality_heightfield_traversal(ctx, orc):
    from radeonrays_sdk_gb300 import scenes
    v, i = scenes.heightfield(257, scenes.rng(101))
    n = i.shape[0]
    q = ctx.build_geometry(to_dev(v), to_dev(i), node_format=1, quality=True)
    want_nodes = _oracle_quality(orc, v, i)
    assert same_nodes(nodes_of(q, n), want_nodes)
    fast_nodes, _, _ = orc.build_mesh(v, i)
    assert not np.array_equal(want_nodes["child0"], fast_nodes["child0"])  # the pass did change the tree
    rays = scenes.incoherent_rays(20000, v.min(axis=0), v.max(axis=0), scenes.rng(101, 1))
    want = orc.trace(want_nodes, rays)
    for trav in (1, 3):
        assert np.array_equal(trace(ctx, q, rays, traversal=trav), want), trav
    fast = orc.trace(fast_nodes, rays)
    assert np.array_equal(want[:, 2] != INVALID, fast[:, 2] != INVALID)
    tie_only_mismatch(orc, rays, want, fast, v, i)
    wide = trace(ctx, q, rays, traversal=2)
    assert np.array_equal(wide[:, 2] != INVALID, want[:, 2] != INVALID)
    tie_only_mismatch(orc, rays, wide, want, v, i)
    assert ctx.device_errors() == 0


def test_quality_fused_build(ctx, orc):
    from radeonrays_sdk_gb300 import scenes
    sizes = [0, 1, 2, 5, 64, 65, 1000, 9000]
    ms = []
    for k, s in enumerate(sizes):
        ms.append((np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32)) if s == 0
                  else scenes.soup(s, scenes.rng(102, k)))
    res = ctx.build_geometries([(to_dev(v), to_dev(i)) for v, i in ms], node_format=1, quality=True)
    for (v, i), r in zip(ms, res):
        if i.shape[0]:
            assert same_nodes(nodes_of(r, i.shape[0]), _oracle_quality(orc, v, i)), i.shape[0]
    assert ctx.device_errors() == 0


def test_quality_build_then_update(ctx, orc):
    from radeonrays_sdk_gb300 import scenes
    v, i = scenes.soup(3000, scenes.rng(103))
    res = ctx.build_geometry(to_dev(v), to_dev(i), node_format=1, quality=True)
    v2 = (v * np.float32(0.5) + np.float32(3.0)).astype(np.float32)
    ctx.update_geometry(to_dev(v2), to_dev(i), res)
    want = orc.fit(_oracle_quality(orc, v, i), v2, i)
    assert same_nodes(nodes_of(res, 3000), want)


@pytest.mark.parametrize("bits", [30, 63])
def test_quality_build_default_format_and_key_widths(ctx, orc, bits):
    """The quality build in the default node format (8-bit 4-wide nodes) and
    with either key width: binary nodes bit-identical to the oracle's, and
    the collapsed nodes conservative over the restructured tree."""
    from radeonrays_sdk_gb300 import rr, scenes
    from test_gpu_bvh4q8 import check_conservative
    v, i = scenes.heightfield(321, scenes.rng(104, bits))
    n = i.shape[0]
    res = ctx.build_geometry(to_dev(v), to_dev(i), node_format=rr.RR_CUDA_NODE_FORMAT_BVH4Q8, morton_bits=bits,
                             quality=True)
    nodes, _, _ = orc.build_mesh(v, i, bits=bits)
    want, changed = orc.restructure(nodes, n, 64, 3)
    assert changed > 0
    assert same_nodes(nodes_of(res, n), want)
    check_conservative(res, v, i)
    assert ctx.device_errors() == 0
