"""GPU build parity: the CUDA LBVH (bounds, Morton codes, onesweep sort,
Karras emit, atomic refit) against the oracle, bit for bit, through the C-ABI;
structural checks of the 8-wide collapse."""
import numpy as np
import pytest

from conftest import MESH_FIXTURES, golden
from gpu_util import INVALID, build, nodes_of, to_dev, trailer_of

pytestmark = pytest.mark.gpu


def same_nodes(a, b):
    ua, ub = a.view(np.uint32).reshape(-1, 16), b.view(np.uint32).reshape(-1, 16)
    if np.array_equal(ua, ub):
        return True
    # Allow only a different sign of zero in box coordinates.
    fa, fb = a.view(np.float32).reshape(-1, 16), b.view(np.float32).reshape(-1, 16)
    ints = [3, 7, 11, 15]
    return np.array_equal(ua[:, ints], ub[:, ints]) and np.array_equal(
        np.delete(fa, ints, axis=1), np.delete(fb, ints, axis=1))


@pytest.mark.parametrize("name", MESH_FIXTURES)
@pytest.mark.parametrize("fmt", [0, 1, 2])
def test_build_matches_oracle_on_fixtures(ctx, orc, name, fmt):
    g = golden(name)
    n = g["indices"].shape[0]
    res = build(ctx, g["vertices"], g["indices"], node_format=fmt)
    got = nodes_of(res, n)
    ref = g["nodes"].view(orc.NODE_DTYPE).reshape(-1)
    assert same_nodes(got, ref)
    tr = trailer_of(res, n)
    assert tr["magic"] == 0x52524742 and tr["leaf_count"] == n and tr["node_format"] == fmt
    assert np.array_equal(tr["bounds"], g["aabb"])
    assert ctx.device_errors() == 0


@pytest.mark.parametrize("ntri", [1000, 65536, 300_000])
def test_build_matches_oracle_on_soups(ctx, orc, ntri):
    from radeonrays_sdk_gb300 import scenes
    v, i = scenes.soup(ntri, scenes.rng(30, ntri))
    res = build(ctx, v, i, node_format=0)
    nodes, _, _ = orc.build_mesh(v, i)
    assert same_nodes(nodes_of(res, ntri), nodes)


def test_build_matches_oracle_heightfield_1m(ctx, orc):
    """513 x 513 grid: 524,288 triangles, many equal Morton codes."""
    from radeonrays_sdk_gb300 import scenes
    v, i = scenes.heightfield(513, scenes.rng(31))
    res = build(ctx, v, i, node_format=1)
    nodes, _, _ = orc.build_mesh(v, i)
    assert same_nodes(nodes_of(res, i.shape[0]), nodes)
    assert ctx.device_errors() == 0


def test_build_63bit_keys(ctx, orc):
    from radeonrays_sdk_gb300 import scenes
    v, i = scenes.heightfield(257, scenes.rng(32))
    res = build(ctx, v, i, node_format=0, morton_bits=63)
    nodes, _, _ = orc.build_mesh(v, i, bits=63)
    assert same_nodes(nodes_of(res, i.shape[0]), nodes)


def test_build_vertex_stride_16(ctx, orc):
    g = golden("height17")
    v4 = np.concatenate([g["vertices"], np.full((g["vertices"].shape[0], 1), 7.0, np.float32)], axis=1)
    res = ctx.build_geometry(to_dev(v4), to_dev(g["indices"]), node_format=0, stride=16)
    assert same_nodes(nodes_of(res, g["indices"].shape[0]), g["nodes"].view(orc.NODE_DTYPE).reshape(-1))


def decode_wide(res, tr):
    raw = res.cpu().numpy()
    wn = raw[tr["wide_nodes_off"]: tr["wide_nodes_off"] + 80 * int(tr["wide_count"])].reshape(-1, 80)
    wt = raw[tr["wide_tris_off"]: tr["wide_tris_off"] + 48 * int(tr["wide_tri_count"])].reshape(-1, 48)
    return wn, wt


def test_wide_collapse_structure(ctx, orc):
    """Every triangle appears once in the wide triangle array, every child is
    referenced once, and every decoded child box contains its subtree."""
    from radeonrays_sdk_gb300 import scenes
    v, i = scenes.soup(20000, scenes.rng(33))
    n = i.shape[0]
    res = build(ctx, v, i, node_format=1)
    tr = trailer_of(res, n)
    assert tr["wide_tri_count"] == n and 1 <= tr["wide_count"] <= n - 1
    wn, wt = decode_wide(res, tr)
    prims = wt[:, 12:16].copy().view(np.uint32).reshape(-1)
    assert np.array_equal(np.sort(prims), np.arange(n, dtype=np.uint32))
    tri_v = wt.view(np.float32).reshape(-1, 12)[:, [0, 1, 2, 4, 5, 6, 8, 9, 10]].reshape(-1, 3, 3)
    p = wn[:, 0:12].copy().view(np.float32).reshape(-1, 3)
    e = wn[:, 12:15].astype(np.int64)
    imask = wn[:, 15]
    cbase = wn[:, 16:20].copy().view(np.uint32).reshape(-1)
    tbase = wn[:, 20:24].copy().view(np.uint32).reshape(-1)
    meta = wn[:, 24:32]
    qlo = wn[:, 32:56].reshape(-1, 3, 8).astype(np.float32)
    qhi = wn[:, 56:80].reshape(-1, 3, 8).astype(np.float32)
    scale = np.ldexp(np.float32(1.0), (e - 127)).astype(np.float32)
    lo = (qlo * scale[:, :, None] + p[:, :, None]).astype(np.float32)
    hi = (qhi * scale[:, :, None] + p[:, :, None]).astype(np.float32)
    # Subtree boxes bottom-up (children have larger indices than parents).
    W = wn.shape[0]
    sub_lo = np.full((W, 3), np.inf, np.float32)
    sub_hi = np.full((W, 3), -np.inf, np.float32)
    seen_child = np.zeros(W, np.int64)
    for w in range(W - 1, -1, -1):
        for k in range(8):
            m = int(meta[w, k])
            if m == 0:
                continue
            if imask[w] >> k & 1:
                c = int(cbase[w]) + (m & 0x7F)
                seen_child[c] += 1
                blo, bhi = sub_lo[c], sub_hi[c]
            else:
                cnt, off = m >> 5, m & 31
                t = tri_v[int(tbase[w]) + off: int(tbase[w]) + off + cnt]
                blo, bhi = t.reshape(-1, 3).min(0), t.reshape(-1, 3).max(0)
            # conservative: decoded box contains the exact child box
            assert np.all(lo[w, :, k] <= blo) and np.all(hi[w, :, k] >= bhi), (w, k)
            sub_lo[w] = np.minimum(sub_lo[w], blo)
            sub_hi[w] = np.maximum(sub_hi[w], bhi)
    assert seen_child[0] == 0 and np.all(seen_child[1:] == 1)


def test_empty_mesh(ctx):
    import torch
    v = torch.zeros((3, 3), dtype=torch.float32, device="cuda")
    i = torch.zeros((0, 3), dtype=torch.int32, device="cuda")
    res = ctx.build_geometry(v, i)
    tr = trailer_of(res, 0)
    assert tr["magic"] == 0x52524742 and tr["leaf_count"] == 0
    from radeonrays_sdk_gb300 import scenes
    rays = scenes.incoherent_rays(100, (0, 0, 0), (1, 1, 1), scenes.rng(34))
    for trav in (1, 2):
        ctx.set_traversal(trav)
        h = ctx.intersect(res, to_dev(rays)).cpu().numpy().view(np.uint32)
        assert np.all(h[:, 2] == INVALID)
    ctx.set_traversal(0)
