"""CPU tests of the oracle: frozen golden outputs, the pins against the
reference's own CPU traversal (bvh_analyzer), and the reference tests'
structural checks (test/test_vk/hlbvh_test.h:69-100, algos_test.h:277-393)."""
from collections import deque

import numpy as np
import pytest

from conftest import MESH_FIXTURES, golden

INVALID = 0xFFFFFFFF


def clip_window(t):
    """max_t used on the reference side: a little above the oracle's hit."""
    return t * np.float32(1.0 + 2.0 ** -12) + np.float32(1e-7)


def assert_clip_agreement(orc, rays, t, prim, ref_prim, vertices, indices):
    """bvh_analyzer accepts every hit up to max_t and keeps the last one it
    visits (bvh.h:296-307), so with max_t = clip_window(t) it must return the
    oracle's closest primitive, or another one hit no nearer than t inside
    the window (overlapping triangles)."""
    diff = np.where(ref_prim != prim)[0]
    assert diff.size <= max(2, prim.size // 500)
    if diff.size:
        assert np.all(ref_prim[diff] != INVALID)
        idx = indices.astype(np.int64)
        tri = vertices[idx[ref_prim[diff]]].reshape(-1, 9)
        r = rays[diff].copy()
        r[:, 7] = clip_window(t[diff])
        tr = orc.tri_test(r, tri)[:, 0]
        assert np.all(tr >= t[diff]) and np.all(tr <= r[:, 7])


def node_box(n):
    """GetAabb (test/test_vk/common.h:215-235)."""
    if n["child0"] != INVALID:
        return np.minimum(n["a0"], n["b0"]), np.maximum(n["a1"], n["b1"])
    v = np.stack([n["a0"], n["a1"], n["b0"]])
    return v.min(0), v.max(0)


def consistent(nodes) -> bool:
    """CheckConstistency (test/test_vk/hlbvh_test.h:69-100): parent links and
    child-box containment (Aabb::Includes with 1e-8 slack)."""
    q = deque([(0, INVALID)])
    seen = 0
    while q:
        addr, parent = q.popleft()
        nd = nodes[addr]
        seen += 1
        if nd["parent"] != parent:
            return False
        if nd["child0"] != INVALID:
            lo, hi = node_box(nd)
            for c in (nd["child0"], nd["child1"]):
                clo, chi = node_box(nodes[c])
                if np.any(clo - lo < -1e-8) or np.any(hi - chi < -1e-8):
                    return False
                q.append((int(c), addr))
    return seen == nodes.size


@pytest.mark.parametrize("name", MESH_FIXTURES)
def test_oracle_matches_golden(orc, name):
    g = golden(name)
    nodes, sidx, scodes = orc.build_mesh(g["vertices"], g["indices"])
    assert np.array_equal(nodes.view(np.uint32).reshape(-1, 16), g["nodes"])
    assert np.array_equal(sidx, g["sorted_idx"])
    assert np.array_equal(scodes, g["sorted_codes"])
    assert np.array_equal(orc.mesh_aabb(g["vertices"], g["indices"]), g["aabb"])
    for q in (0, 1):
        for o in (0, 1):
            assert np.array_equal(orc.trace(nodes, g["rays"], query=q, output=o), g[f"hits_q{q}_o{o}"])


@pytest.mark.parametrize("name", [n for n in MESH_FIXTURES if n != "one"])
def test_oracle_pinned_to_reference_traversal(orc, name):
    """Hit flags (closest and any) equal bvh_analyzer's on every ray; the
    closest primitive equals bvh_analyzer's on rays clipped to the oracle's t;
    the oracle-built BVH passes bvh_analyzer's IsValid."""
    g = golden(name)
    nodes, _, _ = orc.build_mesh(g["vertices"], g["indices"])
    closest = orc.trace(nodes, g["rays"], query=0, output=0)
    anyh = orc.trace(nodes, g["rays"], query=1, output=0)
    assert bool(g["ref_valid"][0])
    assert np.array_equal(closest[:, 2] != INVALID, g["ref_hit_closest"])
    assert np.array_equal(anyh[:, 2] != INVALID, g["ref_hit_any"])
    hit = closest[:, 2] != INVALID
    assert_clip_agreement(orc, g["rays"][hit], g["t"][hit], closest[hit, 3], g["ref_clip_prim"], g["vertices"],
                          g["indices"])
    # bvh_analyzer reports Moller-Trumbore (b1, b2); isect.comp recomputes
    # barycentrics from the hit point (common.h:187-209): same point, other formula.
    same = closest[hit, 3] == g["ref_clip_prim"]
    uv = closest[hit, :2].view(np.float32)[same]
    assert np.allclose(uv, g["ref_clip_uv"][same], atol=2e-2)


@pytest.mark.parametrize("name", MESH_FIXTURES)
def test_oracle_tree_consistency(orc, name):
    g = golden(name)
    nodes, _, _ = orc.build_mesh(g["vertices"], g["indices"])
    assert consistent(nodes)
    n = g["indices"].shape[0]
    internal = nodes[: n - 1]
    leaves = nodes[n - 1:]
    assert np.all(leaves["child0"] == INVALID) and np.all(leaves["update"] == 0)
    assert np.all(internal["update"] == 1)
    assert sorted(leaves["child1"].tolist()) == list(range(n))


def test_oracle_sort_matches_stable_sort(orc):
    """algos_test.h:269-378: 1 Mi keys from uniform_int(0, 1000) vs a CPU sort;
    additionally checks stability (the LBVH relies on it)."""
    keys = np.random.default_rng(0).integers(0, 1001, size=1 << 20).astype(np.uint32)
    sc, si = orc.sort(keys)
    ref = np.argsort(keys, kind="stable")
    assert np.array_equal(si, ref.astype(np.uint32))
    assert np.array_equal(sc, keys[ref])
    k64 = np.random.default_rng(1).integers(0, 1 << 62, size=1 << 16, dtype=np.uint64)
    sc, si = orc.sort(k64)
    assert np.array_equal(si, np.argsort(k64, kind="stable").astype(np.uint32))


def test_oracle_scene_matches_golden(orc):
    g = golden("scene6")
    bn = [orc.build_mesh(g[f"v{k}"], g[f"i{k}"])[0] for k in range(3)]
    which = g["which"]
    tlas, xf = orc.build_scene([bn[w] for w in which], [g[f"i{w}"].shape[0] for w in which], g["M"])
    assert np.array_equal(tlas.view(np.uint32).reshape(-1, 16), g["tlas"])
    assert np.array_equal(xf, g["xforms"])
    assert consistent(tlas)
    for q in (0, 1):
        for o in (0, 1):
            assert np.array_equal(orc.trace_scene(tlas, xf, [bn[w] for w in which], g["rays"], query=q, output=o),
                                  g[f"hits_q{q}_o{o}"])


def test_oracle_scene_single_instance_equals_geometry(orc):
    """With an identity instance the two-level traversal returns the
    single-level hits (instance id 0)."""
    g = golden("height17")
    nodes, _, _ = orc.build_mesh(g["vertices"], g["indices"])
    M = np.eye(3, 4, dtype=np.float32)[None]
    tlas, xf = orc.build_scene([nodes], [g["indices"].shape[0]], M)
    a = orc.trace(nodes, g["rays"])
    b = orc.trace_scene(tlas, xf, [nodes], g["rays"])
    assert np.array_equal(a, b)


def test_oracle_live_against_reference(orc):
    """Live pin on a 65,536-triangle soup (skipped where the reference harness
    was not built, e.g. on the GPU machine)."""
    if orc.ref_lib() is None:
        pytest.skip("reference harness not built here")
    from radeonrays_sdk_gb300 import scenes
    v, i, rays = scenes.config0()
    sub = rays[::32].copy()
    nodes, _, _ = orc.build_mesh(v, i)
    ok, _ = orc.ref_validate(nodes)
    assert ok
    h = orc.trace(nodes, sub)
    rh, _ = orc.ref_trace(nodes, sub)
    assert np.array_equal(h[:, 2] != INVALID, rh[:, 2] != INVALID)
    t = orc.trace_t(nodes, sub)
    hit = np.isfinite(t)
    clip = sub[hit].copy()
    clip[:, 7] = clip_window(t[hit])
    rc, _ = orc.ref_trace(nodes, clip)
    assert_clip_agreement(orc, sub[hit], t[hit], h[hit, 3], rc[:, 3], v, i)


def test_oracle_fp64_t_error_small(orc):
    """t of the fp32 closest hit against the exact (fp64) intersection with the
    same triangle, on the heightfield fixture."""
    g = golden("height17")
    nodes, _, _ = orc.build_mesh(g["vertices"], g["indices"])
    h = orc.trace(nodes, g["rays"])
    t32 = orc.trace_t(nodes, g["rays"])
    hit = h[:, 2] != INVALID
    v, idx = g["vertices"], g["indices"].astype(np.int64)
    tri9 = np.zeros((h.shape[0], 9), np.float32)
    tri9[hit] = v[idx[h[hit, 3]]].reshape(-1, 9)
    e = orc.fp64_hit(g["rays"], tri9, hit.astype(np.uint32))
    rel = np.abs(t32[hit].astype(np.float64) - e[hit, 0]) / np.spacing(np.abs(t32[hit]))
    assert rel.max() < 64  # ulps; typical 0-2


def test_oracle_fit_is_the_build_refit(orc):
    """The update restatement (leaves take their primitive's vertices, then a
    bottom-up refit) reproduces the built tree from the same vertices, and
    every box still contains its subtree after moving the vertices."""
    from radeonrays_sdk_gb300 import scenes
    v, i = scenes.soup(3000, scenes.rng(80))
    nodes, _, _ = orc.build_mesh(v, i)
    again = orc.fit(nodes, v, i)
    assert np.array_equal(again.view(np.uint32).reshape(-1, 16)[:, :12],
                          nodes.view(np.uint32).reshape(-1, 16)[:, :12])
    v2 = (v * np.float32(2.0) + np.float32(0.25)).astype(np.float32)
    moved = orc.fit(nodes, v2, i)
    assert np.array_equal(moved["child0"], nodes["child0"]) and np.array_equal(moved["child1"], nodes["child1"])
    n = i.shape[0]
    lo = np.minimum(np.minimum(moved["a0"], moved["a1"]), moved["b0"])[n - 1:]
    hi = np.maximum(np.maximum(moved["a0"], moved["a1"]), moved["b0"])[n - 1:]
    # The root's two child boxes together contain every moved leaf.
    root = moved[0]
    rlo = np.minimum(root["a0"], root["b0"])
    rhi = np.maximum(root["a1"], root["b1"])
    assert np.all(lo >= rlo) and np.all(hi <= rhi)


def test_oracle_aabb_leaves(orc):
    """AABB-list semantics: a ray through a box hits it at the slab entry
    distance, the nearest entry wins, a ray starting inside hits at min_t,
    and a ray that misses every box writes only inst_id."""
    b = np.zeros((3, 8), np.float32)
    b[0, 0:3], b[0, 4:7] = (0.0, 0.0, 2.0), (1.0, 1.0, 3.0)   # entry t = 2
    b[1, 0:3], b[1, 4:7] = (0.0, 0.0, 5.0), (1.0, 1.0, 6.0)   # behind box 0
    b[2, 0:3], b[2, 4:7] = (4.0, 4.0, -1.0), (5.0, 5.0, 1.0)  # holds the origin of ray 2
    nodes, _, _ = orc.build_aabbs(b)
    rays = np.array([[0.5, 0.5, 0.0, 0.0, 0.0, 0.0, 1.0, 100.0],
                     [0.5, 0.5, 0.0, 0.0, 0.0, 0.0, -1.0, 100.0],
                     [4.5, 4.5, 0.0, 0.25, 0.0, 0.0, 1.0, 100.0]], np.float32)
    h = orc.trace(nodes, rays, box_leaves=True)
    assert list(h[0]) == [0, 0, 0, 0] and h[2, 3] == 2 and h[2, 2] == 0
    assert h[1, 2] == INVALID and h[1, 0] == INVALID  # miss: only inst_id written, the rest keeps the fill
    hi = orc.trace(nodes, rays, output=1, box_leaves=True)
    assert list(hi) == [0, INVALID, 2]


def _check_tree(nodes, n):
    """Every leaf reached exactly once from the root, parent links consistent,
    every stored child box equal to the child's own box."""
    seen = np.zeros(2 * n - 1, np.int32)
    stack = [0]
    while stack:
        x = stack.pop()
        seen[x] += 1
        if x >= n - 1:
            continue
        for c, lo, hi in ((nodes["child0"][x], "a0", "a1"), (nodes["child1"][x], "b0", "b1")):
            assert nodes["parent"][c] == x
            if c < n - 1:
                clo = np.minimum(nodes["a0"][c], nodes["b0"][c])
                chi = np.maximum(nodes["a1"][c], nodes["b1"][c])
            else:
                tri = np.stack([nodes["a0"][c], nodes["a1"][c], nodes["b0"][c]])
                clo, chi = tri.min(axis=0), tri.max(axis=0)
            assert np.array_equal(nodes[lo][x], clo) and np.array_equal(nodes[hi][x], chi)
            stack.append(int(c))
    assert np.all(seen == 1)


def _half_area_sum(nodes, n):
    lo = np.minimum(nodes["a0"][: n - 1], nodes["b0"][: n - 1]).astype(np.float64)
    hi = np.maximum(nodes["a1"][: n - 1], nodes["b1"][: n - 1]).astype(np.float64)
    e = hi - lo
    return float((e[:, 0] * e[:, 1] + e[:, 1] * e[:, 2] + e[:, 2] * e[:, 0]).sum())


def test_oracle_restructure_is_a_valid_cheaper_tree(orc):
    """The treelet restructure keeps a valid tree in the reference layout,
    lowers the summed node area, is deterministic, and keeps every hit."""
    from radeonrays_sdk_gb300 import scenes
    v, i = scenes.heightfield(129, scenes.rng(81))
    n = i.shape[0]
    nodes, _, _ = orc.build_mesh(v, i)
    r1, changed = orc.restructure(nodes, n, 64, 3)
    r2, _ = orc.restructure(nodes, n, 64, 3)
    assert changed > 0 and np.array_equal(r1.view(np.uint32), r2.view(np.uint32))
    _check_tree(r1, n)
    assert _half_area_sum(r1, n) < _half_area_sum(nodes, n)
    assert np.array_equal(r1["child0"][n - 1:], nodes["child0"][n - 1:])  # leaves untouched
    assert np.array_equal(r1["child1"][n - 1:], nodes["child1"][n - 1:])
    rays = scenes.incoherent_rays(20000, v.min(axis=0), v.max(axis=0), scenes.rng(81, 1))
    a, fa = orc.trace(nodes, rays, fetches=True)
    b, fb = orc.trace(r1, rays, fetches=True)
    assert np.array_equal(a[:, 2] != INVALID, b[:, 2] != INVALID)
    assert fb.mean() < fa.mean()
    if orc.ref_lib() is not None:
        ok, _ = orc.ref_validate(r1)
        assert ok


def test_precise_oracle_is_watertight(orc):
    """Rays aimed exactly at shared vertices and edges of a grid mesh: the
    reference's Moller-Trumbore test (common.h:103-137) lets some through
    the cracks between triangles; the precise mode's watertight test (exact
    edge-function signs on the sheared vertices) hits every one."""
    from edge_rays import bumpy_grid, edge_rays
    v, i = bumpy_grid()
    rays = edge_rays(v)
    nodes, _, _ = orc.build_mesh(v, i)
    ref = orc.trace(nodes, rays)
    hp, tp = orc.trace_precise(nodes, rays)
    assert (ref[:, 2] == 0xFFFFFFFF).sum() > 1000
    assert (hp[:, 2] == 0xFFFFFFFF).sum() == 0
    assert np.all(np.isfinite(tp))


def test_precise_oracle_t_and_uv_accuracy(orc):
    """Precise mode: t within 1 ulp and uv within 1e-6 of the fp64
    intersection of the same ray and triangle, on every hit; the reference's
    arithmetic is far outside that bound on the same rays."""
    from radeonrays_sdk_gb300 import scenes
    v, i, rays = scenes.config1(grid=129, nrays=1 << 16)
    nodes, _, _ = orc.build_mesh(v, i)
    hp, tp = orc.trace_precise(nodes, rays)
    hit = hp[:, 2] != 0xFFFFFFFF
    assert hit.sum() > 10000
    idx = i.astype(np.int64)
    tri9 = np.zeros((rays.shape[0], 9), np.float32)
    tri9[hit] = v[idx[hp[hit, 3]]].reshape(-1, 9)
    e = orc.fp64_hit(rays, tri9, hit.astype(np.uint32))
    ulp = np.abs(tp[hit].astype(np.float64) - e[hit, 0]) / np.spacing(np.abs(tp[hit])).astype(np.float64)
    assert ulp.max() <= 1.0, ulp.max()
    uv = hp[hit, :2].view(np.float32).astype(np.float64)
    assert np.abs(uv - e[hit, 1:3]).max() <= 1e-6
    # The same rays with the reference's test: hit flags agree except at cracks.
    ref = orc.trace(nodes, rays)
    assert np.mean((ref[:, 2] != 0xFFFFFFFF) == hit) > 0.999
    tr = orc.trace_t(nodes, rays)
    rh = ref[:, 2] != 0xFFFFFFFF
    tri9r = np.zeros((rays.shape[0], 9), np.float32)
    tri9r[rh] = v[idx[ref[rh, 3]]].reshape(-1, 9)
    er = orc.fp64_hit(rays, tri9r, rh.astype(np.uint32))
    ulp_r = np.abs(tr[rh].astype(np.float64) - er[rh, 0]) / np.spacing(np.abs(tr[rh])).astype(np.float64)
    assert ulp_r.max() > 10.0
