"""Generate the golden fixtures of tests/golden/ (run in a checkout where the
reference's bvh_analyzer is available; the fixtures then travel without it).

Each fixture stores its inputs and:
  * the oracle's outputs (nodes, sorted permutation, hits for closest/any x
    full/instance) -- frozen so that any change to the oracle is visible;
  * the reference's own CPU traversal results (bvh_analyzer BvhIntersect via
    oracle/_ref): hit flags for closest and any hit, the closest primitive on
    rays whose max_t is clipped to the oracle's hit distance (bvh_analyzer
    accepts any hit up to max_t, bvh.h:296-307, so clipping leaves only the
    closest), its validity check and SAH of the oracle-built BVH.

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from radeonrays_sdk_gb300 import scenes  # noqa: E402

OUT = Path(__file__).resolve().parent


def mesh_cases():
    g = scenes.rng(10)
    cases = {}
    v, i = scenes.soup(256, g, extent=0.08)
    cases["soup256"] = (v, i, np.concatenate([scenes.pinhole_rays(32, 32),
                                              scenes.incoherent_rays(1024, v.min(0), v.max(0), scenes.rng(10, 1))]))
    v, i = scenes.heightfield(17, scenes.rng(11))
    cases["height17"] = (v, i, scenes.incoherent_rays(2048, v.min(0), v.max(0), scenes.rng(11, 1)))
    # Edge cases: one, two and three triangles; identical triangles (equal
    # Morton codes); a planar mesh (zero extent on one axis); uint16 indices.
    v, i = scenes.soup(1, scenes.rng(12), extent=0.5)
    cases["one"] = (v, i, scenes.incoherent_rays(256, v.min(0) - 0.01, v.max(0) + 0.01, scenes.rng(12, 1)))
    v, i = scenes.soup(2, scenes.rng(13), extent=0.5)
    cases["two"] = (v, i, scenes.incoherent_rays(256, v.min(0) - 0.01, v.max(0) + 0.01, scenes.rng(13, 1)))
    v, i = scenes.soup(3, scenes.rng(14), extent=0.5)
    cases["three"] = (v, i, scenes.incoherent_rays(256, v.min(0) - 0.01, v.max(0) + 0.01, scenes.rng(14, 1)))
    v1, i1 = scenes.soup(1, scenes.rng(15), extent=0.5)
    v = np.tile(v1, (40, 1))
    i = np.arange(120, dtype=np.uint32).reshape(40, 3)
    cases["dupes"] = (v, i, scenes.incoherent_rays(512, v.min(0) - 0.01, v.max(0) + 0.01, scenes.rng(15, 1)))
    v, i = scenes.heightfield(9, scenes.rng(16))
    v[:, 2] = 0.25
    cases["planar"] = (v, i, scenes.incoherent_rays(512, v.min(0) - 0.01, v.max(0) + 0.01, scenes.rng(16, 1)))
    v, i = scenes.heightfield(20, scenes.rng(17))
    cases["u16"] = (v, i.astype(np.uint16), scenes.incoherent_rays(512, v.min(0), v.max(0), scenes.rng(17, 1)))
    return cases


def main():
    if oracle.ref_lib() is None:
        oracle.build()
    assert oracle.ref_lib() is not None, "the reference harness (oracle/_ref) is required to make the fixtures"
    for name, (v, i, rays) in mesh_cases().items():
        nodes, sidx, scodes = oracle.build_mesh(v, i)
        out = {"vertices": v, "indices": i, "rays": rays, "nodes": nodes.view(np.uint32).reshape(-1, 16),
               "sorted_idx": sidx, "sorted_codes": scodes, "aabb": oracle.mesh_aabb(v, i)}
        for q in (0, 1):
            for o in (0, 1):
                out[f"hits_q{q}_o{o}"] = oracle.trace(nodes, rays, query=q, output=o)
        t32 = oracle.trace_t(nodes, rays)
        out["t"] = t32
        if nodes.size < 3:
            # bvh_analyzer indexes its internal-node array at the root and
            # cannot represent a one-leaf tree; nothing reference-side to record.
            np.savez_compressed(OUT / f"{name}.npz", **out)
            print(name, "tris", i.size // 3, "(no reference-side record)")
            continue
        ok, sah = oracle.ref_validate(nodes)
        out["ref_valid"] = np.array([ok])
        out["ref_sah"] = np.array([sah], dtype=np.float32)
        rh, _ = oracle.ref_trace(nodes, rays)
        ra, _ = oracle.ref_trace(nodes, rays, any_hit=True)
        out["ref_hit_closest"] = (rh[:, 2] != oracle.INVALID)
        out["ref_hit_any"] = (ra[:, 2] != oracle.INVALID)
        hit = np.isfinite(t32)
        clip = rays[hit].copy()
        # A little above the hit distance: bvh_analyzer's unfused slab test
        # (float3.h:142) can put a zero-thickness box's entry past it when the
        # origin is close to the box plane (cancellation in p*invd - o*invd).
        clip[:, 7] = t32[hit] * np.float32(1.0 + 2.0 ** -12) + np.float32(1e-7)
        rc, _ = oracle.ref_trace(nodes, clip)
        out["ref_clip_prim"] = rc[:, 3]
        out["ref_clip_uv"] = rc[:, :2].view(np.float32)
        np.savez_compressed(OUT / f"{name}.npz", **out)
        print(name, "tris", i.size // 3, "rays", rays.shape[0], "hits", int(hit.sum()), "valid", ok)

    # Two-level scene: 3 BLAS, 6 instances.
    blas = [scenes.soup(64, scenes.rng(20, k)) for k in range(3)]
    R = scenes.random_rotations(6, scenes.rng(21))
    M = np.zeros((6, 3, 4))
    M[:, :, :3] = R * scenes.rng(22).uniform(0.5, 2.0, size=6)[:, None, None]
    M[:, :, 3] = scenes.rng(23).uniform(0.0, 3.0, size=(6, 3))
    M = M.astype(np.float32)
    which = np.array([0, 1, 2, 0, 1, 2], dtype=np.int64)
    bn = [oracle.build_mesh(v, i)[0] for (v, i) in blas]
    tlas, xf = oracle.build_scene([bn[w] for w in which], [blas[w][1].shape[0] for w in which], M)
    rays = scenes.incoherent_rays(2048, (-1, -1, -1), (5, 5, 5), scenes.rng(24))
    out = {"which": which, "M": M, "tlas": tlas.view(np.uint32).reshape(-1, 16), "xforms": xf, "rays": rays}
    for k, (v, i) in enumerate(blas):
        out[f"v{k}"] = v
        out[f"i{k}"] = i
    for q in (0, 1):
        for o in (0, 1):
            out[f"hits_q{q}_o{o}"] = oracle.trace_scene(tlas, xf, [bn[w] for w in which], rays, query=q, output=o)
    np.savez_compressed(OUT / "scene6.npz", **out)
    print("scene6 instances", len(which))


if __name__ == "__main__":
    main()
