"""Seeded synthetic workloads (no public dataset exists for this path; these
stand in for the reference's Sponza test scene, which is not in its snapshot).

Every generator is numpy-only and deterministic for a given seed.  Rays are
float32 arrays of shape (R, 8) in the RRRay layout
(origin xyz, min_t, direction xyz, max_t).

  soup(n)                      C0/C2 style: centre ~ U[0,1]^3, vertices centre + U[-0.01, 0.01]^3
  heightfield(g)               C1 style: g x g vertex grid over [0,1]^2, z = 0.1 * sum of 8 seeded sinusoids
  pinhole_rays(w, h)           C0 primary rays: eye (0.5, 0.5, -1.5) looking +z, 60 degree vertical FOV
  incoherent_rays(n, lo, hi)   origins ~ U(box), directions uniform on the sphere
"""
from __future__ import annotations

import math

import numpy as np

SEED_BASE = 0x52520000


def rng(config_index: int, stream: int = 0) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64([SEED_BASE + config_index, stream]))


def soup(n: int, seed_rng: np.random.Generator, extent: float = 0.01):
    c = seed_rng.random((n, 1, 3))
    v = c + seed_rng.uniform(-extent, extent, size=(n, 3, 3))
    vertices = v.reshape(-1, 3).astype(np.float32)
    indices = np.arange(3 * n, dtype=np.uint32).reshape(n, 3)
    return vertices, indices


def heightfield(g: int, seed_rng: np.random.Generator):
    f = seed_rng.uniform(-4.0, 4.0, size=(8, 2))
    phi = seed_rng.uniform(0.0, 2.0 * math.pi, size=8)
    xs = np.linspace(0.0, 1.0, g)
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    Z = np.zeros_like(X)
    for k in range(8):
        Z += np.sin(2.0 * math.pi * (f[k, 0] * X + f[k, 1] * Y) + phi[k])
    Z *= 0.1
    vertices = np.stack([X, Y, Z], axis=-1).reshape(-1, 3).astype(np.float32)
    i = np.arange(g - 1)
    I, J = np.meshgrid(i, i, indexing="xy")  # I = column, J = row
    v00 = (J * g + I).reshape(-1)
    v10 = v00 + 1
    v01 = v00 + g
    v11 = v01 + 1
    t0 = np.stack([v00, v10, v11], axis=-1)
    t1 = np.stack([v00, v11, v01], axis=-1)
    indices = np.stack([t0, t1], axis=1).reshape(-1, 3).astype(np.uint32)
    return vertices, indices


def pinhole_rays(w: int, h: int, eye=(0.5, 0.5, -1.5), fov_deg: float = 60.0, tmin: float = 0.0,
                 tmax: float = 1e30) -> np.ndarray:
    t = math.tan(math.radians(fov_deg) * 0.5)
    xs = ((np.arange(w) + 0.5) / w * 2.0 - 1.0) * t
    ys = ((np.arange(h) + 0.5) / h * 2.0 - 1.0) * t
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    d = np.stack([X, Y, np.ones_like(X)], axis=-1).reshape(-1, 3)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.empty((w * h, 8), dtype=np.float32)
    r[:, 0:3] = np.asarray(eye, dtype=np.float64)
    r[:, 3] = tmin
    r[:, 4:7] = d
    r[:, 7] = tmax
    return r


def sphere_dirs(n: int, seed_rng: np.random.Generator) -> np.ndarray:
    z = seed_rng.uniform(-1.0, 1.0, size=n)
    p = seed_rng.uniform(0.0, 2.0 * math.pi, size=n)
    s = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    return np.stack([s * np.cos(p), s * np.sin(p), z], axis=-1)


def incoherent_rays(n: int, lo, hi, seed_rng: np.random.Generator, tmin: float = 0.0, tmax=1e30) -> np.ndarray:
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    r = np.empty((n, 8), dtype=np.float32)
    r[:, 0:3] = lo + seed_rng.random((n, 3)) * (hi - lo)
    r[:, 3] = tmin
    r[:, 4:7] = sphere_dirs(n, seed_rng)
    if isinstance(tmax, tuple):
        r[:, 7] = seed_rng.uniform(tmax[0], tmax[1], size=n)
    else:
        r[:, 7] = tmax
    return r


def config0():
    """65,536-triangle soup + 1024x1024 pinhole primary rays (closest hit)."""
    g = rng(0)
    v, i = soup(65536, g)
    return v, i, pinhole_rays(1024, 1024)


def config1(grid: int = 1449, nrays: int = 16_777_216, any_hit: bool = False):
    """Heightfield (grid^2 vertices) + incoherent rays in its bounding box.
    grid=1449 gives 4,193,408 triangles (2 * 1448^2)."""
    g = rng(1)
    v, i = heightfield(grid, g)
    lo, hi = v.min(axis=0), v.max(axis=0)
    rays = incoherent_rays(nrays, lo, hi, rng(1, 1), tmax=(0.01, 0.5) if any_hit else 1e30)
    return v, i, rays


def random_rotations(n: int, seed_rng: np.random.Generator) -> np.ndarray:
    q = seed_rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - z * w)
    R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w)
    R[:, 2, 1] = 2 * (y * z + x * w)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def config2(n_blas: int = 2048, lo_tris: int = 64, hi_tris: int = 262144, nrays: int = 8_388_608):
    """Batching: n_blas soups with log-uniform triangle counts, instances with
    random rotation, scale U[0.5, 2] and translation U[0, 100]^3."""
    g = rng(2)
    counts = np.rint(np.exp(g.uniform(math.log(lo_tris), math.log(hi_tris), size=n_blas))).astype(np.int64)
    blas = [soup(int(c), rng(2, 100 + k)) for k, c in enumerate(counts)]
    R = random_rotations(n_blas, g)
    s = g.uniform(0.5, 2.0, size=n_blas)
    t = g.uniform(0.0, 100.0, size=(n_blas, 3))
    M = np.zeros((n_blas, 3, 4))
    M[:, :, :3] = R * s[:, None, None]
    M[:, :, 3] = t
    M = M.astype(np.float32)
    # Scene box from transformed unit-box corners.
    corners = np.array([[x, y, z, 1.0] for x in (0, 1) for y in (0, 1) for z in (0, 1)])
    pts = np.einsum("irc,kc->ikr", M.astype(np.float64), corners).reshape(-1, 3)
    lo, hi = pts.min(axis=0), pts.max(axis=0)
    rays = incoherent_rays(nrays, lo, hi, rng(2, 1))
    return blas, M, rays
