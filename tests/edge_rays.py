"""A bumpy grid mesh and rays aimed exactly at its interior vertices and edge
points, where 2 to 6 triangles meet: the workload of the watertightness
checks.  Every ray comes from above, more steeply than any slope of the
surface, so in exact arithmetic every ray hits the mesh; a ray that misses
has leaked through a crack between triangles."""
import numpy as np


def bumpy_grid(g=64):
    xs = np.linspace(0, 1, g + 1, dtype=np.float32)
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    Z = (0.05 * np.sin(7 * X) * np.cos(5 * Y) + 0.3 * X + 0.1 * Y).astype(np.float32)
    v = np.stack([X, Y, Z], -1).reshape(-1, 3).astype(np.float32)
    p = (np.arange(g)[:, None] * (g + 1) + np.arange(g)[None, :]).reshape(-1)
    i = np.concatenate([np.stack([p, p + g + 1, p + 1], 1), np.stack([p + 1, p + g + 1, p + g + 2], 1)], 0)
    return v, np.ascontiguousarray(i.astype(np.uint32))


def edge_rays(v, g=64, n=200_000, seed=5):
    """Rays from 1.5 above (and up to 0.5 to the side of) a target that is an
    interior vertex or a point on an interior edge; surface slopes stay below
    1, the rays' slopes above 2."""
    rng = np.random.default_rng(seed)
    a, b = rng.integers(1, g, n), rng.integers(1, g, n)
    kind = rng.integers(0, 3, n)
    p0 = v[a * (g + 1) + b]
    nb = np.where(kind == 1, (a + 1) * (g + 1) + b, np.where(kind == 2, a * (g + 1) + b + 1, (a + 1) * (g + 1) + b + 1))
    p1 = v[nb]
    w = rng.random(n).astype(np.float32)
    t = np.where((kind == 0)[:, None], p0, p0 + (p1 - p0) * w[:, None]).astype(np.float32)
    o = (t + np.concatenate([rng.uniform(-0.5, 0.5, (n, 2)), np.full((n, 1), 1.5)], 1).astype(np.float32))
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = o
    rays[:, 4:7] = (t - o).astype(np.float32)
    rays[:, 7] = np.float32(1e30)
    return rays
