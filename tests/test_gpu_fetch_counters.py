"""Device traversal counters against the oracle's counts on the same BVH.

The roofline's algorithmic bytes are 32 + 16 + 64 x node fetches per ray,
with the node fetches counted by the kernels themselves (collect_stats).
Both binary-node kernels visit nodes in the reference order (isect.comp:
105-245), so their fetch totals must equal the oracle's per-ray counts summed,
on the 65,536-triangle soup with 1024x1024 pinhole rays and on an incoherent
heightfield batch, for closest and any hit."""
import numpy as np
import pytest

from gpu_util import build, to_dev
from radeonrays_sdk_gb300 import scenes

pytestmark = pytest.mark.gpu

BINARY, WIDE, PERSISTENT = 1, 2, 3


def _device_fetches(ctx, res, rays, traversal, query):
    ctx.set_traversal(traversal, collect_stats=1)
    ctx.stats()  # clear
    ctx.intersect(res, to_dev(rays), query=query)
    s = ctx.stats()
    ctx.set_traversal(0)
    return s


def _cases():
    v, i, rays = scenes.config0()
    yield "soup65536_pinhole1024", v, i, rays
    hv, hi = scenes.heightfield(257, scenes.rng(1))
    hr = scenes.incoherent_rays(262144, hv.min(0), hv.max(0), scenes.rng(1, 1))
    yield "heightfield257_incoherent", hv, hi, hr


@pytest.mark.parametrize("query", [0, 1])
def test_binary_fetch_counts_equal_oracle(ctx, orc, query):
    for name, v, i, rays in _cases():
        nodes, _, _ = orc.build_mesh(v, i)
        _, f = orc.trace(nodes, rays, query=query, fetches=True)
        want = int(f.sum())
        res = build(ctx, v, i, node_format=1)  # binary nodes + 8-wide nodes
        for trav in (BINARY, PERSISTENT):
            s = _device_fetches(ctx, res, rays, trav, query)
            assert s["rays"] == rays.shape[0], (name, trav)
            assert s["node_fetches"] == want, (name, trav, s["node_fetches"], want)
            assert s["triangle_fetches"] == 0, (name, trav)
        # The 8-wide kernel counts its own (fewer, larger) fetches.
        s = _device_fetches(ctx, res, rays, WIDE, query)
        assert s["rays"] == rays.shape[0]
        assert 0 < s["node_fetches"] < want, (name, s["node_fetches"], want)
    assert ctx.device_errors() == 0
