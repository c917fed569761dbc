"""Serving loop: many resident scenes, ray requests of uneven size arriving
over time, continuous batching into multi-request traversal launches.

No reference counterpart (the reference is a library that traces what its
caller submits).  Everything here drives the library through its C-ABI:
scene BVHs are built with rrCmdBuildGeometry, and every launch is one
rrCudaCmdIntersectBatch over the requests packed into it.

Model:
  * ScenePool keeps built BVHs resident under a device-memory budget (bytes of
    result buffers).  A scene is built the first time a request needs it; when
    the budget would be exceeded, least-recently-used scenes that no launch in
    flight uses are evicted.
  * Server owns `slots` launch slots.  Each slot has its own CUDA stream, a
    ray arena and a hit arena of `slot_rays` rays, and a batch scratch.  The
    host loop admits queued requests (oldest first) into a free slot while
    they fit its arena and the scene budget, copies their rays in, records one
    batched launch and the copy of the hits back, and marks the slot busy
    until an event after the copy completes.  Requests that arrive while other
    launches run are admitted into the next free slot, so launches of
    different slots overlap on the device: continuous batching at launch
    granularity, with no device-side wait of any kind.
  * Each request's hits are bit-identical to tracing it alone (the batched
    kernel runs, per ray, the visit order of the single-request kernel it
    stands for: the 4-wide kernel on the pool's default 4-wide scenes, the
    reference's binary order otherwise), whatever it is packed with; the
    tests check this.
"""
from __future__ import annotations

import collections
import dataclasses
import gc
import time

import numpy as np

from . import rr


@dataclasses.dataclass
class Request:
    rid: int
    arrival: float          # seconds from the start of the run
    scene: int
    rays: np.ndarray        # (R, 8) float32, host
    query: int = rr.RR_INTERSECT_QUERY_CLOSEST
    output: int = rr.RR_INTERSECT_QUERY_OUTPUT_FULL_HIT
    # pinned host views (ray pools, make_requests(pools=...)): the server
    # uses them instead of pinning a copy of `rays`
    pinned_rays: object = None
    # filled by the server
    admitted: float = -1.0
    done: float = -1.0
    hits: np.ndarray | None = None

    @property
    def latency(self) -> float:
        return self.done - self.arrival


class ScenePool:
    """Resident BVHs of many meshes under a byte budget.  The default node
    format (binary + 4-wide nodes with 8-bit bounds, half the bytes of the
    fp32 ones) lets a launch whose requests all have such nodes run the
    4-wide multi-request kernel; with binary-only scenes the launches run
    the reference-order binary kernel."""

    def __init__(self, ctx: rr.Context, budget_bytes: int, node_format: int = rr.RR_CUDA_NODE_FORMAT_BVH4Q8):
        self.ctx = ctx
        self.budget = int(budget_bytes)
        self.node_format = node_format
        self.meshes: dict[int, tuple[np.ndarray, np.ndarray]] = {}
        self.resident: collections.OrderedDict[int, object] = collections.OrderedDict()  # LRU order
        self.pins: collections.Counter = collections.Counter()
        self.bytes = 0
        self.builds = 0
        self.evictions = 0
        self.handles: dict = {}  # scene -> RRDevicePtr of its resident buffer

    def register(self, scene: int, vertices: np.ndarray, indices: np.ndarray) -> None:
        self.meshes[scene] = (np.ascontiguousarray(vertices, np.float32), np.ascontiguousarray(indices, np.uint32))

    def result_bytes(self, scene: int) -> int:
        v, i = self.meshes[scene]
        return self.ctx.geometry_requirements(i.shape[0], self.node_format, 30, v.shape[0], 12)[1]

    def _make_room(self, need: int) -> bool:
        if self.bytes + need <= self.budget:
            return True
        for sid in list(self.resident.keys()):
            if self.bytes + need <= self.budget:
                break
            if self.pins[sid] == 0:
                buf = self.resident.pop(sid)
                self.bytes -= buf.numel()
                self.evictions += 1
                h = self.handles.pop(sid, None)
                if h is not None:
                    self.ctx.L.rrReleaseDevicePtr(self.ctx.ctx, h)
                del buf
        return self.bytes + need <= self.budget

    def handle(self, scene: int):
        """RRDevicePtr of a resident scene's buffer, made once and kept while it is resident."""
        import ctypes as C
        h = self.handles.get(scene)
        if h is None:
            h = C.c_void_p()
            rr.check(self.ctx.L.rrGetDevicePtrFromCudaPtr(self.ctx.ctx, C.c_void_p(self.resident[scene].data_ptr()),
                                                          0, C.byref(h)), "rrGetDevicePtrFromCudaPtr")
            self.handles[scene] = h
        return h

    def build(self, scene: int):
        """Build one scene's BVH through rrCmdBuildGeometry; returns the result buffer."""
        import torch
        v, i = self.meshes[scene]
        vd = torch.from_numpy(v).cuda()
        idd = torch.from_numpy(i.view(np.int32)).cuda()
        buf = self.ctx.build_geometry(vd, idd, node_format=self.node_format)
        self.ctx.release_ptrs()
        return buf

    def acquire(self, scene: int):
        """Pin the scene's BVH (building it if needed) and return its result buffer."""
        if scene in self.resident:
            self.resident.move_to_end(scene)
            self.pins[scene] += 1
            return self.resident[scene]
        need = self.result_bytes(scene)
        if not self._make_room(need):
            raise MemoryError(f"scene {scene} ({need} bytes) does not fit the budget")
        buf = self.build(scene)
        self.builds += 1
        self.resident[scene] = buf
        self.bytes += buf.numel()
        self.pins[scene] += 1
        return buf

    def release(self, scene: int) -> None:
        self.pins[scene] -= 1


class _Slot:
    def __init__(self, ctx: rr.Context, slot_rays: int, max_requests: int):
        import torch
        self.stream = torch.cuda.Stream()
        self.cs = ctx.external_stream(self.stream)
        self.rays = torch.empty((slot_rays, 8), dtype=torch.float32, device="cuda")
        self.hits = torch.empty((slot_rays, 4), dtype=torch.int32, device="cuda")
        self.scratch = torch.empty(ctx.batch_scratch_bytes(max_requests, slot_rays), dtype=torch.uint8,
                                   device="cuda")
        # Handles of the arenas, made once (the loop passes them every launch).
        self.h_rays, self.h_hits, self.h_scratch = (self._handle(ctx, t) for t in (self.rays, self.hits,
                                                                                  self.scratch))
        self.event = torch.cuda.Event()
        self.busy = False
        self.reqs: list[tuple[Request, int]] = []  # (request, ray offset in the arena)
        self.launches = 0

    @staticmethod
    def _handle(ctx, t):
        import ctypes as C
        h = C.c_void_p()
        rr.check(ctx.L.rrGetDevicePtrFromCudaPtr(ctx.ctx, C.c_void_p(t.data_ptr()), 0, C.byref(h)),
                 "rrGetDevicePtrFromCudaPtr")
        return h


class Server:
    """Continuous-batching request loop over a ScenePool."""

    def __init__(self, ctx: rr.Context, pool: ScenePool, slot_rays: int = 1 << 22, slots: int = 2,
                 max_requests: int = 256):
        self.ctx = ctx
        self.pool = pool
        self.slot_rays = int(slot_rays)
        self.max_requests = int(max_requests)
        self.slots = [_Slot(ctx, self.slot_rays, self.max_requests) for _ in range(slots)]

    def _admit(self, queue: collections.deque) -> list:
        """Oldest-first requests that fit one slot's arena and the scene
        budget; their scenes are pinned (built if not resident)."""
        batch, rays = [], 0
        while queue and len(batch) < self.max_requests:
            r = queue[0]
            n = r.rays.shape[0]
            if rays + n > self.slot_rays:
                break
            try:
                bvh = self.pool.acquire(r.scene)
            except MemoryError:
                break
            batch.append((queue.popleft(), bvh))
            rays += n
        return batch

    def _launch(self, slot: _Slot, batch: list, now: float) -> None:
        """One rrCudaCmdIntersectBatchHost on the slot's stream: the library
        copies every request's rays in, fills the hit arena, traces all
        requests in one persistent launch and copies every request's hits
        back to its pinned buffer (misses read 0xFFFFFFFF outside inst_id)."""
        import ctypes as C
        off = 0
        slot.reqs = []
        arr = (rr.RRCudaHostIntersectRequest * len(batch))()
        for k, (r, _) in enumerate(batch):
            n = r.rays.shape[0]
            rays_h, hits_h = self._pinned[r.rid]
            arr[k] = rr.RRCudaHostIntersectRequest(self.pool.handle(r.scene), r.query, r.output,
                                                   C.c_void_p(rays_h.data_ptr()), n, C.c_void_p(hits_h.data_ptr()))
            slot.reqs.append((r, off))
            off += n
        rr.check(self.ctx.L.rrCudaCmdIntersectBatchHost(self.ctx.ctx, len(batch), arr, slot.h_rays, slot.h_hits,
                                                        slot.h_scratch, slot.cs), "rrCudaCmdIntersectBatchHost")
        slot.event.record(slot.stream)
        for r, _ in batch:
            r.admitted = now
        slot.busy = True
        slot.launches += 1

    def _complete(self, slot: _Slot, now: float) -> int:
        for r, o in slot.reqs:
            n = r.rays.shape[0]
            hh = self._pinned[r.rid][1].numpy().view(np.uint32)
            r.hits = hh if r.output == rr.RR_INTERSECT_QUERY_OUTPUT_FULL_HIT else hh.reshape(-1)[:n]
            r.done = now
            self.pool.release(r.scene)
        done = len(slot.reqs)
        slot.reqs = []
        slot.busy = False
        return done

    def _pin(self, requests) -> None:
        """Page-locked host buffers of every request's rays and hit records (a
        client of the loop hands over pinned buffers; done before the clock
        starts).  Requests with pinned views of a ray pool use those, and take
        their hit records from a pinned ring in arrival order: admission is
        oldest first, so requests in flight together never share ring memory
        while the ring holds twice the rays all slots can hold.  A ring
        request's `hits` stay valid until the ring comes round again."""
        import torch
        self._pinned = {}
        ring_req = [r for r in requests if r.pinned_rays is not None]
        ring_rays = 2 * len(self.slots) * self.slot_rays
        if ring_req and (getattr(self, "_ring", None) is None or self._ring.shape[0] < ring_rays):
            self._ring = torch.empty((ring_rays, 4), dtype=torch.int32).pin_memory()
        cur = 0
        for r in sorted(requests, key=lambda q: q.arrival):
            n = r.rays.shape[0]
            if r.pinned_rays is not None:
                if cur + n > self._ring.shape[0]:
                    cur = 0
                self._pinned[r.rid] = (r.pinned_rays, self._ring[cur:cur + n])
                cur += n
                continue
            rays = torch.from_numpy(np.ascontiguousarray(r.rays, np.float32)).pin_memory()
            hits = torch.empty((n, 4), dtype=torch.int32).pin_memory()
            self._pinned[r.rid] = (rays, hits)

    def run(self, requests: list[Request], poll_sleep: float = 2e-5) -> dict:
        """Serve `requests` (arrival times in seconds from now) to completion;
        returns throughput and latency figures."""
        for r in requests:
            if r.rays.shape[0] > self.slot_rays:
                raise ValueError(f"request {r.rid} has {r.rays.shape[0]} rays, more than a slot holds")
        self._pin(requests)
        # The loop allocates little, but a cyclic-garbage pass in the middle
        # of it delays every request in flight: collection waits until the
        # requests are served.
        gc_on = gc.isenabled()
        gc.disable()
        try:
            return self._serve(requests, poll_sleep)
        finally:
            if gc_on:
                gc.enable()

    def _serve(self, requests: list[Request], poll_sleep: float) -> dict:
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        queue: collections.deque[Request] = collections.deque()
        t0 = time.perf_counter()
        left = len(requests)
        while left:
            now = time.perf_counter() - t0
            while pending and pending[0].arrival <= now:
                queue.append(pending.popleft())
            progressed = False
            for s in self.slots:
                if s.busy and s.event.query():
                    left -= self._complete(s, time.perf_counter() - t0)
                    progressed = True
            for s in self.slots:
                if s.busy or not queue:
                    continue
                batch = self._admit(queue)
                if batch:
                    self._launch(s, batch, time.perf_counter() - t0)
                    progressed = True
            if not progressed:
                if queue and all(not s.busy for s in self.slots):
                    raise MemoryError("a queued request cannot be admitted: its scene does not fit the budget")
                time.sleep(poll_sleep)
        end = time.perf_counter() - t0
        lat = np.array([r.latency for r in requests])
        rays = sum(r.rays.shape[0] for r in requests)
        return {"requests": len(requests), "rays": int(rays), "makespan_s": end,
                "throughput_mrays_s": rays / end / 1e6,
                "latency_ms": {"p50": 1e3 * float(np.percentile(lat, 50)), "p99": 1e3 * float(np.percentile(lat, 99)),
                               "max": 1e3 * float(lat.max())},
                "launches": sum(s.launches for s in self.slots), "scene_builds": self.pool.builds,
                "scene_evictions": self.pool.evictions, "resident_bytes": self.pool.bytes}


def config4(n_scenes: int = 64, lo_tris: float = 1e4, hi_tris: float = 2e6, seed: int = 4):
    """Scenes of the serving workload: log-uniform triangle counts, soup or
    heightfield by a seeded bit.  Returns [(vertices, indices), ...]."""
    import math
    from . import scenes
    g = scenes.rng(seed)
    out = []
    for k in range(n_scenes):
        n = int(round(math.exp(g.uniform(math.log(lo_tris), math.log(hi_tris)))))
        if g.integers(0, 2):
            grid = max(2, int(round(math.sqrt(n / 2.0))) + 1)
            out.append(scenes.heightfield(grid, scenes.rng(seed, 100 + k)))
        else:
            out.append(scenes.soup(n, scenes.rng(seed, 100 + k)))
    return out


class RayPools:
    """Pinned host pools of incoherent rays, one closest-hit and one any-hit
    pool (tmax ~ U[0.01, 0.5]) of `pool_rays` rays per scene, so that long
    runs of requests need no per-request host buffers.  One unit pool
    (origins in [0, 1]^3, directions uniform on the sphere) is mapped into
    each scene's bounding box."""

    def __init__(self, meshes, pool_rays: int = 1 << 20, seed: int = 4):
        import torch
        from . import scenes
        self.pool_rays = int(pool_rays)
        g = scenes.rng(seed, 9)
        unit = scenes.incoherent_rays(self.pool_rays, (0, 0, 0), (1, 1, 1), g)
        tmax_any = g.uniform(0.01, 0.5, size=self.pool_rays).astype(np.float32)
        self.closest, self.any = [], []
        for v, _ in meshes:
            lo, hi = v.min(axis=0).astype(np.float64), v.max(axis=0).astype(np.float64)
            r = unit.copy()
            r[:, 0:3] = (lo + unit[:, 0:3].astype(np.float64) * (hi - lo)).astype(np.float32)
            self.closest.append(torch.from_numpy(r).pin_memory())
            r[:, 7] = tmax_any
            self.any.append(torch.from_numpy(r).pin_memory())


def make_requests(meshes, n_requests: int, rate_per_s: float, lo_rays: int = 1024, hi_rays: int = 1 << 20,
                  any_fraction: float = 0.3, seed: int = 4, pools: RayPools | None = None) -> list[Request]:
    """Poisson arrivals at `rate_per_s`; request sizes log-uniform in
    [lo_rays, hi_rays]; 30% any-hit (tmax ~ U[0.01, 0.5]) and 70% closest-hit
    incoherent rays inside the scene's box.  With `pools`, a request's rays
    are a random slice of its scene's pinned pool (no copy)."""
    import math
    from . import scenes
    g = scenes.rng(seed, 7)
    t = 0.0
    reqs = []
    for k in range(n_requests):
        t += g.exponential(1.0 / rate_per_s)
        sid = int(g.integers(0, len(meshes)))
        n = int(round(math.exp(g.uniform(math.log(lo_rays), math.log(hi_rays)))))
        v = meshes[sid][0]
        any_hit = g.random() < any_fraction
        q = rr.RR_INTERSECT_QUERY_ANY if any_hit else rr.RR_INTERSECT_QUERY_CLOSEST
        if pools is not None:
            n = min(n, pools.pool_rays)
            off = int(g.integers(0, pools.pool_rays - n + 1))
            pool = (pools.any if any_hit else pools.closest)[sid]
            view = pool[off:off + n]
            reqs.append(Request(k, t, sid, view.numpy(), q, pinned_rays=view))
            continue
        rays = scenes.incoherent_rays(n, v.min(axis=0), v.max(axis=0), scenes.rng(seed, 1000 + k))
        if any_hit:
            rays[:, 7] = g.uniform(0.01, 0.5, size=n).astype(np.float32)
        reqs.append(Request(k, t, sid, rays, q))
    return reqs
