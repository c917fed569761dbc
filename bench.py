"""Benchmark of the RadeonRays GB300 intersection path.

Workload (one GPU): the 1449 x 1449-vertex heightfield (4,193,408 triangles,
z = 0.1 * sum of 8 seeded sinusoids) and 16,777,216 incoherent rays (origins
uniform in its bounding box, directions uniform on the sphere), closest hit,
full RRHit output.  A step is one rrCmdIntersect over all rays.

Reported (one JSON line on rank 0):
  value        chosen path Mrays/s (the kernel rrCudaAutotuneTraversal picks
               for this workload: plain, persistent binary or 8-wide), rays
               and BVH resident in HBM, CUDA events on the launch stream
  plain        the plain binary-node kernel on the same rays (reference order)
  latency_ms   p50 / p99 of the per-step (per-batch) latency of the chosen path
  e2e          the same metric through the C-ABI with pinned host buffers:
               H2D of the rays, trace, D2H of the hits inside the timed region
               (one streamed launch that traces each chunk of rays as it lands
               and whose hits are copied out part by part as they complete)
  roofline     algorithmic bytes of the chosen kernel per launch (ray + hit +
               node bytes x node fetches + 48 B x triangle fetches, counted by
               the kernel's own counters) / mean launch time, against the
               measured HBM copy bandwidth
  build        LBVH + wide collapse of the mesh through rrCmdBuildGeometry
  hit_id_identity  chosen vs plain on every ray
  any_hit      occlusion rays (same rays, tmax ~ U[0.01, 0.5]): chosen (autotuned
               for any hit) and plain Mrays/s, hit-flag identity
  precision_wide8  the 8-wide nodes with 8-bit conservative bounds on the fast
               tree: Mrays/s, hit identity against the plain kernel on
               every ray, and its own fp64 t / uv error
  fp64_t_error t / uv error of the chosen hits against an fp64 evaluation of
               the same ray-triangle pairs on the first 1,048,576 rays
  precise      the opt-in precise triangle test (watertight decision, accurate
               t and uv in fp32): Mrays/s of its autotuned kernel, its hit
               differences from the plain kernel classified, and its own fp64
               t / uv error
  cpu_baseline the oracle's C++ restatement of the reference traversal on the
               host cores, on a bounded sample of the same rays
With --gpus N under torchrun every rank traces its own 16,777,216 rays against
its own replica of the BVH (replicas only: the path has no exchange step).

  blas2048     the batching configuration: fused build of 2,048 BLASes and
               two-level traversal, chosen vs plain (summary of
               --workload blas2048, without its one-by-one build baseline)
  serving      the serving configuration: resident scenes, continuous
               batching, throughput and p50/p99 request latency at 50/80/95%
               of saturation, 10,000 requests per load point, and a checked
               sample (summary of --workload serving)
Other workloads (their own JSON line): --workload blas2048 and
--workload serving.

--impl reference times the reference's CPU implementation of the path (the
oracle port of isect.comp; the reference's own bvh_analyzer cannot be built
on the GPU host) on the host cores, on a bounded sample of each step.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "incoherent closest-hit Mrays/s + p99 batch latency, chosen vs plain on same GB300"
# RRCudaTraversal value -> kernel name (the key of profiles/traffic.json)
KERNELS = {1: "k_trace_binary", 2: "k_trace_wide", 3: "k_trace_persistent", 4: "k_trace_bvh4"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--grid", type=int, default=1449)
    ap.add_argument("--rays", type=int, default=16_777_216)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-anyhit", action="store_true", help="skip the any-hit (occlusion) measurement")
    ap.add_argument("--no-precision", action="store_true",
                    help="skip the 8-wide 8-bit-bounds run (hit identity and fp64 error of that format)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the batching (2,048 BLASes) and serving summaries of the default line")
    ap.add_argument("--no-precise", action="store_true",
                    help="skip the precise triangle test run (watertight, accurate t; opt-in mode)")
    ap.add_argument("--e2e-chunk", type=int, default=0,
                    help="rays per copy-in chunk of the e2e run (0: the library's default, 2^17)")
    ap.add_argument("--quality", type=int, default=1,
                    help="1: the chosen path traces a quality build (treelet restructure); 0: the fast build")
    ap.add_argument("--only", default="", help="profiling aid: 'chosen' or 'plain' runs only that kernel")
    ap.add_argument("--block", type=int, default=0, help="chosen kernel threads per block (0: library default)")
    ap.add_argument("--per-sm", type=int, default=0, help="chosen kernel resident blocks per SM (0: occupancy)")
    ap.add_argument("--ray-order", type=int, default=0, help="chosen kernel: 0 default, 1 given order, 2 sorted")
    ap.add_argument("--workload", default="heightfield", choices=["heightfield", "blas2048", "serving"],
                    help="heightfield: the headline line; blas2048: fused multi-BLAS build + two-level traversal; "
                         "serving: resident scenes + continuous batching")
    ap.add_argument("--blas", type=int, default=2048)
    ap.add_argument("--batch-rays", type=int, default=8_388_608)
    ap.add_argument("--no-separate", action="store_true",
                    help="blas2048: skip the one-by-one build baseline (about 160,000 launches)")
    ap.add_argument("--scenes", type=int, default=64)
    ap.add_argument("--requests", type=int, default=10000, help="serving: requests per load point")
    ap.add_argument("--slots", type=int, default=3)
    ap.add_argument("--scene-format", default="bvh4q8", choices=["bvh4", "bvh4q8", "binary"],
                    help="serving: node format of the resident scenes (bvh4 and bvh4q8 run the 4-wide "
                         "multi-request kernel over fp32 or 8-bit nodes)")
    ap.add_argument("--slot-rays", type=int, default=1 << 22)
    ap.add_argument("--hbm-budget-gb", type=float, default=120.0)
    ap.add_argument("--chosen-format", default="auto", choices=["auto", "wide8", "bvh4", "bvh4q8"],
                    help="node format of the chosen path's tree (the binary nodes are always there); auto: the "
                         "node-format autotuner's pick (rrCudaAutotuneNodeFormat) on the workload's rays")
    ap.add_argument("--chosen", type=int, default=0,
                    help="chosen traversal: 0 autotuned (rrCudaAutotuneTraversal), 2 wide (8-wide nodes, "
                         "--chosen-format wide8), 3 binary persistent, 4 4-wide fp32 nodes (--chosen-format bvh4)")
    return ap.parse_args()


def dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as tdist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        tdist.init_process_group(backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as tdist
        tdist.barrier()


def max_over_ranks(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as tdist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi samples every 20 ms while the timed region runs (the
    sampler is running before the region starts: __enter__ waits for its
    first line)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index, self.lines, self.proc = index, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.perf_counter()
            while not self.lines and time.perf_counter() - t0 < 3.0:
                time.sleep(0.005)
            self.skip = len(self.lines)  # samples taken before the timed region are not reported
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines[getattr(self, "skip", 0):] or self.lines[-1:]
        for ln in lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def workload(args, rank):
    from radeonrays_sdk_gb300 import scenes
    g = scenes.rng(1)
    v, i = scenes.heightfield(args.grid, g)
    lo, hi = v.min(axis=0), v.max(axis=0)
    rays = scenes.incoherent_rays(args.rays, lo, hi, scenes.rng(1, 1 + rank))
    return v, i, rays


def describe(args, ntri):
    return {"workload": f"heightfield {args.grid}x{args.grid} vertices ({ntri:,} triangles), {args.rays:,} incoherent "
                        "rays per GPU (origins uniform in the mesh box, directions uniform on the sphere), "
                        "closest hit, full RRHit output",
            "triangles": ntri, "rays_per_gpu": args.rays, "query": "closest", "output": "full_hit",
            "chosen": "autotuned: the node format (rrCudaAutotuneNodeFormat: 4-wide nodes with fp32 bounds "
                      "(bvh4) or 8-bit bounds (bvh4q8), or 8-wide 8-bit nodes (wide8)), then the kernel "
                      "(rrCudaAutotuneTraversal among plain binary, persistent lane-refill binary and the format's "
                      "wide kernel), the winner's resident blocks per SM and (4-wide) shared-stack depth; format "
                      f"here: {args.chosen_format}",
            "plain": "64-byte binary nodes, one thread per ray, reference visit order",
            "l2": "inputs larger than L2 (rays 32 B x rays, BVH > 129 MB); no flush needed",
            "parallelism": "replicas (rays sharded per GPU, BVH replicated)"}


def cpu_model():
    """The host CPU's model name (or its part and implementer codes on Arm)."""
    try:
        text = open("/proc/cpuinfo").read()
    except OSError:
        return None
    for key in ("model name", "Model Name"):
        for ln in text.splitlines():
            if ln.startswith(key):
                return ln.split(":", 1)[1].strip()
    parts = {ln.split(":", 1)[0].strip(): ln.split(":", 1)[1].strip() for ln in text.splitlines() if ":" in ln}
    if "CPU part" in parts:
        return f"{os.uname().machine} CPU implementer {parts.get('CPU implementer')} part {parts['CPU part']}"
    return os.uname().machine


def cpu_baseline(v, i, rays, seconds, threads=None):
    """Oracle port of isect.comp on the host cores over a bounded ray sample,
    and the oracle's C++ LBVH restatement (the reference has no CPU builder)
    timed on one thread and on all cores."""
    import oracle
    oracle.build()
    threads = threads or os.cpu_count() or 1
    t0 = time.perf_counter()
    oracle.build_mesh(v, i, threads=1)
    build_1 = time.perf_counter() - t0
    t0 = time.perf_counter()
    nodes, _, _ = oracle.build_mesh(v, i, threads=threads)
    build_n = time.perf_counter() - t0
    n = 1 << 14
    t0 = time.perf_counter()
    oracle.trace(nodes, rays[:n], threads=threads)
    dt = time.perf_counter() - t0
    target = int(min(rays.shape[0], max(n, n * seconds / max(dt, 1e-6))))
    t0 = time.perf_counter()
    oracle.trace(nodes, rays[:target], threads=threads)
    dt = time.perf_counter() - t0
    ntri = i.shape[0]
    return {"value": target / dt / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
            "sample": f"first {target:,} rays of the workload, closest hit, binary nodes built by the oracle",
            "cpu_model": cpu_model(),
            "build": {"kind": "port (the oracle's C++ LBVH restatement: bounds, Morton codes, stable sort, "
                              "Karras emit, refit)",
                      "ms_1_thread": 1e3 * build_1, "mtris_s_1_thread": ntri / build_1 / 1e6,
                      "ms_all_cores": 1e3 * build_n, "mtris_s_all_cores": ntri / build_n / 1e6,
                      "cores": threads}}, nodes


def precision_report(v, i, rays, hits, nodes, n=1 << 20, precise=False):
    """t and uv error of the fp32 closest hits against the exact (fp64)
    intersection of the same ray with the same triangle, on the first n rays.
    `hits` are the chosen path's RRHit records (uint32 view); t32 is the
    oracle's fp32 distance, which equals the kernels' (same arithmetic: the
    reference's test, or with `precise` the precise triangle test)."""
    import oracle
    sub = rays[:n]
    h = hits[:n]
    hit = h[:, 2] != 0xFFFFFFFF
    if precise:
        t32 = oracle.trace_precise(nodes, sub, threads=os.cpu_count() or 1)[1]
    else:
        t32 = oracle.trace_t(nodes, sub, threads=os.cpu_count() or 1)
    idx = i.astype(np.int64)
    tri9 = np.zeros((n, 9), np.float32)
    tri9[hit] = v[idx[h[hit, 3]]].reshape(-1, 9)
    e = oracle.fp64_hit(sub, tri9, hit.astype(np.uint32))
    t = t32[hit].astype(np.float64)
    ulp = np.abs(t - e[hit, 0]) / np.spacing(np.abs(t32[hit])).astype(np.float64)
    uv = h[hit, :2].view(np.float32).astype(np.float64)
    uv_err = np.abs(uv - e[hit, 1:3]).max(axis=1)
    return {"rays": int(n), "hits": int(hit.sum()), "t_ulp_max": float(ulp.max()), "t_ulp_mean": float(ulp.mean()),
            "t_ulp_p999": float(np.percentile(ulp, 99.9)), "t_within_2ulp": float(np.mean(ulp <= 2.0)),
            "uv_abs_err_max": float(uv_err.max()), "uv_abs_err_mean": float(uv_err.mean()),
            "reference": "fp64 Moller-Trumbore + barycentrics of the same ray and triangle (oracle rro_fp64_hit)"}


def classify_mismatches(v, i, rays, a, b, diff):
    """Closest-hit rays where kernels a and b kept different triangles
    (`diff`), by the gap between the two triangles' fp32 distances (the
    reference's triangle test): equal t, within 2 ulp, farther apart."""
    rep = {"mismatches": int(diff.size), "mismatches_are_equal_t_ties": None, "equal_t": None,
           "within_2ulp": None, "farther_than_2ulp": None, "mismatch_t_gap_ulp_max": None}
    if diff.size == 0:
        rep.update({"mismatches_are_equal_t_ties": True, "equal_t": 0, "within_2ulp": 0, "farther_than_2ulp": 0,
                    "mismatch_t_gap_ulp_max": 0.0})
    elif diff.size < 100000:
        import oracle
        idx = i.astype(np.int64)
        ta = oracle.tri_test(rays[diff], v[idx[a[diff, 3]]].reshape(-1, 9))[:, 0]
        tb = oracle.tri_test(rays[diff], v[idx[b[diff, 3]]].reshape(-1, 9))[:, 0]
        gap = np.abs(ta.astype(np.float64) - tb) / np.spacing(np.maximum(np.abs(ta), np.abs(tb))).astype(np.float64)
        rep.update({"mismatches_are_equal_t_ties": bool(np.all(gap == 0)), "equal_t": int(np.sum(gap == 0)),
                    "within_2ulp": int(np.sum((gap > 0) & (gap <= 2))), "farther_than_2ulp": int(np.sum(gap > 2)),
                    "mismatch_t_gap_ulp_max": float(gap.max())})
    return rep


def precise_vs_plain(v, i, rays, hp, ph):
    """Hit-ID differences of the precise triangle test from the plain kernel
    (the reference's test) on every ray, classified: hit flags that differ
    either way, and for rays where both hit different triangles the gap
    between the two triangles' precise distances."""
    import oracle
    mp, mr = hp[:, 2] != 0xFFFFFFFF, ph[:, 2] != 0xFFFFFFFF
    diff = np.where(mp & mr & (hp[:, 3] != ph[:, 3]))[0]
    rep = {"rays": int(rays.shape[0]), "hit_only_with_precise": int(np.sum(mp & ~mr)),
           "hit_only_with_reference_test": int(np.sum(mr & ~mp)), "different_triangle": int(diff.size)}
    if diff.size and diff.size < 200000:
        idx = i.astype(np.int64)
        ta = oracle.tri_test_precise(rays[diff], v[idx[hp[diff, 3]]].reshape(-1, 9))[:, 0].astype(np.float64)
        tb = oracle.tri_test_precise(rays[diff], v[idx[ph[diff, 3]]].reshape(-1, 9))[:, 0].astype(np.float64)
        gap = np.abs(ta - tb) / np.spacing(np.abs(ta).astype(np.float32)).astype(np.float64)
        gap[~np.isfinite(tb)] = np.inf  # the plain path's triangle is no hit for the precise test
        rep.update({"plain_triangle_at_equal_t": int(np.sum(gap == 0)),
                    "plain_triangle_within_2ulp": int(np.sum((gap > 0) & (gap <= 2))),
                    "plain_triangle_farther_than_2ulp": int(np.sum(gap > 2)),
                    "precise_triangle_never_farther": bool(np.all(ta <= tb)),
                    "note": "distances by the precise test; where they differ by more than 2 ulp, the "
                            "reference's arithmetic kept a triangle that is not the nearest"})
    return rep


def run_reference(args):
    """--impl reference: the reference's traversal (oracle port) on the host cores."""
    ws, rank, _ = dist()
    if rank != 0:
        return
    v, i, rays = workload(args, 0)
    import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    nodes, _, _ = oracle.build_mesh(v, i, threads=threads)
    # Size a step so the whole run stays within a few minutes.
    n = 1 << 14
    t0 = time.perf_counter()
    oracle.trace(nodes, rays[:n], threads=threads)
    per_ray = (time.perf_counter() - t0) / n
    budget = 150.0 / max(1, args.steps + args.warmup)
    sample = int(max(n, min(rays.shape[0], budget / per_ray)))
    for k in range(args.warmup):
        oracle.trace(nodes, rays[:sample], threads=threads)
    times = []
    for k in range(args.steps):
        off = (k * sample) % max(1, rays.shape[0] - sample + 1)
        t0 = time.perf_counter()
        oracle.trace(nodes, rays[off:off + sample], threads=threads)
        times.append(time.perf_counter() - t0)
    value = sample * len(times) / sum(times) / 1e6
    line = {"metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": describe(args, i.shape[0]), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": threads, "kind": "port",
                             "sample": f"{sample:,} rays per step of the same workload (oracle restatement of "
                                       "isect.comp; bvh_analyzer is not buildable on the GPU host)"},
            "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "latency_ms": {"p50": 1e3 * statistics.median(times), "p99": 1e3 * float(np.percentile(times, 99))}}
    print(json.dumps(line), flush=True)


def time_steps(step, K, W, ws, stream):
    import torch
    for _ in range(W):
        step()
    torch.cuda.synchronize()
    barrier(ws)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    for s, e in ev:
        s.record(stream)
        step()
        e.record(stream)
    torch.cuda.synchronize()
    barrier(ws)
    torch.cuda.synchronize()
    per = [s.elapsed_time(e) for s, e in ev]
    total = ev[0][0].elapsed_time(ev[-1][1])
    return per, total


def run_ours(args):
    import torch
    ws, rank, local = dist()
    torch.cuda.set_device(local)
    from radeonrays_sdk_gb300 import rr
    v, i, rays = workload(args, rank)
    R, ntri = rays.shape[0], i.shape[0]
    ctx = rr.Context()
    stream = torch.cuda.current_stream()
    ext = ctx.external_stream(stream)
    v_d = torch.from_numpy(v).cuda()
    i_d = torch.from_numpy(i.view(np.int32)).cuda()

    # ---- build (LBVH + wide collapse) through rrCmdBuildGeometry
    # The library's default node format (binary + 4-wide nodes with 8-bit bounds).
    dfmt = rr.RR_CUDA_NODE_FORMAT_BVH4Q8
    s_bytes, r_bytes = ctx.geometry_requirements(ntri, dfmt, 30, v.shape[0], 12)
    scratch_b = torch.empty(s_bytes, dtype=torch.uint8, device="cuda")
    bvh = torch.empty(r_bytes, dtype=torch.uint8, device="cuda")

    def build_step():
        ctx.build_geometry(v_d, i_d, node_format=dfmt, stream=ext, scratch=scratch_b, result=bvh)
        ctx.release_ptrs()
    b_per, b_total = time_steps(build_step, 5, 2, 1, stream)
    build = {"ms": statistics.median(b_per), "mtris_s": ntri / statistics.median(b_per) / 1e3,
             "format": "binary + bvh4q8 (the default)", "triangles": ntri,
             "flags": "PREFER_FAST_BUILD (reference LBVH)"}
    # RR_BUILD_OPERATION_UPDATE (refit of the same topology, then the 4-wide
    # collapse again) with the vertices moved up by 1 %; then back, so that
    # the tree traced below is the built one.
    v_up = (v_d * 1.01).contiguous()
    u_scratch = torch.empty(max(1, s_bytes), dtype=torch.uint8, device="cuda")

    def update_step(vv=v_up):
        ctx.update_geometry(vv, i_d, bvh, stream=ext, scratch=u_scratch)
        ctx.release_ptrs()
    u_per, _ = time_steps(update_step, 5, 2, 1, stream)
    update_step(v_d)
    torch.cuda.synchronize()
    build["update"] = {"ms": statistics.median(u_per), "mtris_s": ntri / statistics.median(u_per) / 1e3,
                       "operation": "RR_BUILD_OPERATION_UPDATE: leaves take the new vertices, atomic refit, "
                                    "4-wide nodes requantised in place (topology kept)"}
    del v_up
    # The chosen path traces a quality build (flags without PREFER_FAST_BUILD:
    # LBVH + treelet restructure); the plain path the reference's fast LBVH.
    bvh_c = bvh
    format_tuned = None
    if args.chosen_format == "auto":
        # The node-format autotuner: builds the chosen tree in each wide
        # format, tunes the traversal of each on the workload's rays (untimed)
        # and keeps the fastest.
        rays_tune = torch.from_numpy(rays).cuda()
        cfmt = ctx.autotune_node_format(v_d, i_d, rays_tune, quality=bool(args.quality))
        format_tuned = {rr.RR_CUDA_NODE_FORMAT_BVH4: "bvh4", rr.RR_CUDA_NODE_FORMAT_BVH4Q8: "bvh4q8",
                        rr.RR_CUDA_NODE_FORMAT_WIDE8: "wide8"}[cfmt]
        del rays_tune
        torch.cuda.empty_cache()
    else:
        cfmt = {"bvh4": rr.RR_CUDA_NODE_FORMAT_BVH4, "bvh4q8": rr.RR_CUDA_NODE_FORMAT_BVH4Q8,
                "wide8": rr.RR_CUDA_NODE_FORMAT_WIDE8}[args.chosen_format]
    if args.quality or cfmt != dfmt:
        cs_bytes, cr_bytes = ctx.geometry_requirements(ntri, cfmt, 30, v.shape[0], 12)
        bvh_c = torch.empty(cr_bytes, dtype=torch.uint8, device="cuda")
        scratch_c = scratch_b if cs_bytes <= scratch_b.numel() else torch.empty(cs_bytes, dtype=torch.uint8,
                                                                                  device="cuda")

        def qbuild_step():
            ctx.build_geometry(v_d, i_d, node_format=cfmt, stream=ext, scratch=scratch_c, result=bvh_c,
                               quality=bool(args.quality))
            ctx.release_ptrs()
        q_per, _ = time_steps(qbuild_step, 3, 1, 1, stream)
        build["quality"] = {"ms": statistics.median(q_per), "mtris_s": ntri / statistics.median(q_per) / 1e3,
                            "format": "binary + " + {rr.RR_CUDA_NODE_FORMAT_BVH4: "bvh4",
                                                     rr.RR_CUDA_NODE_FORMAT_BVH4Q8: "bvh4q8",
                                                     rr.RR_CUDA_NODE_FORMAT_WIDE8: "wide8"}[cfmt],
                            "flags": "no PREFER_FAST_BUILD: LBVH + 3 treelet-restructure passes (nodes >= 64 tris)"}

    rays_d = torch.from_numpy(rays).cuda()
    hits_d = torch.empty((R, 4), dtype=torch.int32, device="cuda")
    scratch_t = torch.empty(ctx.trace_scratch_bytes(R), dtype=torch.uint8, device="cuda")
    hb, hcb, rb, hitb = ctx.ptr(bvh), ctx.ptr(bvh_c), ctx.ptr(rays_d), ctx.ptr(hits_d)
    sb = ctx.ptr(scratch_t)
    L = ctx.L
    cur = {"bvh": hcb}

    def trace_step():
        rr.check(L.rrCmdIntersect(ctx.ctx, cur["bvh"], rr.RR_INTERSECT_QUERY_CLOSEST, rb, R, None,
                                  rr.RR_INTERSECT_QUERY_OUTPUT_FULL_HIT, hitb, sb, ext), "rrCmdIntersect")

    out = {}
    # Chosen path: the autotuner's pick (untimed tuning on the workload's rays)
    # unless a kernel is forced on the command line.
    chosen_trav, chosen_order, tuned = args.chosen, args.ray_order, None
    chosen_per_sm, chosen_stack = args.per_sm, 0
    if args.chosen == 0 and args.only != "plain":
        tuned = ctx.autotune(bvh_c, rays_d, hits=hits_d, scratch=scratch_t)
        chosen_trav, chosen_order = tuned["traversal"], tuned["ray_order"]
        chosen_per_sm = args.per_sm or tuned["blocks_per_sm"]
        chosen_stack = tuned["short_stack"]
    # Fetch counters of each kernel (untimed run) -> algorithmic bytes.
    for name, trav in (("chosen", chosen_trav), ("plain", rr.RR_CUDA_TRAVERSAL_BINARY)):
        if args.only and args.only != name:
            continue
        if name == "plain" and args.no_plain:
            continue
        shape = (args.block, chosen_per_sm) if name == "chosen" else (0, 0)
        order = chosen_order if name == "chosen" else 0
        depth = chosen_stack if name == "chosen" else 0
        cur["bvh"] = hcb if name == "chosen" else hb
        ctx.set_traversal(trav, *shape, collect_stats=1, ray_order=order, short_stack=depth)
        trace_step()
        torch.cuda.synchronize()
        st = ctx.stats()
        ctx.set_traversal(trav, *shape, ray_order=order, short_stack=depth)
        # Bytes per fetch: binary node 64; 8-wide node 80 (+ 48-byte triangles);
        # 4-wide node 128 (+ the 48 bytes of a binary leaf's three vertices).
        node_b = {rr.RR_CUDA_TRAVERSAL_WIDE: 80,
                  rr.RR_CUDA_TRAVERSAL_BVH4: 64 if cfmt == rr.RR_CUDA_NODE_FORMAT_BVH4Q8 else 128}.get(trav, 64)
        if name == "plain":
            node_b = 64
        alg = R * (32 + 16) + st["node_fetches"] * node_b + st["triangle_fetches"] * 48
        clocks = Clocks(local)
        with clocks:
            per, total = time_steps(trace_step, args.steps, args.warmup, ws, stream)
        total = max_over_ranks(total, ws)
        out[name] = {"per": per, "total": total, "alg_bytes": alg, "stats": st, "clocks": clocks.summary(),
                     "hits": hits_d.cpu().numpy().view(np.uint32).copy(), "trav": trav, "order": order}
    assert ctx.device_errors() == 0, "device error word set during the benchmark"

    # ---- 8-wide nodes with 8-bit conservative child bounds (the precision
    # configuration): the fast tree in the WIDE8 format, traced by the 8-wide
    # kernel, against the plain kernel's hits on the same binary tree.
    wide8 = None
    if not args.no_precision and "plain" in out and not args.only:
        s8, r8 = ctx.geometry_requirements(ntri, rr.RR_CUDA_NODE_FORMAT_WIDE8, 30, v.shape[0], 12)
        scratch8 = scratch_b if s8 <= scratch_b.numel() else torch.empty(s8, dtype=torch.uint8, device="cuda")
        bvh8 = torch.empty(r8, dtype=torch.uint8, device="cuda")
        ctx.build_geometry(v_d, i_d, node_format=rr.RR_CUDA_NODE_FORMAT_WIDE8, stream=ext, scratch=scratch8,
                           result=bvh8)
        cur["bvh"] = ctx.ptr(bvh8)
        ctx.set_traversal(rr.RR_CUDA_TRAVERSAL_WIDE, collect_stats=1, ray_order=1)
        trace_step()
        torch.cuda.synchronize()
        st8 = ctx.stats()
        ctx.set_traversal(rr.RR_CUDA_TRAVERSAL_WIDE, ray_order=1)
        per8, total8 = time_steps(trace_step, max(3, args.steps // 3), args.warmup, ws, stream)
        h8 = hits_d.cpu().numpy().view(np.uint32).copy()
        ph = out["plain"]["hits"]
        hit = ph[:, 2] != 0xFFFFFFFF
        d8 = np.where(hit & (h8[:, 3] != ph[:, 3]))[0]

        wide8 = {"kernel": "k_trace_wide", "format": "binary + 8-wide nodes, 8-bit child bounds rounded outward "
                                                     "against a per-node fp32 origin and power-of-two scale",
                 "tree": "fast LBVH (the plain kernel's tree)",
                 "value": R * ws * max(3, args.steps // 3) / (total8 / 1e3) / 1e6, "unit": "Mrays/s",
                 "wide_node_fetches_per_ray": st8["node_fetches"] / R,
                 "triangle_fetches_per_ray": st8["triangle_fetches"] / R,
                 "hit_id_identity": {"rays": int(R),
                                     "hit_flags_identical": bool(np.array_equal(h8[:, 2] != 0xFFFFFFFF, hit)),
                                     **classify_mismatches(v, i, rays, h8, ph, d8),
                                     "note": "the conservative 8-bit boxes reach every triangle the reference's "
                                             "fp32 slab test reaches and each leaf triangle is re-tested on its "
                                             "exact box; a mismatch is an equal-t tie, or a near tie (within 2 "
                                             "ulp) decided by the visit order through the reference's fp32 slab "
                                             "test"},
                 "hits": h8}
        assert ctx.device_errors() == 0, "device error word set during the 8-wide run"

    # ---- any hit (occlusion): the same origins and directions with
    # tmax ~ U[0.01, 0.5]; the chosen kernel autotuned for the any-hit query
    # on the chosen tree, the plain kernel on the fast tree.
    anyhit = None
    if not args.no_anyhit and "plain" in out and not args.only:
        rays_a = rays.copy()
        rays_a[:, 7] = np.random.default_rng(0x52520001).uniform(0.01, 0.5, R).astype(np.float32)
        rays_d.copy_(torch.from_numpy(rays_a))

        def any_step():
            rr.check(L.rrCmdIntersect(ctx.ctx, cur["bvh"], rr.RR_INTERSECT_QUERY_ANY, rb, R, None,
                                      rr.RR_INTERSECT_QUERY_OUTPUT_FULL_HIT, hitb, sb, ext), "rrCmdIntersect")
        tuned_a = ctx.autotune(bvh_c, rays_d, query=rr.RR_INTERSECT_QUERY_ANY, hits=hits_d, scratch=scratch_t)
        res_a = {}
        for name, trav, tree in (("chosen", tuned_a["traversal"], hcb), ("plain", rr.RR_CUDA_TRAVERSAL_BINARY, hb)):
            cur["bvh"] = tree
            if name == "chosen":
                ctx.set_traversal(trav, 0, tuned_a["blocks_per_sm"], ray_order=tuned_a["ray_order"],
                                  short_stack=tuned_a["short_stack"])
            else:
                ctx.set_traversal(trav)
            per_a, total_a = time_steps(any_step, max(3, args.steps // 3), args.warmup, ws, stream)
            res_a[name] = {"value": R * ws * max(3, args.steps // 3) / (total_a / 1e3) / 1e6, "unit": "Mrays/s",
                           "p50_ms": statistics.median(per_a), "p99_ms": float(np.percentile(per_a, 99)),
                           "hits": hits_d.cpu().numpy().view(np.uint32).copy()}
        ha, pa = res_a["chosen"].pop("hits"), res_a["plain"].pop("hits")
        anyhit = {"query": "any hit (occlusion), tmax ~ U[0.01, 0.5], full RRHit output",
                  "chosen": res_a["chosen"], "plain": res_a["plain"],
                  "chosen_kernel": KERNELS.get(tuned_a["traversal"], "?"),
                  "speedup_vs_plain": res_a["chosen"]["value"] / res_a["plain"]["value"],
                  "hit_flags_identical": bool(np.array_equal(ha[:, 2] != 0xFFFFFFFF, pa[:, 2] != 0xFFFFFFFF)),
                  "occluded_fraction": float(np.mean(pa[:, 2] != 0xFFFFFFFF))}
        rays_d.copy_(torch.from_numpy(rays))
        ctx.set_traversal(chosen_trav, args.block, chosen_per_sm, ray_order=chosen_order, short_stack=chosen_stack)
        assert ctx.device_errors() == 0, "device error word set during the any-hit run"

    # ---- the precise triangle test (opt-in RR_CUDA_TRIANGLE_TEST_WATERTIGHT):
    # the same rays and chosen tree, kernel autotuned for the mode; its
    # hits against the plain kernel's, classified, and its fp64 error below.
    precise = None
    if not args.no_precise and "plain" in out and not args.only:
        ctx.set_traversal(0, triangle_test=rr.RR_CUDA_TRIANGLE_TEST_WATERTIGHT)
        tuned_p = ctx.autotune(bvh_c, rays_d, hits=hits_d, scratch=scratch_t)
        cur["bvh"] = hcb
        kp = max(3, args.steps // 3)
        per_p, total_p = time_steps(trace_step, kp, args.warmup, ws, stream)
        hp = hits_d.cpu().numpy().view(np.uint32).copy()
        precise = {"triangle_test": "watertight decision (Woop et al. 2013, exact edge signs), t and uv from "
                                    "exact differences and compensated products, robust box test (Ize 2013); fp32",
                   "kernel": KERNELS.get(tuned_p["traversal"], "?"), "tree": "the chosen path's",
                   "value": R * ws * kp / (total_p / 1e3) / 1e6, "unit": "Mrays/s",
                   "p50_ms": statistics.median(per_p), "p99_ms": float(np.percentile(per_p, 99)),
                   "vs_plain_hits": precise_vs_plain(v, i, rays, hp, out["plain"]["hits"]), "hits": hp}
        ctx.set_traversal(chosen_trav, args.block, chosen_per_sm, ray_order=chosen_order, short_stack=chosen_stack)
        assert ctx.device_errors() == 0, "device error word set during the precise run"

    # ---- end to end through the C-ABI with pinned host buffers
    e2e = None
    if not args.no_e2e and not args.only:
        # The chosen kernel, through the host-buffer entry point: H2D of the
        # rays, the traversal and D2H of the hits, in chunks pipelined over
        # three streams, all inside the timed region.
        ctx.set_traversal(chosen_trav, args.block, chosen_per_sm, ray_order=chosen_order, short_stack=chosen_stack)
        rays_h = torch.from_numpy(rays).pin_memory()
        hits_h = torch.empty((R, 4), dtype=torch.int32).pin_memory()
        rh, hh = C.c_void_p(rays_h.data_ptr()), C.c_void_p(hits_h.data_ptr())

        def e2e_step():
            rr.check(L.rrCudaCmdIntersectHostBuffers(ctx.ctx, hcb, rr.RR_INTERSECT_QUERY_CLOSEST, rh, R,
                                                     rr.RR_INTERSECT_QUERY_OUTPUT_FULL_HIT, hh, rb, hitb, sb,
                                                     args.e2e_chunk, ext), "rrCudaCmdIntersectHostBuffers")
        per_e, total_e = time_steps(e2e_step, args.steps, args.warmup, ws, stream)
        total_e = max_over_ranks(total_e, ws)
        e2e = {"value": R * ws * args.steps / (total_e / 1e3) / 1e6, "unit": "Mrays/s",
               "h2d_bytes_per_step": int(rays_h.numel() * 4), "d2h_bytes_per_step": int(hits_h.numel() * 4),
               "ms_per_step": total_e / args.steps,
               "api": "rrCudaCmdIntersectHostBuffers (pinned host rays/hits; one streamed persistent launch: "
                      f"rays copied in chunks of {args.e2e_chunk or 2 ** 17:,}, hits copied out in parts of 8 "
                      "chunks as the kernel's warps publish them; the hits of rays still in flight at their "
                      "part's publication written to the host by a small kernel after the trace)"}
        e2e_hits = hits_h.numpy().view(np.uint32)
        if "chosen" in out:
            # A miss writes only inst_id (isect.comp:238-244): compare the
            # records of hits and the inst_id of every ray.
            dev = out["chosen"]["hits"]
            hit = dev[:, 2] != 0xFFFFFFFF
            e2e["hits_identical_to_device_run"] = bool(np.array_equal(e2e_hits[:, 2], dev[:, 2]) and
                                                       np.array_equal(e2e_hits[hit], dev[hit]))

    if rank != 0:
        ctx.close()
        return
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    key = "chosen" if "chosen" in out else "plain"
    c = out[key]
    value = R * ws * args.steps / (c["total"] / 1e3) / 1e6
    mean_launch_s = statistics.mean(c["per"]) / 1e3
    achieved = c["alg_bytes"] / mean_launch_s / 1e9
    traffic = None
    kernel = KERNELS.get(c["trav"], "k_trace_binary")
    traffic_key = kernel + ("_q8" if key == "chosen" and c["trav"] == rr.RR_CUDA_TRAVERSAL_BVH4 and
                            cfmt == rr.RR_CUDA_NODE_FORMAT_BVH4Q8 else "")
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists():
        t = json.loads(tf.read_text()).get(traffic_key)
        if t and t.get("dram_bytes_per_ray"):
            traffic = t["dram_bytes_per_ray"] * R
    line = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": c["total"] / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded heightfield + incoherent rays)",
        "config": describe(args, ntri),
        "latency_ms": {"p50": statistics.median(c["per"]), "p99": float(np.percentile(c["per"], 99)),
                       "max": max(c["per"])},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_source": "MEASURED_PEAKS.json hbm_gbs (burst copy)" if peaks else
                     "fallback 6800 GB/s",
                     "alg_bytes_per_ray": c["alg_bytes"] / R,
                     "node_fetches_per_ray": c["stats"]["node_fetches"] / R,
                     "tri_fetches_per_ray": c["stats"]["triangle_fetches"] / R,
                     "bytes_per_node_fetch": {rr.RR_CUDA_TRAVERSAL_WIDE: 80,
                                              rr.RR_CUDA_TRAVERSAL_BVH4: 64 if cfmt == rr.RR_CUDA_NODE_FORMAT_BVH4Q8
                                              else 128}.get(c["trav"], 64) if key == "chosen" else 64,
                     "note": "achieved = algorithmic bytes (ray, hit, node and leaf fetches at their sizes) per "
                             "launch / launch time; the traversal kernels are latency- and issue-bound (DRAM "
                             "traffic well below the algorithmic bytes: nodes hit in L1/L2), so frac is not "
                             "their limit, and 64-byte 8-bit nodes lower it while raising throughput"},
        "clocks": c["clocks"], "gpu_launches": args.steps, "build": build, "traversal": key,
        "chosen_format": {"format": format_tuned or args.chosen_format,
                          "selected_by": "rrCudaAutotuneNodeFormat" if format_tuned else "command line"},
        "chosen_kernel": {"kernel": kernel, "traversal": c["trav"], "ray_order": c["order"],
                          "blocks_per_sm": chosen_per_sm or "occupancy maximum",
                          "short_stack": chosen_stack or 16,
                          "selected_by": "rrCudaAutotuneTraversal" if tuned else "command line"},
    }
    if "plain" in out and "chosen" in out:
        p = out["plain"]
        pv = R * ws * args.steps / (p["total"] / 1e3) / 1e6
        line["plain"] = {"value": pv, "unit": "Mrays/s", "ms_per_step": p["total"] / args.steps,
                         "latency_ms": {"p50": statistics.median(p["per"]), "p99": float(np.percentile(p["per"], 99))},
                         "alg_bytes_per_ray": p["alg_bytes"] / R, "node_fetches_per_ray": p["stats"]["node_fetches"] / R,
                         "achieved_gbs": p["alg_bytes"] / (statistics.mean(p["per"]) / 1e3) / 1e9}
        line["speedup_vs_plain"] = value / pv
        ch, ph = out["chosen"]["hits"], out["plain"]["hits"]
        flags_equal = bool(np.array_equal(ch[:, 2] != 0xFFFFFFFF, ph[:, 2] != 0xFFFFFFFF))
        hit = ph[:, 2] != 0xFFFFFFFF
        diff = np.where(hit & (ch[:, 3] != ph[:, 3]))[0]
        line["hit_id_identity"] = {"rays": int(R), "hit_flags_identical": flags_equal,
                                   "prim_id_identical_fraction": float(1.0 - diff.size / max(1, int(hit.sum()))),
                                   **classify_mismatches(v, i, rays, ch, ph, diff),
                                   "note": "chosen traces the quality (restructured) tree, plain the fast LBVH; "
                                           "a mismatch is two triangles hit at the same t, or within 2 ulp where "
                                           "the reference's fp32 slab test culls a box whose entry rounds past the "
                                           "closest t found so far (visit-order dependent)"}
    if e2e:
        line["e2e"] = e2e
    if not args.no_cpu:
        cb, nodes = cpu_baseline(v, i, rays, args.cpu_seconds)
        line["cpu_baseline"] = cb
        line["fp64_t_error"] = precision_report(v, i, rays, c["hits"], nodes)
    if anyhit:
        line["any_hit"] = anyhit
    if precise:
        hp = precise.pop("hits")
        if not args.no_cpu:
            precise["fp64_t_error"] = precision_report(v, i, rays, hp, nodes, precise=True)
        line["precise"] = precise
    if wide8:
        h8 = wide8.pop("hits")
        if not args.no_cpu:
            wide8["fp64_t_error"] = precision_report(v, i, rays, h8, nodes)
        line["precision_wide8"] = wide8
    ctx.close()
    if ws == 1 and not args.no_extras and not args.only:
        # The batching and serving configurations, summarised in the same line.
        del rays_d, hits_d, scratch_t, bvh, bvh_c, v_d, i_d
        torch.cuda.empty_cache()
        b = batch_summary(args, separate=False)
        line["blas2048"] = {"workload": b["workload"], "fused_build_ms": b["build"]["fused_ms"],
                            "fused_build_mtris_s": b["build"]["fused_mtris_s"], "tlas_ms": b["build"]["tlas_ms"],
                            "chosen": b["trace"]["chosen"], "plain": b["trace"]["plain"],
                            "chosen_kernel": b["chosen_traversal"]["kernel"],
                            "speedup_vs_plain": b["speedup_vs_plain"], "hit_flags_identical": b["hit_flags_identical"],
                            "hit_mismatches_vs_plain": b["hit_mismatches_vs_plain"], "device_errors": b["device_errors"]}
        torch.cuda.empty_cache()
        sv = serving_summary(args)
        line["serving"] = {"workload": sv["workload"], "requests_per_point": args.requests,
                           "saturation_mrays_s": sv["saturation"]["throughput_mrays_s"],
                           "load_sweep": [{"offered_load": r["offered_load"], "throughput_mrays_s":
                                           r["throughput_mrays_s"], "p50_ms": r["latency_ms"]["p50"],
                                           "p99_ms": r["latency_ms"]["p99"], "makespan_s": r["makespan_s"],
                                           "launches": r["launches"]} for r in sv["load_sweep"]],
                           "hits_checked": sv["hits_checked"], "device_errors": sv["device_errors"]}
    print(json.dumps(line), flush=True)


def run_batch(args):
    """--workload blas2048: the summary below as its own JSON line."""
    import torch
    ws, rank, local = dist()
    torch.cuda.set_device(local)
    print(json.dumps(batch_summary(args, separate=not args.no_separate)), flush=True)


def batch_summary(args, separate=True):
    """2,048 soups with log-uniform 64..262,144 triangles built in one fused
    build (rrCudaCmdBuildGeometries, replayed as a CUDA graph) against one
    rrCmdBuildGeometry per BLAS (`separate`); then the instance tree and
    incoherent two-level closest-hit traversal, chosen (autotuned) vs plain,
    with the hits of the two classified."""
    import torch
    from radeonrays_sdk_gb300 import rr, scenes
    blas, M, rays = scenes.config2(n_blas=args.blas, nrays=args.batch_rays)
    counts = np.array([i.shape[0] for _, i in blas])
    ntri = int(counts.sum())
    v_all = torch.from_numpy(np.concatenate([v for v, _ in blas])).cuda()
    i_all = torch.from_numpy(np.concatenate([i for _, i in blas]).view(np.int32)).cuda()
    meshes, vo, io = [], 0, 0
    for v, i in blas:
        meshes.append((v_all[vo:vo + v.shape[0]], i_all[io:io + i.shape[0]]))
        vo, io = vo + v.shape[0], io + i.shape[0]
    ctx = rr.Context()
    fmt = rr.RR_CUDA_NODE_FORMAT_BVH4Q8  # the library default

    def timed(fn, k, w):
        for _ in range(w):
            fn()
        t = []
        for _ in range(k):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            t.append(time.perf_counter() - t0)
        return t

    # Fused: recorded once, every submission replays the captured graph.
    cs = ctx.command_stream()
    fused = ctx.build_geometries(meshes, node_format=fmt, stream=cs, api="batch")
    keep = ctx._keep
    f_t = timed(lambda: ctx.submit(cs), max(3, args.steps // 10), 2)
    # One rrCmdBuildGeometry per BLAS, each enqueued at once on a CUDA stream.
    s_t = [float("nan")] if not separate else \
        timed(lambda: ctx.build_geometries(meshes, node_format=fmt, api="separate"), 2, 1)
    errors = ctx.device_errors()
    scene = ctx.build_scene(fused, M)
    # TLAS: rrCmdBuildScene recorded on a CUDA stream into preallocated
    # buffers, timed with CUDA events on that stream (the instance records
    # are host memory, as in the reference API: their upload is inside).
    sbi, inst_keep = ctx.scene_build_input(fused, M)
    sreq = rr.RRMemoryRequirements()
    rr.check(ctx.L.rrGetSceneBuildMemoryRequirements(ctx.ctx, C.byref(sbi), None, C.byref(sreq)),
             "rrGetSceneBuildMemoryRequirements")
    tl_scratch = torch.empty(max(sreq.temporary_build_buffer_size, 256), dtype=torch.uint8, device="cuda")
    tl_result = torch.empty(sreq.result_buffer_size, dtype=torch.uint8, device="cuda")
    tl_stream = torch.cuda.current_stream()
    tl_ext = ctx.external_stream(tl_stream)
    tl_args = (ctx.ctx, C.byref(sbi), None, ctx.ptr(tl_scratch), ctx.ptr(tl_result), tl_ext)

    def tlas_step():
        rr.check(ctx.L.rrCmdBuildScene(*tl_args), "rrCmdBuildScene")
    tl_per, _ = time_steps(tlas_step, 5, 2, 1, tl_stream)
    tl_t = [x / 1e3 for x in tl_per]

    R = rays.shape[0]
    stream = torch.cuda.current_stream()
    ext = ctx.external_stream(stream)
    rays_d = torch.from_numpy(rays).cuda()
    hits_d = torch.empty((R, 4), dtype=torch.int32, device="cuda")
    scratch_t = torch.empty(ctx.trace_scratch_bytes(R), dtype=torch.uint8, device="cuda")
    hb, rb, hitb, sb = ctx.ptr(scene), ctx.ptr(rays_d), ctx.ptr(hits_d), ctx.ptr(scratch_t)

    def trace_step():
        rr.check(ctx.L.rrCmdIntersect(ctx.ctx, hb, rr.RR_INTERSECT_QUERY_CLOSEST, rb, R, None,
                                      rr.RR_INTERSECT_QUERY_OUTPUT_FULL_HIT, hitb, sb, ext), "rrCmdIntersect")
    out = {}
    # Chosen: the autotuner's pick among the two-level kernels the scene allows
    # (plain, persistent binary, 4-wide BLASes).
    tuned = ctx.autotune(scene, rays_d, hits=hits_d, scratch=scratch_t)
    for name, trav in (("chosen", tuned["traversal"]), ("plain", rr.RR_CUDA_TRAVERSAL_BINARY)):
        if name == "chosen":
            ctx.set_traversal(trav, 0, tuned["blocks_per_sm"], ray_order=tuned["ray_order"],
                              short_stack=tuned["short_stack"])
        else:
            ctx.set_traversal(trav)
        per, total = time_steps(trace_step, max(3, args.steps // 3), max(3, args.warmup), 1, stream)
        out[name] = {"ms": statistics.median(per), "mrays_s": R / statistics.median(per) / 1e3,
                     "p99_ms": float(np.percentile(per, 99)), "hits": hits_d.cpu().numpy().view(np.uint32).copy()}
    ctx.set_traversal(0)
    ch, ph = out["chosen"].pop("hits"), out["plain"].pop("hits")
    flags_equal = bool(np.array_equal(ch[:, 2] != 0xFFFFFFFF, ph[:, 2] != 0xFFFFFFFF))
    mism = int(np.sum((ch[:, 2] != ph[:, 2]) | (ch[:, 3] != ph[:, 3])))
    errors |= ctx.device_errors()
    line = {"metric": "fused 2,048-BLAS build Mtris/s and two-level incoherent closest-hit Mrays/s",
            "workload": f"{len(blas)} soups, log-uniform 64..262,144 triangles ({ntri:,} total), random "
                        f"rotation / scale U[0.5,2] / translation U[0,100]^3 instances, {R:,} incoherent rays "
                        "in the scene box, closest hit, full RRHit output",
            "build": {"fused_ms": 1e3 * statistics.median(f_t), "fused_mtris_s": ntri / statistics.median(f_t) / 1e6,
                      "separate_ms": 1e3 * statistics.median(s_t),
                      "separate_mtris_s": ntri / statistics.median(s_t) / 1e6,
                      "fused_speedup": statistics.median(s_t) / statistics.median(f_t),
                      "tlas_ms": 1e3 * statistics.median(tl_t),
                      "tlas_timing": "CUDA events around rrCmdBuildScene on its stream (instance upload included)",
                      "format": "binary + bvh4q8 (the default)",
                      "fused_timing": "host clock around rrSumbitCommandStream + rrWaitEvent (CUDA graph replay)"},
            "trace": out, "chosen_traversal": {"traversal": tuned["traversal"],
                                               "kernel": {1: "k_trace_scene_binary", 3: "k_trace_scene_persistent",
                                                          4: "k_trace_scene_bvh4"}.get(tuned["traversal"], "?"),
                                               "blocks_per_sm": tuned["blocks_per_sm"] or "occupancy maximum",
                                               "selected_by": "rrCudaAutotuneTraversal"},
            "speedup_vs_plain": out["plain"]["ms"] / out["chosen"]["ms"],
            "hit_flags_identical": flags_equal, "hit_mismatches_vs_plain": mism, "device_errors": int(errors)}
    del keep
    ctx.release_stream(cs)
    ctx.close()
    return line


def run_serving(args):
    """--workload serving: the summary below as its own JSON line."""
    import torch
    ws, rank, local = dist()
    torch.cuda.set_device(local)
    print(json.dumps(serving_summary(args)), flush=True)


def serving_summary(args):
    """64 resident scenes (log-uniform 10^4..2x10^6 triangles, soup or
    heightfield), Poisson arrivals of log-uniform 1,024..1,048,576-ray
    requests (70% closest, 30% any-hit), continuous batching into
    rrCudaCmdIntersectBatchHost launches.  Saturation throughput first (all
    requests at t = 0), then offered loads of 50/80/95% of it: throughput and
    p50/p99 request latency (arrival to hits in host memory)."""
    import torch
    from radeonrays_sdk_gb300 import rr, serving
    meshes = serving.config4(args.scenes)
    ntri = sum(i.shape[0] for _, i in meshes)
    ctx = rr.Context()
    pool = serving.ScenePool(ctx, int(args.hbm_budget_gb * (1 << 30)),
                             node_format={"binary": rr.RR_CUDA_NODE_FORMAT_BINARY, "bvh4": rr.RR_CUDA_NODE_FORMAT_BVH4,
                                          "bvh4q8": rr.RR_CUDA_NODE_FORMAT_BVH4Q8}[args.scene_format])
    for k, (v, i) in enumerate(meshes):
        pool.register(k, v, i)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(len(meshes)):
        pool.acquire(k)
        pool.release(k)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    server = serving.Server(ctx, pool, slot_rays=args.slot_rays, slots=args.slots, max_requests=256)
    # Checked first: requests with their own buffers, each against the same
    # request traced alone by rrCmdIntersect with the kernel the launches run.
    check = serving.make_requests(meshes, 48, rate_per_s=1e9, hi_rays=1 << 16, seed=39)
    server.run(check)
    alone_trav = rr.RR_CUDA_TRAVERSAL_BINARY if args.scene_format == "binary" else rr.RR_CUDA_TRAVERSAL_BVH4
    ctx.set_traversal(alone_trav)
    same = 0
    for r in check:
        alone = ctx.intersect(pool.build(r.scene), torch.from_numpy(r.rays).cuda(), query=r.query,
                              output=r.output).cpu().numpy().view(np.uint32)
        same += int(np.array_equal(r.hits, alone))
    ctx.set_traversal(0)
    # Timed runs: rays are slices of pinned per-scene pools, hits go to a
    # pinned ring, so that thousands of requests need no per-request buffers.
    pools = serving.RayPools(meshes)
    warm = serving.make_requests(meshes, 64, rate_per_s=1e9, seed=40, pools=pools)
    server.run(warm)
    sat_reqs = serving.make_requests(meshes, args.requests, rate_per_s=1e9, seed=41, pools=pools)
    sat = server.run(sat_reqs)
    mean_rays = sat["rays"] / sat["requests"]
    cap = sat["throughput_mrays_s"] * 1e6 / mean_rays  # requests per second at saturation
    sweep = []
    for k, frac in enumerate((0.5, 0.8, 0.95)):
        reqs = serving.make_requests(meshes, args.requests, rate_per_s=frac * cap, seed=42 + k, pools=pools)
        res = server.run(reqs)
        res["offered_load"] = frac
        res["rate_req_s"] = frac * cap
        sweep.append(res)
    line = {"metric": "serving: throughput Mrays/s and p50/p99 request latency (continuous batching)",
            "workload": f"{len(meshes)} resident scenes ({ntri:,} triangles), requests of 1,024..1,048,576 rays "
                        "(log-uniform), 70% closest / 30% any-hit (tmax U[0.01,0.5]), incoherent rays in each "
                        "scene's box, Poisson arrivals",
            "slots": args.slots, "slot_rays": args.slot_rays, "hbm_budget_gb": args.hbm_budget_gb,
            "scene_build_s": build_s, "resident_bytes": pool.bytes, "saturation": sat, "load_sweep": sweep,
            "latency_definition": "arrival to hits copied to the request's pinned host buffer",
            "scene_format": "binary nodes only (launches run the reference-order multi-request kernel)"
                            if args.scene_format == "binary" else
                            "binary + 4-wide nodes with " + ("8-bit" if args.scene_format == "bvh4q8" else "fp32")
                            + " bounds (launches run the 4-wide multi-request kernel)",
            "hits_checked": {"requests": len(check), "identical_to_alone": same,
                             "against": "each request traced alone by rrCmdIntersect with "
                                        + ("RR_CUDA_TRAVERSAL_BINARY" if args.scene_format == "binary" else
                                           "RR_CUDA_TRAVERSAL_BVH4")},
            "device_errors": ctx.device_errors()}
    ctx.close()
    return line


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "blas2048":
        run_batch(args)
    elif args.workload == "serving":
        run_serving(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
