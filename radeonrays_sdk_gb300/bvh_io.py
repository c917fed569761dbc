"""On-disk BVH files: store and load geometry result buffers, and export a
tree for the reference's bvh_analyzer tool.

A geometry result buffer is position-independent (node indices, not
pointers), so its bytes are the file.  The file is a 64-byte header followed
by the buffer:

    offset  size  field
    0       8     magic b"RRBVHGEO"
    8       4     format version (1)
    12      4     triangle count
    16      4     node format (RRCudaNodeFormat)
    20      4     Morton key width (30 or 63)
    24      8     buffer bytes
    32      32    reserved (zero)

Loading copies the bytes into a device buffer and registers it with the
context (rrCudaRegisterGeometry), which checks the buffer's own trailer.  A
scene buffer holds the addresses of its BLAS buffers and is not stored: load
the BLASes and build the scene again (rrCmdBuildScene), which takes
milliseconds.

bvh_analyzer (the reference's CPU analysis tool, bvh_analyzer/config.h) reads
a raw array of 64-byte nodes in the same layout as the binary node array here,
a raw ray array and a 7-line text config; export_bvh_analyzer writes the
three files.
"""
from __future__ import annotations

import ctypes as C
import struct
from pathlib import Path

import numpy as np

from . import rr

MAGIC = b"RRBVHGEO"
VERSION = 1
HEADER = struct.Struct("<8sIIIIQ32x")
assert HEADER.size == 64


def _trailer(raw: np.ndarray, n: int) -> np.ndarray:
    off = (((2 * n - 1) * 64 if n else 0) + 255) // 256 * 256
    if raw.size < off + 256:
        raise ValueError(f"buffer of {raw.size} bytes is too small for a build of {n} triangles")
    return rr.read_trailer(raw, n)


def save_geometry(path, buffer, triangle_count: int) -> int:
    """Write a geometry result buffer (device tensor or host uint8 array) to
    `path`; returns the bytes written."""
    raw = buffer.cpu().numpy() if hasattr(buffer, "cpu") else np.asarray(buffer, dtype=np.uint8)
    raw = np.ascontiguousarray(raw.view(np.uint8).reshape(-1))
    tr = _trailer(raw, triangle_count)
    if int(tr["magic"]) != 0x52524742 or int(tr["leaf_count"]) != triangle_count:
        raise ValueError("buffer is not a geometry build of this triangle count")
    head = HEADER.pack(MAGIC, VERSION, triangle_count, int(tr["node_format"]), int(tr["morton_bits"]), raw.size)
    with open(path, "wb") as f:
        f.write(head)
        f.write(raw.tobytes())
    return HEADER.size + raw.size


def read_header(path) -> dict:
    with open(path, "rb") as f:
        magic, ver, n, fmt, bits, size = HEADER.unpack(f.read(HEADER.size))
    if magic != MAGIC or ver != VERSION:
        raise ValueError(f"{path}: not a BVH file of version {VERSION}")
    return {"triangle_count": n, "node_format": fmt, "morton_bits": bits, "bytes": size}


def load_geometry(ctx: rr.Context, path):
    """Read a file written by save_geometry into a new device buffer and
    register it with `ctx`.  Returns (buffer tensor, triangle count)."""
    import torch
    h = read_header(path)
    with open(path, "rb") as f:
        f.seek(HEADER.size)
        data = np.frombuffer(f.read(h["bytes"]), dtype=np.uint8)
    if data.size != h["bytes"]:
        raise ValueError(f"{path}: truncated ({data.size} of {h['bytes']} bytes)")
    buf = torch.from_numpy(data.copy()).cuda()
    torch.cuda.synchronize()
    rr.check(ctx.L.rrCudaRegisterGeometry(ctx.ctx, ctx.ptr(buf), h["triangle_count"]), "rrCudaRegisterGeometry")
    return buf, h["triangle_count"]


def export_bvh_analyzer(directory, name: str, buffer, triangle_count: int, rays: np.ndarray, width: int = 0):
    """Write `name.bvh` (the binary nodes), `name.rays` and `name.cfg` for
    bvh_analyzer.  Its config holds the internal-node and triangle counts and
    the rays as width x height (height = ray count / width)."""
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    raw = buffer.cpu().numpy() if hasattr(buffer, "cpu") else np.asarray(buffer, dtype=np.uint8)
    n = triangle_count
    nodes = raw.view(np.uint8).reshape(-1)[: max(2 * n - 1, 0) * 64]
    rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
    width = width or rays.shape[0]
    if rays.shape[0] % width:
        raise ValueError("ray count must be a multiple of width")
    (d / f"{name}.bvh").write_bytes(nodes.tobytes())
    (d / f"{name}.rays").write_bytes(rays.tobytes())
    cfg = [str(d / f"{name}.bvh"), "vkbvh2", str(max(n - 1, 0)), str(n), str(d / f"{name}.rays"), str(width),
           str(rays.shape[0] // width)]
    (d / f"{name}.cfg").write_text("\n".join(cfg) + "\n")
    return d / f"{name}.cfg"


def save_pool(pool, directory) -> list:
    """Checkpoint every resident scene of a serving ScenePool as one file per
    scene; returns the paths."""
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    out = []
    for sid, buf in pool.resident.items():
        n = pool.meshes[sid][1].shape[0]
        p = d / f"scene_{sid}.rrbvh"
        save_geometry(p, buf, n)
        out.append(p)
    return out


def load_pool(pool, directory) -> int:
    """Resume: load every scene file of `directory` that the pool has
    registered as resident (no build).  Returns the number loaded."""
    loaded = 0
    for p in sorted(Path(directory).glob("scene_*.rrbvh")):
        sid = int(p.stem.split("_")[1])
        if sid not in pool.meshes or sid in pool.resident:
            continue
        buf, n = load_geometry(pool.ctx, p)
        if n != pool.meshes[sid][1].shape[0]:
            raise ValueError(f"{p}: triangle count does not match scene {sid}")
        pool.resident[sid] = buf
        pool.bytes += buf.numel()
        loaded += 1
    return loaded
