"""On-disk BVH files on CPU: header round trip and rejection, and interop with
the reference's own bvh_analyzer tool (run where it was built from the
reference checkout; skipped elsewhere)."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from radeonrays_sdk_gb300 import bvh_io, rr, scenes

ROOT = Path(__file__).resolve().parents[1]
ANALYZER = ROOT / "oracle" / "_ref" / "bvh_analyzer"


def _host_buffer(orc, n, fmt=0):
    """A binary-format result buffer assembled on the host: oracle nodes, then
    the 256-byte trailer the GPU build writes."""
    v, i = scenes.soup(n, scenes.rng(91, n))
    nodes, _, _ = orc.build_mesh(v, i)
    nb = nodes.view(np.uint8).reshape(-1)
    toff = (nb.size + 255) // 256 * 256
    buf = np.zeros(toff + 256, np.uint8)
    buf[: nb.size] = nb
    tr = np.zeros(1, rr.TRAILER_DTYPE)
    tr["magic"], tr["version"], tr["kind"], tr["node_format"] = 0x52524742, 2, 1, fmt
    tr["leaf_count"], tr["node_count"], tr["morton_bits"] = n, 2 * n - 1, 30
    buf[toff:] = tr.view(np.uint8)
    return buf, nodes


def test_save_and_header_round_trip(orc, tmp_path):
    buf, _ = _host_buffer(orc, 777)
    p = tmp_path / "a.rrbvh"
    assert bvh_io.save_geometry(p, buf, 777) == 64 + buf.size
    h = bvh_io.read_header(p)
    assert h == {"triangle_count": 777, "node_format": 0, "morton_bits": 30, "bytes": buf.size}
    assert np.array_equal(np.frombuffer(p.read_bytes()[64:], np.uint8), buf)


def test_save_rejects_mismatch_and_bad_files(orc, tmp_path):
    buf, _ = _host_buffer(orc, 100)
    with pytest.raises(ValueError):
        bvh_io.save_geometry(tmp_path / "x", buf, 101)
    (tmp_path / "junk").write_bytes(b"not a bvh file at all, clearly" * 4)
    with pytest.raises(ValueError):
        bvh_io.read_header(tmp_path / "junk")


@pytest.mark.skipif(not ANALYZER.exists(), reason="bvh_analyzer is built only where the reference checkout exists")
def test_reference_bvh_analyzer_accepts_exported_tree(orc, tmp_path):
    buf, nodes = _host_buffer(orc, 5000)
    rays = scenes.pinhole_rays(64, 64)
    cfg = bvh_io.export_bvh_analyzer(tmp_path, "soup", buf, 5000, rays, width=64)
    # The tool writes its images into its working directory: keep them in tmp_path.
    r = subprocess.run([str(ANALYZER), str(cfg)], capture_output=True, text=True, timeout=300, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    assert "is_valid: 1" in r.stdout
    assert "Triangles: 5000" in r.stdout and "Internal nodes: 4999" in r.stdout
