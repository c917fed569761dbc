"""The library used from compiled code, the way a reference client uses it:
tests/c_client/abi_check.c (C99) and tests/c_client/client.cpp (C++17) are
compiled against include/*.h and linked against librr.so.  The C program runs
on the CPU (argument checks only); the C++ client builds a mesh, traces it
through a recorded command stream and through an external CUDA stream with
the autotuner's pick, and checks every hit against the analytic answer."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

from conftest import ROOT

SRC = ROOT / "tests" / "c_client"
CUDA = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def _compile(tmp_path, compiler, src, out, extra):
    cc = shutil.which(compiler)
    if cc is None:
        pytest.skip(f"{compiler} not found")
    libdir = ROOT / "radeonrays_sdk_gb300"
    cmd = [cc, str(SRC / src), f"-I{ROOT / 'include'}", f"-I{CUDA / 'include'}", f"-L{libdir}", "-lrr",
           f"-Wl,-rpath,{libdir}", "-o", str(tmp_path / out), *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return tmp_path / out


def test_c_program_compiles_links_and_checks_arguments(rrlib, tmp_path):
    exe = _compile(tmp_path, "gcc", "abi_check.c", "abi_check", ["-std=c99", "-Wall", "-Werror"])
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr


def _client(rrlib, tmp_path):
    if not (CUDA / "include" / "cuda_runtime.h").exists():
        pytest.skip("CUDA headers not found")
    return _compile(tmp_path, "g++", "client.cpp", "client",
                    ["-std=c++17", "-Wall", "-Werror", f"-L{CUDA / 'lib64'}", "-lcudart"])


def test_cpp_client_compiles_and_links(rrlib, tmp_path):
    assert _client(rrlib, tmp_path).exists()


@pytest.mark.gpu
def test_cpp_client_runs(rrlib, tmp_path):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    exe = _client(rrlib, tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().splitlines()[-1].startswith("ok:"), r.stdout
