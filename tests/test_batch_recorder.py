"""The host side of the batched launches (gevolution-1.2_gb300/csrc/gev_batch.cuh):
the recorder's argument packs, their alignment and conversions, and the launcher
identity that cohorts are formed on.  tests/cpp/batch_recorder_host.cu is built with
nvcc for sm_103a and run on the host; it makes no device call, so it needs no GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_recorder_packs_and_launchers(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "batch_recorder_host")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O1",
                    "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "batch_recorder_host.cu"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr
