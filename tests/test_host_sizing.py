"""Host-side sizing rules of the tree and batched-system buffers
(nbgb_internal.cuh, sysmem.cuh), compiled with nvcc and run on the CPU: no
device code runs."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_sizing_rules(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("no nvcc")
    exe = tmp_path / "sizing"
    src = os.path.join(ROOT, "tests", "cpp", "sizing_check.cu")
    inc = os.path.join(ROOT, "nbodysimulation_gb300", "csrc")
    subprocess.run([nvcc, "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a", "-I", inc, src, "-o",
                    str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
