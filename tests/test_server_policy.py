"""The job server's host-side policy (csrc/server_policy.hpp), built with
g++ and run on the CPU: admission order and limits, rounds, snapshots,
percentiles."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_server_policy(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = tmp_path / "policy"
    src = os.path.join(ROOT, "tests", "cpp", "server_policy_check.cpp")
    inc = os.path.join(ROOT, "nbodysimulation_gb300", "csrc")
    subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-I", inc, src, "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
