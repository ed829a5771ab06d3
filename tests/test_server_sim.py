"""The query server's scheduling on the CPU: csrc/server.cpp compiled with g++
against a host-only stand-in engine (tests/server_sim/), driven through
streams of BFS/SSSP/CC/PageRank queries on three graphs under an ample and a
tight budget, bursts and spaced arrivals, cancellations, an injected batch
launch failure and FIFO mode. Every query completes with its values (or fails
with the injected failure's message) within a deadline; the stand-in checks
that device bytes never exceed the budget and that the batch worker and the
whole-run worker never have device work in flight, or allocate and free
device memory, at the same time."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SIM = os.path.join(ROOT, "tests", "server_sim")


def _cuda_include():
    cands = [os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"]
    nvcc = shutil.which("nvcc")
    if nvcc:
        cands.append(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))))
    for c in cands:
        if c and os.path.exists(os.path.join(c, "include", "cuda_runtime.h")):
            return os.path.join(c, "include")
    return None


def test_server_scheduling_on_the_stand_in_engine(tmp_path):
    gxx = shutil.which("g++")
    inc = _cuda_include()
    if not gxx or not inc:
        pytest.skip("needs g++ and the CUDA headers")
    exe = str(tmp_path / "server_sim")
    cmd = [gxx, "-std=c++17", "-O1", "-pthread", "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "ascetic_gb300", "csrc"), "-I" + SIM, "-I" + inc,
           os.path.join(SIM, "mock_engine.cpp"), os.path.join(SIM, "sim_main.cpp"),
           os.path.join(ROOT, "ascetic_gb300", "csrc", "server.cpp"), "-o", exe]
    build = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert build.returncode == 0, build.stderr[-3000:]
    run = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert run.returncode == 0, (run.stdout[-3000:], run.stderr[-3000:])
    assert "all scenarios passed" in run.stdout
