"""Host-side launch logic, compiled with nvcc and run on the host (no GPU):
the batched kernels' work queue (work_queue.cuh) -- every item once,
round-major, each unit after the whole previous round of its instance (so a
unit waits only for items earlier in the queue and the persistent kernels
cannot deadlock), active instances a prefix, over-long queues refused -- and
the Game-of-Life pass's z-chunk model (gol.h)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.mark.parametrize("name", ["queue_host_check", "gol_chunks_check"])
def test_host_launch_logic(tmp_path, name):
    nvcc = os.environ.get("NVCC", "nvcc")
    if shutil.which(nvcc) is None:
        pytest.skip("nvcc not found")
    exe = str(tmp_path / name)
    cmd = [nvcc, "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a",
           "-I", os.path.join(ROOT, "b2r_gb300", "csrc"), "-I", os.path.join(ROOT, "include"),
           os.path.join(HERE, name + ".cu"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
