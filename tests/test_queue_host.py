"""The batched kernels' work queue, built on the host (work_queue.cuh):
every item once, round-major, each unit after the whole previous round of
its instance (so a unit waits only for items earlier in the queue and the
persistent kernels cannot deadlock), active instances a prefix, and
over-long queues refused.  Compiles tests/queue_host_check.cu with nvcc and
runs it on the host; no GPU needed."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_work_queue_order_on_the_host(tmp_path):
    nvcc = os.environ.get("NVCC", "nvcc")
    if shutil.which(nvcc) is None:
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "queue_host_check")
    cmd = [nvcc, "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a",
           "-I", os.path.join(ROOT, "b2r_gb300", "csrc"), "-I", os.path.join(ROOT, "include"),
           os.path.join(HERE, "queue_host_check.cu"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
