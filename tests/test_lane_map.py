"""CPU check of the step kernels' lane mapping (internal.cuh: flat_tasks,
flat_magic, flat_site): full coverage of every (row, lane item), one parity
per warp, the divide-free row computation, and the source lanes of the
neighbour and seam shuffles.  tests/lane_map_check.cu is built with nvcc as
host code and run here; no GPU is needed."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT


def test_lane_mapping_covers_rows_and_shuffle_sources(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = tmp_path / "lane_map_check"
    subprocess.run([nvcc, "-O2", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                    os.path.join(ROOT, "tests", "lane_map_check.cu"), "-o", str(exe)],
                   check=True, capture_output=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout[-2000:]
