"""CPU check of the GPU collision circuit: collide.cuh is plain C++ as well, so
it is compiled here with g++ and its table compared with the reference's
collision tables (all 2^D states x 2 chiralities, every model)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_npz


def test_bit_sliced_collision_equals_reference_tables(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "collide_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-x", "c++",
                    os.path.join(ROOT, "tests", "collide_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    rows = np.array([list(map(int, l.split())) for l in out.strip().splitlines()])
    tables = load_npz("collide_tables.npz")
    for m in range(4):
        sel = rows[rows[:, 0] == m]
        got = np.zeros_like(tables[f"m{m}"])
        got[sel[:, 1], sel[:, 2]] = sel[:, 3]
        assert np.array_equal(got, tables[f"m{m}"]), m
