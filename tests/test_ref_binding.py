"""The backend subclass of the reference's own Lattice<Model>
(include/lgca/ref_binding.h), compiled against the reference's src/lattice.h
and linked with its src/lattice.cpp from where they lie (only on a machine
with the reference sources; the GPU machine has none).  The binary runs an app's
set-up through the binding on the host -- the reference's constructor,
geometry setter, init_random and particle count -- and its dimensions and
forcing amounts equal this repository's restatement of them."""
import json
import os
import subprocess

import pytest

from conftest import ROOT
from lgca_gb300 import params as P


@pytest.fixture(scope="module")
def binary(tmp_path_factory, ref):
    import lgca_gb300
    lgca_gb300.build()
    src = os.path.join(ref.REFERENCE_DIR, "src")
    out = str(tmp_path_factory.mktemp("ref_binding") / "ref_binding_check")
    pkg = os.path.join(ROOT, "lgca_gb300")
    cmd = ["g++", "-O1", "-std=c++14", "-fopenmp", "-w",
           "-I", os.path.join(ROOT, "oracle", "tbb_shim"), "-I", src,
           "-I", os.path.join(ref.REFERENCE_DIR, "lib"), "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "ref_binding_check.cpp"), os.path.join(src, "lattice.cpp"),
           "-L", pkg, "-llgca_gpu", f"-Wl,-rpath,{pkg}", "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return out


@pytest.mark.parametrize("case,model", [("pipe", 3), ("karman", 1), ("box", 0), ("periodic", 2)])
def test_binding_runs_reference_setup_on_host(binary, case, model):
    r = subprocess.run([binary, "host", case, str(model)], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    got = json.loads(r.stdout.strip().splitlines()[-1])
    p = P.lattice_parameters(model, case, 80.0, 0.3, 20 if case == "karman" else 10)
    assert got["dims"] == [p["dim_x"], p["dim_y"]]
    assert got["coarse"] == [p["coarse_dim_x"], p["coarse_dim_y"]]
    assert got["initial_forcing"] == p["initial_forcing"]
    assert got["equilibrium_forcing"] == p["equilibrium_forcing"]
    # the reference's init_random occupies each channel of a fluid cell with
    # probability 1/NUM_DIR: about one particle per cell
    cells = p["dim_x"] * p["dim_y"]
    assert 0.8 * cells < got["particles"] < 1.1 * cells
