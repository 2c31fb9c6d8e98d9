"""Headless application loops (lgca_gb300/apps/lgca_headless.cpp over the C++
GB_Lattice class, include/lgca/gb_lattice.h) and the headless writers
(include/lgca/io.h).  CPU tests cover the writers and the argument handling;
GPU tests run the reference apps' loops and compare their output files with
the oracle."""
import json
import os
import struct
import subprocess
import zlib

import numpy as np
import pytest

from conftest import ROOT
from lgca_gb300 import geometry as G
from lgca_gb300 import params as P


def read_vti(path):
    """{array name: float32 array} of a raw-appended .vti written by io.h."""
    raw = open(path, "rb").read()
    head, _, rest = raw.partition(b'<AppendedData encoding="raw">')
    blob = rest[rest.index(b"_") + 1:]
    out = {}
    import re
    for m in re.finditer(rb'Name="([^"]+)" NumberOfComponents="(\d+)" format="appended" offset="(\d+)"',
                         head):
        name, comps, off = m.group(1).decode(), int(m.group(2)), int(m.group(3))
        (n,) = struct.unpack_from("<Q", blob, off)
        out[name] = np.frombuffer(blob[off + 8: off + 8 + n], np.float32).reshape(-1, comps)
    return out, head.decode()


def read_png(path):
    b = open(path, "rb").read()
    assert b[:8] == bytes([137, 80, 78, 71, 13, 10, 26, 10])
    pos, chunks = 8, {}
    while pos < len(b):
        (n,) = struct.unpack(">I", b[pos:pos + 4])
        typ = b[pos + 4:pos + 8]
        data = b[pos + 8:pos + 8 + n]
        (crc,) = struct.unpack(">I", b[pos + 8 + n:pos + 12 + n])
        assert zlib.crc32(typ + data) & 0xffffffff == crc, typ
        chunks.setdefault(typ, b"")
        chunks[typ] += data
        pos += 12 + n
    w, h, depth, ctype = struct.unpack(">IIBB", chunks[b"IHDR"][:10])
    raw = zlib.decompress(chunks[b"IDAT"])
    assert depth == 8 and ctype == 2 and len(raw) == h * (3 * w + 1)
    return w, h, raw


def test_writers_vti_and_png(tmp_path):
    exe = tmp_path / "io_check"
    subprocess.run(["g++", "-O1", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "io_check.cpp"), "-o", str(exe)], check=True)
    subprocess.run([str(exe), str(tmp_path) + "/"], check=True)
    cell, head = read_vti(tmp_path / "cell_res_7.vti")
    assert 'WholeExtent="0 5 0 3 0 0"' in head and "<CellData" in head
    assert np.array_equal(cell["Cell density"][:, 0], np.arange(15, dtype=np.float32))
    assert np.array_equal(cell["Cell momentum"].ravel(), 0.5 * np.arange(30, dtype=np.float32) - 3)
    mean, head = read_vti(tmp_path / "mean_res_7.vti")
    assert 'WholeExtent="0 1 0 0 0 0"' in head and "<PointData" in head
    assert np.array_equal(mean["Mean density"][:, 0], np.array([1.25, 2.5], np.float32))
    w, h, raw = read_png(tmp_path / "field.png")
    assert (w, h) == (350, 200)
    assert all(raw[y * (3 * w + 1)] == 0 for y in range(h))  # filter bytes


def test_headless_app_rejects_bad_arguments(gpu):
    from lgca_gb300 import _build
    r = subprocess.run([_build.app_path("lgca_headless"), "--case"], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


def run_app(gpu, *args):
    from lgca_gb300 import _build
    r = subprocess.run([_build.app_path("lgca_headless"), *map(str, args)], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1]), r


@pytest.mark.gpu
def test_single_collision_app_matches_oracle(gpu, oracle, tmp_path):
    summary, _ = run_app(gpu, "--case", "single", "--frames", 9, "--format", "vti", "--out",
                         tmp_path)
    W, H = summary["dims"]
    p = P.lattice_parameters(3, "collision", 80.0, 0.2, 1)
    assert (W, H) == (p["dim_x"], p["dim_y"])
    st = P.init_single_collision(3, W, H)
    fin = oracle.run(3, st, summary["steps"], types=G.pipe(W, H), seed=0)
    cd, cm, md, mm = oracle.post_process(3, fin, 1)
    cell, _ = read_vti(tmp_path / f"cell_res_{summary['steps']}.vti")
    mean, _ = read_vti(tmp_path / f"mean_res_{summary['steps']}.vti")
    assert np.array_equal(cell["Cell density"].ravel().view(np.uint32), cd.ravel().view(np.uint32))
    assert np.array_equal(cell["Cell momentum"].ravel().view(np.uint32), cm.ravel().view(np.uint32))
    assert np.array_equal(mean["Mean density"].ravel().view(np.uint32), md.ravel().view(np.uint32))
    assert np.array_equal(mean["Mean momentum"].ravel().view(np.uint32), mm.ravel().view(np.uint32))
    assert summary["particles_start"] == summary["particles_end"] == 2


@pytest.mark.gpu
def test_diffusion_app_matches_oracle(gpu, oracle, tmp_path):
    summary, _ = run_app(gpu, "--case", "diffusion", "--Re", 64, "--frames", 15, "--format", "vti",
                         "--every", 14, "--out", tmp_path, "--seed", 9)
    W, H = summary["dims"]
    types = G.reflecting(W, H, "back")
    full = oracle.init_bernoulli(3, W, H, types, seed=9, p_move=1 / 7, p_rest=1 / 7)
    cx, cy, diam = W // 2, H // 2, np.float32(H // 4)
    y, x = np.mgrid[0:H, 0:W]
    dist = np.sqrt((x - cx).astype(np.float64) ** 2 + (y - cy).astype(np.float64) ** 2)
    disc = dist.astype(np.float32).astype(np.float64) < np.float64(diam) / 2.0
    st = np.where(disc, full, 0).astype(np.uint8)
    fin = oracle.run(3, st, summary["steps"], types=types, seed=9)
    cd, cm, md, mm = oracle.post_process(3, fin, 1)
    cell, _ = read_vti(tmp_path / f"cell_res_{summary['steps']}.vti")
    assert np.array_equal(cell["Cell density"].ravel().view(np.uint32), cd.ravel().view(np.uint32))
    assert np.array_equal(cell["Cell momentum"].ravel().view(np.uint32), cm.ravel().view(np.uint32))
    assert summary["particles_start"] == summary["particles_end"] == oracle.count_particles(st)


@pytest.mark.gpu
@pytest.mark.parametrize("case,extra", [("pipe", ["--frames", 12]), ("karman", ["--frames", 6]),
                                        ("box", ["--steps", 40, "--Re", 96]),
                                        ("periodic", ["--steps", 40, "--Re", 96, "--model", "HPP"]),
                                        ("pipe", ["--frames", 5, "--model", "FHP_I", "--format", "png"])])
def test_app_loops_conserve_particles(gpu, tmp_path, case, extra):
    summary, r = run_app(gpu, "--case", case, "--out", tmp_path, *extra)
    assert summary["particles_start"] == summary["particles_end"] > 0
    if case in ("pipe", "karman"):
        model = {"FHP_I": 1}.get(extra[extra.index("--model") + 1], 3) if "--model" in extra else 3
        p = P.lattice_parameters(model, case, 80.0, 0.3, 10 if case == "pipe" else 20)
        assert summary["dims"] == [p["dim_x"], p["dim_y"]]
        assert summary["mean_velocity"][0] > 0.0  # the forcing drives the flow in +x
    if "png" in extra:
        pngs = sorted(tmp_path.glob("res_*.png"))
        assert pngs
        w, h, _ = read_png(pngs[-1])
        assert (w, h) == (summary["dims"][0] // 20, summary["dims"][1] // 20)


# ------------------------------------------------------------------ oracle app loops
def oracle_viewer_loop(oracle, model, case, frames, seed, Re, Ma, r, pp=5):
    """The pipe / karman viewer loop (apps/pipe/pipe_viewer.cpp:100-146,
    apps/karman/karman_viewer.cpp: same loop) on the oracle: mean velocity,
    the forcing controller with the reference's thresholds, the random-cell
    body force (src/omp_lattice.cpp:254-346), then pp steps per frame.
    Returns the final state and the controller's trace."""
    p = P.lattice_parameters(model, case, Re, Ma, r)
    W, H = p["dim_x"], p["dim_y"]
    types = G.pipe(W, H) if case == "pipe" else G.karman_reference(W, H)
    D = P.NUM_DIR[model]
    st = oracle.init_bernoulli(model, W, H, types, seed=seed, p_move=1 / D, p_rest=1 / D)
    u_ref = np.float32(p["u"])
    forcing, call, steps, trace = p["initial_forcing"], 0, 0, []
    for _ in range(frames):
        ux, _ = oracle.mean_velocity(model, st, types)
        ux = np.float32(ux)
        applied, nrev = -1, 0
        if ux < u_ref:  # float comparison, as Real < Real
            if float(ux) > 0.9 * float(u_ref):  # double comparison, as Real > double
                forcing = p["equilibrium_forcing"]
            st, nrev = oracle.apply_body_force(model, st, forcing, types=types, seed=seed, call=call,
                                               bf_dir="x")
            call += 1
            applied = forcing
        trace.append((ux, applied, nrev))
        st = oracle.run(model, st, pp, types=types, seed=seed, t0=steps)
        steps += pp
    return st, trace, (W, H)


# (case, model, frames, Re, Ma, controller branches the run takes): at Ma 0.3
# the flow passes 0.9 u and the controller switches from the initial to the
# equilibrium forcing; at Ma 0.05 it overshoots u and stops forcing
@pytest.mark.gpu
@pytest.mark.parametrize("case,model,frames,Re,Ma,branches", [
    ("pipe", "FHP_III", 20, 20.0, 0.3, ("initial", "equilibrium")),
    ("pipe", "FHP_I", 18, 20.0, 0.3, ("initial", "equilibrium")),
    ("pipe", "HPP", 16, 20.0, 0.3, ("initial", "equilibrium")),
    ("pipe", "FHP_III", 14, 10.0, 0.05, ("initial", "none")),
    ("karman", "FHP_III", 16, 20.0, 0.3, ("initial", "equilibrium"))])
def test_viewer_loop_with_forcing_controller_matches_oracle(gpu, oracle, tmp_path, case, model,
                                                             frames, Re, Ma, branches):
    """The pipe and karman app loops on the GPU (C++ GB_Lattice over the
    shared device half of include/lgca/gb_device.h): the mean velocity
    feeding the controller, the body force it applies and the state after the
    run equal the oracle running the same loop."""
    mnum = {"HPP": 0, "FHP_I": 1, "FHP_III": 3}[model]
    r = 10 if case == "pipe" else 20
    dump = tmp_path / "state.bin"
    summary, _ = run_app(gpu, "--case", case, "--model", model, "--frames", frames, "--Re", Re,
                         "--Ma", Ma, "--r", r, "--seed", 5, "--dump", dump)
    want, trace, (W, H) = oracle_viewer_loop(oracle, mnum, case, frames, 5, Re, Ma, r)
    assert summary["dims"] == [W, H]
    got_trace = summary["trace"]
    assert len(got_trace) == frames
    for (ux_bits, applied, nrev), (ux, w_applied, w_nrev) in zip(got_trace, trace):
        gux = np.array([ux_bits], np.uint32).view(np.float32)[0]
        assert gux == pytest.approx(float(ux), rel=1e-5, abs=1e-7)
        assert (applied, nrev) == (w_applied, w_nrev)
    applied = {a for _, a, _ in trace}
    p = P.lattice_parameters(mnum, case, Re, Ma, r)
    names = {"initial": p["initial_forcing"], "equilibrium": p["equilibrium_forcing"], "none": -1}
    assert {names[b] for b in branches} <= applied
    got = np.fromfile(dump, np.uint8).reshape(H, W)
    assert np.array_equal(got, want)


@pytest.mark.gpu
@pytest.mark.parametrize("case,model", [("box", "FHP_III"), ("periodic", "HPP"),
                                        ("periodic", "FHP_II")])
def test_cli_loop_matches_oracle(gpu, oracle, tmp_path, case, model):
    """The box / periodic CLI loop (apps/box/main.cpp:230-312): steps 0..N,
    no forcing (bf_dir is 0 for these test cases)."""
    mnum = {"HPP": 0, "FHP_II": 2, "FHP_III": 3}[model]
    dump = tmp_path / "state.bin"
    summary, _ = run_app(gpu, "--case", case, "--model", model, "--steps", 30, "--Re", 96,
                         "--seed", 3, "--dump", dump)
    p = P.lattice_parameters(mnum, case, 96.0, 0.3, 4)
    W, H = p["dim_x"], p["dim_y"]
    types = G.reflecting(W, H, "back") if case == "box" else G.periodic(W, H)
    D = P.NUM_DIR[mnum]
    st = oracle.init_bernoulli(mnum, W, H, types, seed=3, p_move=1 / D, p_rest=1 / D)
    want = oracle.run(mnum, st, summary["steps"], types=types, seed=3)
    got = np.fromfile(dump, np.uint8).reshape(H, W)
    assert np.array_equal(got, want)
