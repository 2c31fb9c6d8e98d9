"""CPU parity of the CUDA kernel code itself: the emulators in tests/
(step_emu.cpp, multistep_emu.cpp, batch_emu.cpp) compile the kernel sources
with g++, run every warp as 32 host threads in lockstep (shuffles through a
shared array, __syncthreads a block barrier), and the states they reach are
compared bit for bit with the oracle.  Covered: the one-word and
two-words-per-lane step bodies, the batch kernel's seam shuffles (WRAP), the
kernels k_step2, k_step, k_wave, k_multistep and k_batch on their grids, odd
word counts (a half last pair), narrow rows that share a warp, every model
and geometry mode, and forcing columns at the x seam.  No GPU is needed."""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from lgca_gb300 import geometry as G


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    gxx = shutil.which("g++")
    cuda_inc = "/usr/local/cuda/include"
    if gxx is None or not os.path.isdir(cuda_inc):
        pytest.skip("g++ or the CUDA headers not available")
    exe = tmp_path_factory.mktemp("emu") / "step_emu"
    subprocess.run([gxx, "-O1", "-std=c++20", "-Wno-attributes", "-I", cuda_inc,
                    os.path.join(ROOT, "tests", "step_emu.cpp"), "-o", str(exe), "-pthread",
                    *CUDART], check=True, capture_output=True)
    return exe


# the launchers compiled along with the kernels reference the CUDA runtime
# (never called here)
CUDA_LIB = "/usr/local/cuda/lib64"
CUDART = ["-L", CUDA_LIB, "-lcudart", f"-Wl,-rpath,{CUDA_LIB}"]
ENV = dict(os.environ, ASAN_OPTIONS="detect_leaks=0")


def run_emu(exe, tmp, model, cells, types, steps, seed, t0, force_x, force_thr, path):
    H, W = cells.shape
    inp, out = tmp / "in.bin", tmp / "out.bin"
    with open(inp, "wb") as f:
        f.write(struct.pack("<6i3Q", model, W, H, steps, force_x, path, seed, t0, force_thr))
        f.write(np.ascontiguousarray(cells, np.uint8).tobytes())
        f.write(np.ascontiguousarray(types, np.uint8).tobytes())
    r = subprocess.run([str(exe), str(inp), str(out)], capture_output=True, env=ENV)
    assert r.returncode == 0, (r.returncode, r.stderr[-500:])
    return np.frombuffer(out.read_bytes(), np.uint8).reshape(H, W)


GEOMS = {
    "periodic": lambda w, h: G.periodic(w, h),
    "pipe": G.pipe,
    "disc": lambda w, h: G.disc(w, h, w // 3, h // 2, max(2, h // 5)),
    "slip": lambda w, h: G.reflecting(w, h, "forward"),
}

# (width, height): pair widths with even and odd word counts, rows narrower
# than a warp (several rows per warp) and wider; one-word widths
PAIR = [(64, 12), (128, 10), (192, 14), (256, 8), (320, 12), (640, 6), (2112, 4)]
WORD = [(100, 10), (300, 8)]


@pytest.mark.parametrize("model", [0, 1, 3])
@pytest.mark.parametrize("geom", list(GEOMS))
def test_emulated_step_bodies_equal_oracle(emu, tmp_path, oracle, model, geom):
    rng = np.random.default_rng(model * 31 + len(geom))
    for W, H in PAIR + WORD:
        types = GEOMS[geom](W, H).astype(np.uint8)
        st = oracle.init_bernoulli(model, W, H, GEOMS[geom](W, H), seed=7, p_move=0.35,
                                   p_rest=0.3)
        # forcing on both seam words and at a random column
        for fx in sorted({0, W - 1, int(rng.integers(W))}):
            p = 0.4
            thr = oracle.prob_threshold(p)
            want = oracle.run(model, st, 5, types=GEOMS[geom](W, H), seed=11, t0=3,
                              force_x=fx, force_p=p)
            # step bodies: one word, pair, pair with seam shuffles
            paths = (1, 2) if W % 64 == 0 else (0,)
            for path in paths:
                got = run_emu(emu, tmp_path, model, st, types, 5, 11, 3, fx, thr, path)
                assert np.array_equal(got, want), (model, geom, W, H, fx, path)


@pytest.mark.parametrize("model", [0, 3])
def test_emulated_one_step_kernels_equal_oracle(emu, tmp_path, oracle, model):
    """The kernels k_step2 (chirality drawn before the dependency wait, pairs)
    and k_step (one word per lane) themselves, on grids of 4-warp blocks."""
    for W, H in [(64, 12), (320, 12), (640, 6), (100, 10)]:
        for geom in ("periodic", "slip"):
            types = GEOMS[geom](W, H)
            st = oracle.init_bernoulli(model, W, H, types, seed=7, p_move=0.35, p_rest=0.3)
            thr = oracle.prob_threshold(0.4)
            want = oracle.run(model, st, 4, types=types, seed=11, t0=3, force_x=W - 1,
                              force_p=0.4)
            for path in ((3, 4) if W % 64 == 0 else (4,)):
                got = run_emu(emu, tmp_path, model, st, types.astype(np.uint8), 4, 11, 3, W - 1,
                              thr, path)
                assert np.array_equal(got, want), (model, geom, W, H, path)


def test_emulated_step_bodies_stay_in_bounds(tmp_path, oracle):
    """The step bodies' loads and stores stay inside the state, geometry and
    output buffers: the emulator built with the address and undefined-
    behaviour sanitizers, on the widths where rows share or straddle warps."""
    gxx = shutil.which("g++")
    cuda_inc = "/usr/local/cuda/include"
    if gxx is None or not os.path.isdir(cuda_inc):
        pytest.skip("g++ or the CUDA headers not available")
    exe = tmp_path / "step_emu_asan"
    r = subprocess.run([gxx, "-O0", "-g", "-std=c++20", "-Wno-attributes",
                        "-fsanitize=address,undefined", "-fno-sanitize-recover=all",
                        "-fno-omit-frame-pointer", "-I", cuda_inc,
                        os.path.join(ROOT, "tests", "step_emu.cpp"), "-o", str(exe), "-pthread",
                        *CUDART], capture_output=True)
    if r.returncode != 0:
        pytest.skip("sanitizer runtime not available")
    for model in (0, 3):
        for W, H in [(64, 12), (320, 12), (640, 6), (100, 10)]:
            for geom in ("periodic", "slip"):
                types = GEOMS[geom](W, H).astype(np.uint8)
                st = oracle.init_bernoulli(model, W, H, GEOMS[geom](W, H), seed=7, p_move=0.35,
                                           p_rest=0.3)
                thr = oracle.prob_threshold(0.4)
                want = oracle.run(model, st, 3, types=GEOMS[geom](W, H), seed=11, t0=3,
                                  force_x=W - 1, force_p=0.4)
                for path in ((2, 3) if W % 64 == 0 else (0, 4)):
                    got = run_emu(exe, tmp_path, model, st, types, 3, 11, 3, W - 1, thr, path)
                    assert np.array_equal(got, want), (model, geom, W, H, path)


@pytest.fixture(scope="module")
def multistep_emu(tmp_path_factory):
    gxx = shutil.which("g++")
    cuda = "/usr/local/cuda"
    if gxx is None or not os.path.isdir(os.path.join(cuda, "include")):
        pytest.skip("g++ or the CUDA headers not available")
    exe = tmp_path_factory.mktemp("emu") / "multistep_emu"
    lib = os.path.join(cuda, "lib64")
    subprocess.run([gxx, "-O1", "-std=c++20", "-Wno-attributes", "-I", os.path.join(cuda, "include"),
                    os.path.join(ROOT, "tests", "multistep_emu.cpp"), "-o", str(exe), "-pthread",
                    "-L", lib, "-lcudart", f"-Wl,-rpath,{lib}"], check=True, capture_output=True)
    return exe


@pytest.mark.parametrize("model", [0, 1, 3])
def test_emulated_temporal_blocking_kernels_equal_oracle(multistep_emu, tmp_path, oracle, model):
    """k_wave (register wavefront) and k_multistep (shared-memory tiles) run
    as host threads: K = 2, 4, 8 steps per pass (the FHP wavefront up to 4),
    strips and tiles that wrap around narrow lattices, slabs that do not
    divide the height, every geometry mode and a forcing column on the seam."""
    for W, H in [(640, 40), (2112, 24), (128, 20)]:
        for geom in ("periodic", "pipe", "slip"):
            types = GEOMS[geom](W, H)
            st = oracle.init_bernoulli(model, W, H, types, seed=7, p_move=0.35, p_rest=0.3)
            thr = oracle.prob_threshold(0.4)
            for kernel in (0, 1):
                for depth in (2, 4, 8):
                    if kernel == 0 and depth == 8 and model != 0:
                        continue  # the FHP wavefront holds at most 4 time levels
                    want = oracle.run(model, st, depth, types=types, seed=11, t0=3,
                                      force_x=W - 1, force_p=0.4)
                    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
                    with open(inp, "wb") as f:
                        f.write(struct.pack("<7i3Q", model, W, H, depth, W - 1, kernel, depth,
                                            11, 3, thr))
                        f.write(st.tobytes())
                        f.write(types.astype(np.uint8).tobytes())
                    r = subprocess.run([str(multistep_emu), str(inp), str(out)], capture_output=True)
                    assert r.returncode == 0, (model, W, H, geom, kernel, depth, r.returncode)
                    got = np.frombuffer(out.read_bytes(), np.uint8).reshape(H, W)
                    assert np.array_equal(got, want), (model, W, H, geom, kernel, depth)


def test_emulated_step_bodies_random_configurations(emu, tmp_path, oracle):
    """Seeded random small lattices: any width (pair paths for multiples of
    64), random cell-type noise including slip cells, forcing anywhere with
    any probability, random seeds and start steps."""
    rng = np.random.default_rng(2024)
    for _ in range(40):
        model = int(rng.integers(4))
        W = 64 * int(rng.integers(1, 12)) if rng.random() < 0.6 else int(rng.integers(1, 700))
        H = 2 * int(rng.integers(1, 20))
        kind = int(rng.integers(3))
        if kind == 0:
            types = G.pipe(W, H)
        elif kind == 1:
            types = G.disc(W, H, int(rng.integers(W)), int(rng.integers(H)), int(rng.integers(1, 6)))
        else:
            types = rng.choice([0, 0, 0, 1, 2], size=(H, W)).astype(np.int32)
        types = np.ascontiguousarray(types, dtype=np.int32)
        st = oracle.init_bernoulli(model, W, H, types, seed=int(rng.integers(1000)),
                                   p_move=float(rng.uniform(0.1, 0.6)),
                                   p_rest=float(rng.uniform(0.1, 0.6)))
        fx = int(rng.integers(W)) if rng.random() < 0.7 else -1
        p = float(rng.uniform(0.05, 1.0))
        seed, t0, steps = int(rng.integers(1 << 40)), int(rng.integers(1 << 20)), int(rng.integers(1, 5))
        want = oracle.run(model, st, steps, types=types, seed=seed, t0=t0, force_x=fx,
                          force_p=p if fx >= 0 else 0.0)
        thr = oracle.prob_threshold(p) if fx >= 0 else 0
        for path in ((1, 2, 3) if W % 64 == 0 else (0, 4)):
            got = run_emu(emu, tmp_path, model, st, types.astype(np.uint8), steps, seed, t0, fx,
                          thr, path)
            assert np.array_equal(got, want), (model, W, H, kind, fx, p, seed, t0, steps, path)


@pytest.fixture(scope="module")
def batch_emu(tmp_path_factory):
    gxx = shutil.which("g++")
    cuda_inc = "/usr/local/cuda/include"
    if gxx is None or not os.path.isdir(cuda_inc):
        pytest.skip("g++ or the CUDA headers not available")
    exe = tmp_path_factory.mktemp("emu") / "batch_emu"
    # -O0: the kernel's many instantiations build in seconds; the small
    # lattices here run as fast either way
    subprocess.run([gxx, "-O0", "-std=c++20", "-Wno-attributes", "-I", cuda_inc,
                    os.path.join(ROOT, "tests", "batch_emu.cpp"), "-o", str(exe), "-pthread"],
                   check=True, capture_output=True)
    return exe


def test_emulated_batch_kernel_equals_oracle(batch_emu, tmp_path, oracle):
    """k_batch_keys, k_batch and k_batch_wave on their grids, with the
    call's work-lists: random mixed batches (models, pair / odd / one-word
    widths, geometries with cell-type noise, forcing, start steps, 0 to 6
    steps per member so members leave the work-list part way) at 1, 2, 4 and
    8 tasks per warp, then batches whose members ask for 2, 4 or 8 steps per
    pass (single steps first, then passes, several slabs per member); every
    member equals its lone oracle run."""
    rng = np.random.default_rng(77)
    for trial in range(32):
        wt = (1, 2, 4, 8)[trial % 4]
        mem = []
        for _ in range(int(rng.integers(1, 10))):
            model = int(rng.integers(4))
            W = 64 * int(rng.integers(1, 10)) if rng.random() < 0.7 else int(rng.integers(1, 400))
            H = 2 * int(rng.integers(1, 24 if trial < 16 else 80))
            kind = int(rng.integers(4))
            types = [G.periodic(W, H), G.pipe(W, H), G.reflecting(W, H, "forward"),
                     rng.choice([0, 0, 0, 1, 2], size=(H, W))][kind]
            types = np.ascontiguousarray(types, dtype=np.int32)
            st = oracle.init_bernoulli(model, W, H, types, seed=int(rng.integers(1000)),
                                       p_move=0.3, p_rest=0.3)
            fx = int(rng.integers(W)) if rng.random() < 0.6 else -1
            p = float(rng.uniform(0.05, 1.0))
            # from trial 16 on, members ask for the wavefront (2, 4 or 8 steps
            # per pass; those it does not apply to run one step per launch)
            K = int(rng.choice([0, 2, 4, 8])) if trial >= 16 else 0
            n = int(rng.integers(0, 7)) if trial < 16 else int(rng.integers(0, 20))
            mem.append((model, W, H, n, fx, int(rng.integers(1 << 40)),
                        int(rng.integers(1 << 20)), p, st, types, K))
        inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
        with open(inp, "wb") as f:
            f.write(struct.pack("<2i", len(mem), wt))
            for model, W, H, n, fx, seed, t0, p, st, types, K in mem:
                thr = oracle.prob_threshold(p) if fx >= 0 else 0
                f.write(struct.pack("<6i3Q", model, W, H, n, fx, K, seed, t0, thr))
                f.write(st.tobytes())
                f.write(types.astype(np.uint8).tobytes())
        r = subprocess.run([str(batch_emu), str(inp), str(out)], capture_output=True)
        assert r.returncode == 0, r.returncode
        data, off = out.read_bytes(), 0
        for model, W, H, n, fx, seed, t0, p, st, types, K in mem:
            got = np.frombuffer(data[off:off + W * H], np.uint8).reshape(H, W)
            off += W * H
            want = oracle.run(model, st, n, types=types, seed=seed, t0=t0, force_x=fx,
                              force_p=p if fx >= 0 else 0.0)
            assert np.array_equal(got, want), (trial, wt, model, W, H, n, fx)


def test_emulated_block_sums_equal_oracle(tmp_path, oracle):
    """The integer block-sum kernels (block_sums.cuh) on their grids: B
    dividing 64 (one thread per block row and word), B = 64·2^k (shuffle
    reduction) and any other B (one thread per block), ragged edges."""
    gxx = shutil.which("g++")
    cuda_inc = "/usr/local/cuda/include"
    if gxx is None or not os.path.isdir(cuda_inc):
        pytest.skip("g++ or the CUDA headers not available")
    exe = tmp_path / "block_sums_emu"
    subprocess.run([gxx, "-O1", "-std=c++20", "-Wno-attributes", "-I", cuda_inc,
                    os.path.join(ROOT, "tests", "block_sums_emu.cpp"), "-o", str(exe), "-pthread"],
                   check=True, capture_output=True)
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    for model in (0, 1, 3):
        for W, H in [(64, 16), (100, 30), (640, 40), (4160, 6)]:
            st = oracle.init_bernoulli(model, W, H, G.periodic(W, H), seed=5, p_move=0.4,
                                       p_rest=0.3)
            for B in (8, 16, 32, 64, 128, 2048, 7, 48):
                with open(inp, "wb") as f:
                    f.write(struct.pack("<4i", model, W, H, B))
                    f.write(st.tobytes())
                r = subprocess.run([str(exe), str(inp), str(out)], capture_output=True)
                assert r.returncode == 0, (model, W, H, B)
                Hb, Wb = -(-H // B), -(-W // B)
                got = np.frombuffer(out.read_bytes(), np.int32).reshape(3, Hb, Wb)
                want = oracle.block_sums(model, st, B)
                for i in range(3):
                    assert np.array_equal(got[i], want[i]), (model, W, H, B, i)


def _build_resident(out, sanitize=False):
    gxx = shutil.which("g++")
    cuda_inc = "/usr/local/cuda/include"
    if gxx is None or not os.path.isdir(cuda_inc):
        pytest.skip("g++ or the CUDA headers not available")
    flags = (["-O0", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=all",
              "-fno-omit-frame-pointer"] if sanitize else ["-O1"])
    r = subprocess.run([gxx, *flags, "-std=c++20", "-Wno-attributes", "-I", cuda_inc,
                        os.path.join(ROOT, "tests", "resident_emu.cpp"), "-o", str(out),
                        "-pthread", *CUDART], capture_output=True)
    if r.returncode != 0:
        if sanitize:
            pytest.skip("sanitizer runtime not available")
        raise AssertionError(r.stderr[-2000:])
    return out


@pytest.fixture(scope="module")
def resident_emu(tmp_path_factory):
    return _build_resident(tmp_path_factory.mktemp("res") / "resident_emu")


def run_resident(exe, tmp, model, cells, types, steps, seed, t0, force_x, force_thr, nblk,
                 chunk, withhold=-1, wait_ns=10_000_000_000, aos=0, B=0, rowsync=0):
    H, W = cells.shape
    inp, out = tmp / "rin.bin", tmp / "rout.bin"
    with open(inp, "wb") as f:
        f.write(struct.pack("<11i4Q", model, W, H, steps, force_x, nblk, chunk, withhold, aos, B,
                            rowsync, seed, t0, force_thr, wait_ns))
        f.write(np.ascontiguousarray(cells, np.uint8).tobytes())
        f.write(np.ascontiguousarray(types, np.uint8).tobytes())
    r = subprocess.run([str(exe), str(inp), str(out)], capture_output=True, env=ENV, timeout=600)
    assert r.returncode == 0, (r.returncode, r.stderr[-800:])
    raw = out.read_bytes()
    err = struct.unpack("<i", raw[:4])[0]
    got = np.frombuffer(raw[4:4 + H * W], np.uint8).reshape(H, W)
    rest = raw[4 + H * W:]
    extra = []
    if aos & 2:
        extra.append(np.frombuffer(rest[:H * W], np.uint8).reshape(H, W))
        rest = rest[H * W:]
    if B > 0:
        extra.append(np.frombuffer(rest, np.int32).reshape(3, -(-H // B), -(-W // B)))
    return (err, got, *extra)


# (W, H, blocks): one and two warps per row, a row of a single word pair,
# bands of one row (top row = bottom row), one band for the whole lattice,
# unequal bands
RESIDENT = [(4096, 12, 3), (8192, 8, 2), (128, 6, 6), (1024, 10, 1), (2048, 14, 4),
            (4096, 6, 6)]


@pytest.mark.parametrize("model,rowsync", [(0, 0), (1, 0), (3, 0), (3, 1)])
@pytest.mark.parametrize("geom", list(GEOMS))
def test_emulated_resident_kernel_equals_oracle(resident_emu, tmp_path, oracle, model, geom,
                                                rowsync):
    """The resident kernel k_resident (state on chip across steps, band edges
    exchanged as step-tagged halo items) on its whole grid: every
    model and geometry mode, forcing at the x seam and inside a row, steps
    run as one launch and split over several (forcing at the launch
    boundary, results written back unforced); FHP-III also in the
    row-barrier form."""
    rng = np.random.default_rng(model * 7 + len(geom))
    for W, H, nblk in RESIDENT:
        if model != 0 and H % 2:
            continue
        types = GEOMS[geom](W, H)
        st = oracle.init_bernoulli(model, W, H, types, seed=5, p_move=0.35, p_rest=0.3)
        for fx in (W - 1, int(rng.integers(W))):
            p = 0.4
            thr = oracle.prob_threshold(p)
            want = oracle.run(model, st, 6, types=types, seed=13, t0=9, force_x=fx, force_p=p)
            for chunk in (6, 4):
                err, got = run_resident(resident_emu, tmp_path, model, st, types.astype(np.uint8),
                                        6, 13, 9, fx, thr, nblk, chunk, rowsync=rowsync)
                assert err == 0
                assert np.array_equal(got, want), (model, geom, W, H, nblk, fx, chunk)
            # input read and result written in the byte-per-cell layout by the
            # launch itself (garbage in the bits above the model's channels)
            noisy = st | np.uint8((0xff << oracle.NUM_DIR[model]) & 0xff)
            B = (8, 16, 32, 64)[nblk % 4]
            err, got, aos_out, sums = run_resident(resident_emu, tmp_path, model, noisy,
                                                   types.astype(np.uint8), 6, 13, 9, fx, thr, nblk,
                                                   4, aos=3, B=B, rowsync=rowsync)
            assert err == 0
            assert np.array_equal(got, want) and np.array_equal(aos_out, want), (model, W, H)
            # B x B block sums of the result, fused into the last launch
            for i, w in enumerate(oracle.block_sums(model, want, B)):
                assert np.array_equal(sums[i], w), (model, W, H, nblk, B, i)


@pytest.mark.parametrize("model,geom,rowsync", [(3, "disc", 0), (3, "disc", 1), (1, "periodic", 0),
                                               (0, "pipe", 0)])
def test_emulated_resident_long_calls_equal_oracle(resident_emu, tmp_path, oracle, model, geom,
                                                   rowsync):
    """Calls of more steps than a warp draws random keys for at once (16),
    so that every warp's key ring refills mid-call and the row barriers go
    through many phases: one launch of 37 steps, and 40 steps as launches of
    17."""
    for W, H, nblk in [(2048, 14, 4), (8192, 8, 2)]:
        types = GEOMS[geom](W, H)
        st = oracle.init_bernoulli(model, W, H, types, seed=5, p_move=0.35, p_rest=0.3)
        thr = oracle.prob_threshold(0.3)
        for steps, chunk in ((37, 37), (40, 17)):
            want = oracle.run(model, st, steps, types=types, seed=13, t0=3, force_x=W // 3,
                              force_p=0.3)
            err, got = run_resident(resident_emu, tmp_path, model, st, types.astype(np.uint8),
                                    steps, 13, 3, W // 3, thr, nblk, chunk, rowsync=rowsync)
            assert err == 0 and np.array_equal(got, want), (model, geom, W, H, steps, chunk)


def test_emulated_resident_kernel_stays_in_bounds(tmp_path, oracle):
    """k_resident's shared-memory, halo and state accesses stay in bounds:
    the emulator built with the address and undefined-behaviour sanitizers."""
    exe = _build_resident(tmp_path / "resident_emu_asan", sanitize=True)
    for model, rowsync in ((0, 0), (3, 0), (3, 1)):
        for W, H, nblk in [(4096, 6, 3), (8192, 4, 2), (128, 4, 4)]:
            types = GEOMS["slip"](W, H)
            st = oracle.init_bernoulli(model, W, H, types, seed=5, p_move=0.35, p_rest=0.3)
            thr = oracle.prob_threshold(0.4)
            want = oracle.run(model, st, 3, types=types, seed=13, t0=9, force_x=W - 1,
                              force_p=0.4)
            err, got = run_resident(exe, tmp_path, model, st, types.astype(np.uint8), 3, 13, 9,
                                    W - 1, thr, nblk, 3, rowsync=rowsync)
            assert err == 0 and np.array_equal(got, want), (model, W, H, nblk, rowsync)


@pytest.mark.parametrize("rowsync", [0, 1])
def test_emulated_resident_wait_gives_up(resident_emu, tmp_path, oracle, rowsync):
    """A block that never writes its halo items makes its neighbours' bounded
    waits run out: every block returns, the error flag is set (with row
    barriers, also the waits of the rows behind the band edges)."""
    W, H = 4096, 12
    types = GEOMS["periodic"](W, H)
    st = oracle.init_bernoulli(3, W, H, types, seed=5, p_move=0.35, p_rest=0.3)
    err, _ = run_resident(resident_emu, tmp_path, 3, st, types.astype(np.uint8), 5, 13, 0, -1, 0,
                          3, 5, withhold=1, wait_ns=2_000_000, rowsync=rowsync)
    assert err == 1
