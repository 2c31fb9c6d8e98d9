"""GPU parity of the step kernels (liblgca_gpu.so through the C ABI) against
the golden fixtures made by the reference and against the oracle.  Integer /
bit work: every comparison is bit-exact."""
import hashlib

import numpy as np
import pytest

from conftest import load_json, load_npz
from lgca_gb300 import geometry as G

pytestmark = pytest.mark.gpu
MODELS = [0, 1, 2, 3]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def run_gpu(gpu, model, init, steps, types=None, seed=0, chir=None, force_x=-1, force_p=0.0, t0=0,
            depth=1, chunks=None, variant=0, block_warps=0):
    H, W = init.shape
    with gpu.GpuLattice(model, W, H, seed) as L:
        L.set_block_warps(block_warps)
        if types is not None:
            L.set_cell_types(types)
        L.upload(init)
        L.set_step(t0)
        if chir is not None:
            L.set_chirality(chir)
        L.set_forcing_column(force_x, force_p)
        L.set_temporal_depth(depth)
        L.set_kernel_variant(variant)
        if chunks is None:
            L.collide_and_propagate(steps)
        else:
            done = 0
            for c in chunks:
                L.collide_and_propagate(c)
                done += c
            assert done == steps
        assert L.step_count == t0 + steps
        return L.download()


def test_golden_trajectories(gpu):
    meta = load_json("trajectories.json")
    npz = load_npz("trajectories.npz")
    for i, c in enumerate(meta):
        types = npz[f"c{i}_types"].astype(np.int32)
        chir = npz[f"c{i}_chir"] if f"c{i}_chir" in npz.files else None
        out = run_gpu(gpu, c["model"], npz[f"c{i}_init"], c["steps"], types=types, seed=c["seed"],
                      chir=chir, force_x=c["force_x"], force_p=c["force_p"])
        assert np.array_equal(out, npz[f"c{i}_final"]), c


WIDTHS = [1, 2, 3, 31, 63, 64, 65, 127, 128, 129, 200, 2047, 2048, 2049, 4160]


@pytest.mark.parametrize("model", MODELS)
@pytest.mark.parametrize("W", WIDTHS)
def test_ragged_widths_periodic_vs_oracle(gpu, oracle, model, W):
    H = 6
    st = oracle.init_bernoulli(model, W, H, None, seed=W, p_move=0.4, p_rest=0.3)
    want = oracle.run(model, st, 9, seed=W + 1)
    got = run_gpu(gpu, model, st, 9, seed=W + 1)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("model", MODELS)
@pytest.mark.parametrize("geom", ["pipe", "karman", "reflecting_back", "reflecting_forward", "disc"])
def test_geometries_and_forcing_vs_oracle(gpu, oracle, model, geom):
    rng = np.random.default_rng(17 * model + len(geom))
    for W, H in [(64, 32), (130, 40), (1000, 24), (2112, 10)]:
        types = {"pipe": G.pipe, "karman": G.karman_reference,
                 "reflecting_back": lambda w, h: G.reflecting(w, h, "back"),
                 "reflecting_forward": lambda w, h: G.reflecting(w, h, "forward"),
                 "disc": lambda w, h: G.disc(w, h, w // 3, h // 2, h // 3)}[geom](W, H)
        seed = int(rng.integers(1 << 40))
        st = oracle.init_bernoulli(model, W, H, types, seed=seed, p_move=0.3, p_rest=0.4)
        # forcing columns on word edges, the seam and inside words
        for fx in (0, 1, 63, 64, W - 1, int(rng.integers(0, W))):
            if fx >= W:
                continue
            kw = dict(types=types, seed=seed, force_x=fx, force_p=0.6, t0=int(rng.integers(100)))
            want = oracle.run(model, st, 13, **kw)
            got = run_gpu(gpu, model, st, 13, **kw)
            assert np.array_equal(got, want), (W, H, fx)


@pytest.mark.parametrize("model", [1, 2, 3])
def test_frozen_chirality_vs_oracle(gpu, oracle, model):
    rng = np.random.default_rng(model)
    W, H = 300, 20
    st = oracle.init_bernoulli(model, W, H, None, seed=4, p_move=0.4)
    chir = rng.integers(0, 2, (H, W), dtype=np.uint8)
    want = oracle.run(model, st, 17, chir=chir, seed=4)
    got = run_gpu(gpu, model, st, 17, chir=chir, seed=4)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("model", MODELS)
def test_step_splitting_is_invisible(gpu, oracle, model):
    W, H = 256, 64
    types = G.pipe(W, H)
    st = oracle.init_bernoulli(model, W, H, types, seed=8, p_move=0.3)
    kw = dict(types=types, seed=8, force_x=10, force_p=0.3)
    a = run_gpu(gpu, model, st, 24, **kw)
    b = run_gpu(gpu, model, st, 24, chunks=[1, 5, 7, 11], **kw)
    assert np.array_equal(a, b)
    assert np.array_equal(a, oracle.run(model, st, 24, **kw))


def test_config_pipe_fhp1_1024x512_1000_steps(gpu):
    """BASELINE workload 1 at full size: bit-exact with the reference run."""
    pins = load_json("config_pins.json")["pipe_fhp1_1024x512"]
    W, H = 1024, 512
    with gpu.GpuLattice(1, W, H, seed=1) as L:
        L.set_cell_types(G.pipe(W, H))
        L.init_random(0.2, 0.2)
        assert sha(L.download()) == pins["init_sha"]
        L.set_forcing_column(8, 0.01)
        L.collide_and_propagate(1000)
        fin = L.download()
        assert sha(fin) == pins["final_sha"]
        assert L.count_particles() == pins["particles"]
        N, Jx2, Jy = L.block_sums(16)
    g = load_npz("config_pipe_blocksums.npz")
    assert np.array_equal(N, g["N"]) and np.array_equal(Jx2, g["Jx2"]) and np.array_equal(Jy, g["Jy"])


def blocksum_sha(N, Jx2, Jy):
    return sha(np.stack([N.astype(np.int32), Jx2.astype(np.int32), Jy.astype(np.int32)]))


def run_karman_config(gpu, depth=1, variant=0):
    """BASELINE workload 2 over its whole run: FHP-III 8192x2048, disc r=128
    at (1024,1024), forcing column x=16 p=0.02, 10000 steps, 32x32 block sums
    every 100 steps.  Asserted against the reference run: the full block sums
    at t=100 and t=200, the hash of every one of the 100 block-sum sets and
    the state hash every 1000 steps."""
    pins = load_json("config_pins.json")["karman_fhp3_8192x2048"]
    long = load_json("config_karman_long.json")
    assert long["engine"] == "ref" and long["steps"] == 10000
    g = load_npz("config_karman_blocksums.npz")
    W, H = 8192, 2048
    types = G.disc(W, H, 1024, 1024, 128)
    assert sha(types) == pins["types_sha"]
    with gpu.GpuLattice(3, W, H, seed=2) as L:
        L.set_cell_types(types)
        L.init_random(0.3, 0.3)
        assert sha(L.download()) == pins["init_sha"] == long["init_sha"]
        L.set_forcing_column(16, 0.02)
        L.set_temporal_depth(depth)
        L.set_kernel_variant(variant)
        n0 = L.count_particles()
        checked = 0
        for t in range(100, 10001, 100):
            L.collide_and_propagate(100)
            N, Jx2, Jy = L.block_sums(32)
            assert blocksum_sha(N, Jx2, Jy) == long["blocksum_sha"][str(t)], t
            assert [int(N.sum()), int(Jx2.sum()), int(Jy.sum())] == long["blocksum_total"][t // 100 - 1]
            if t in (100, 200):
                tag = f"t{t}"
                assert np.array_equal(N, g[f"{tag}_N"]) and np.array_equal(Jx2, g[f"{tag}_Jx2"])
                assert np.array_equal(Jy, g[f"{tag}_Jy"])
                assert sha(L.download()) == pins[f"{tag}_sha"]
            if t % 1000 == 0:
                assert sha(L.download()) == long["state_sha"][str(t)], t
            checked += 1
        # forcing turns particles around, walls and the disc reflect them
        assert L.count_particles() == n0
    assert checked == 100


def test_config_karman_fhp3_8192x2048(gpu):
    """The plain kernel over the whole Karman run, bit-exact with the reference."""
    run_karman_config(gpu)


@pytest.mark.parametrize("model", MODELS)
def test_large_periodic_mass_and_block_totals(gpu, model):
    """Full-width roofline lattice (32768 x 16384): mass is conserved and the
    block sums add up to the particle count (size-independent properties)."""
    W, H = 32768, 16384
    with gpu.GpuLattice(model, W, H, seed=3) as L:
        L.init_random(0.5, 0.5)
        n0 = L.count_particles()
        _, jx0, jy0 = L.block_sums(64)
        L.collide_and_propagate(20)
        assert L.count_particles() == n0
        N, Jx2, Jy = L.block_sums(64)
        assert int(N.astype(np.int64).sum()) == n0
        # a periodic lattice without obstacles or forcing conserves momentum
        assert int(Jx2.astype(np.int64).sum()) == int(jx0.astype(np.int64).sum())
        assert int(Jy.astype(np.int64).sum()) == int(jy0.astype(np.int64).sum())


# ------------------------------------------------ temporally blocked kernel
GEOMS = {"periodic": G.periodic, "pipe": G.pipe, "karman": G.karman_reference,
         "reflecting_back": lambda w, h: G.reflecting(w, h, "back"),
         "reflecting_forward": lambda w, h: G.reflecting(w, h, "forward"),
         "disc": lambda w, h: G.disc(w, h, w // 3, h // 2, max(1, h // 3))}


@pytest.mark.parametrize("model", MODELS)
@pytest.mark.parametrize("depth", [2, 3, 4, 5, 8])
@pytest.mark.parametrize("geom", sorted(GEOMS))
@pytest.mark.parametrize("variant", [2, 3, 4])
def test_temporal_blocking_vs_oracle(gpu, oracle, model, depth, geom, variant):
    """k steps per pass give the same bits as one step per pass."""
    rng = np.random.default_rng(depth * 31 + model)
    for W, H in [(64, 2), (128, 10), (2048, 18), (4160, 40), (256, 64)]:
        types = GEOMS[geom](W, H)
        seed = int(rng.integers(1 << 40))
        st = oracle.init_bernoulli(model, W, H, types, seed=seed, p_move=0.35, p_rest=0.3)
        fx = int(rng.choice([x for x in (0, 63, 64, W - 1, int(rng.integers(W))) if x < W]))
        kw = dict(types=types, seed=seed, force_x=fx, force_p=0.5, t0=int(rng.integers(50)))
        want = oracle.run(model, st, 19, **kw)
        got = run_gpu(gpu, model, st, 19, depth=depth, variant=variant, **kw)
        assert np.array_equal(got, want), (W, H, fx)


@pytest.mark.parametrize("model", [1, 3])
@pytest.mark.parametrize("variant", [2, 3, 4])
def test_temporal_blocking_frozen_chirality(gpu, oracle, model, variant):
    rng = np.random.default_rng(5)
    W, H = 640, 36
    st = oracle.init_bernoulli(model, W, H, None, seed=9, p_move=0.4)
    chir = rng.integers(0, 2, (H, W), dtype=np.uint8)
    want = oracle.run(model, st, 16, chir=chir, seed=9)
    got = run_gpu(gpu, model, st, 16, chir=chir, seed=9, depth=8, variant=variant)
    assert np.array_equal(got, want)


def test_resident_karman_config(gpu):
    """The whole Karman run on the resident kernel (152 bands of 13-14 rows,
    two warps per row), 100 steps per launch: the same reference pins."""
    run_karman_config(gpu, variant=6)


@pytest.mark.parametrize("model", MODELS)
@pytest.mark.parametrize("geom", sorted(GEOMS))
def test_resident_kernel_vs_oracle(gpu, oracle, model, geom):
    """The resident kernel gives the oracle's bits: bands of one row and of
    many, one to four warps per row, the forcing column on the x seam and
    inside, steps split over launches (forcing at the launch boundary).
    Widths it cannot hold (odd word counts) take one step per pass."""
    rng = np.random.default_rng(model * 13 + len(geom))
    for W, H in [(128, 10), (256, 64), (4096, 40), (8192, 300), (16384, 160), (2048, 2048),
                 (4160, 40)]:
        types = GEOMS[geom](W, H)
        seed = int(rng.integers(1 << 40))
        st = oracle.init_bernoulli(model, W, H, types, seed=seed, p_move=0.35, p_rest=0.3)
        for fx in (W - 1, int(rng.integers(W))):
            kw = dict(types=types, seed=seed, force_x=fx, force_p=0.5, t0=int(rng.integers(50)))
            want = oracle.run(model, st, 17, **kw)
            for chunks in (None, [1, 9, 7]):
                got = run_gpu(gpu, model, st, 17, variant=6, chunks=chunks, **kw)
                assert np.array_equal(got, want), (W, H, fx, chunks)


@pytest.mark.parametrize("model,geom", [(2, "pipe"), (3, "disc"), (3, "periodic")])
def test_resident_row_barrier_form_vs_oracle(gpu, oracle, model, geom):
    """FHP-II/III lattices whose bands take 24 or more warps run the resident
    kernel with row barriers instead of a block barrier per step: one warp
    per row (4096 x 3648, bands of 24 rows) and two (8192 x 2100, bands of
    14 rows), over 40 steps in one call and in calls of 17 and 23."""
    rng = np.random.default_rng(model * 5 + len(geom))
    for W, H in [(4096, 3648), (8192, 2100)]:
        types = GEOMS[geom](W, H)
        seed = int(rng.integers(1 << 40))
        st = oracle.init_bernoulli(model, W, H, types, seed=seed, p_move=0.3, p_rest=0.3)
        kw = dict(types=types, seed=seed, force_x=int(rng.integers(W)), force_p=0.2, t0=7)
        want = oracle.run(model, st, 40, **kw)
        for chunks in (None, [17, 23]):
            got = run_gpu(gpu, model, st, 40, variant=6, chunks=chunks, **kw)
            assert np.array_equal(got, want), (W, H, chunks)


@pytest.mark.parametrize("model", [1, 3])
def test_resident_kernel_frozen_chirality(gpu, oracle, model):
    rng = np.random.default_rng(7)
    W, H = 4096, 36
    st = oracle.init_bernoulli(model, W, H, None, seed=9, p_move=0.4)
    chir = rng.integers(0, 2, (H, W), dtype=np.uint8)
    want = oracle.run(model, st, 16, chir=chir, seed=9)
    got = run_gpu(gpu, model, st, 16, chir=chir, seed=9, variant=6)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("depth", [2, 4, 8])
@pytest.mark.parametrize("variant", [2, 3, 4])
def test_temporal_blocking_karman_config(gpu, depth, variant):
    """The whole Karman run with k steps per pass (register wavefront, shared-
    memory tiles) and with the persistent kernel: the same reference pins."""
    run_karman_config(gpu, depth=depth, variant=variant)


@pytest.mark.parametrize("model", MODELS)
@pytest.mark.parametrize("geom", sorted(GEOMS))
def test_one_step_kernels_one_and_two_words_per_lane(gpu, oracle, model, geom):
    """Widths that are multiples of 64 run the two-words-per-lane kernel,
    including odd word counts (the last pair holds one word and the row's
    padding); forcing columns sit on pair, word and chunk edges."""
    rng = np.random.default_rng(3 * model + len(geom))
    for W, H in [(64, 6), (128, 6), (192, 8), (256, 10), (320, 6), (384, 8), (1088, 10),
                 (1152, 12), (2112, 4), (4096, 4)]:
        types = GEOMS[geom](W, H)
        seed = int(rng.integers(1 << 40))
        st = oracle.init_bernoulli(model, W, H, types, seed=seed, p_move=0.35, p_rest=0.3)
        for fx in sorted(x for x in {0, 63, 64, 127, 128 % W, W - 64, W - 1, 4095 % W} if x < W):
            kw = dict(types=types, seed=seed, force_x=fx, force_p=0.7, t0=int(rng.integers(50)))
            want = oracle.run(model, st, 11, **kw)
            for variant in (1, 5):
                got = run_gpu(gpu, model, st, 11, variant=variant, **kw)
                assert np.array_equal(got, want), (W, H, fx, variant)


@pytest.mark.parametrize("model", MODELS)
@pytest.mark.parametrize("block_warps", [1, 2, 4, 8])
def test_launch_shapes_give_the_same_bits(gpu, oracle, model, block_warps):
    """Warps per block of the one-step kernels (rows of one or several words
    per lane, rows shared by a warp, partial last blocks) never change the
    result; consecutive steps overlap on the GPU by programmatic dependent
    launch, which must not let a step read its predecessor's input."""
    rng = np.random.default_rng(model * 10 + block_warps)
    for W, H, geom in [(100, 18, "pipe"), (640, 30, "karman"), (1024, 66, "reflecting_forward"),
                       (4096, 12, "periodic")]:
        types = GEOMS[geom](W, H)
        seed = int(rng.integers(1 << 40))
        st = oracle.init_bernoulli(model, W, H, types, seed=seed, p_move=0.3, p_rest=0.3)
        kw = dict(types=types, seed=seed, force_x=W // 3, force_p=0.5)
        want = oracle.run(model, st, 25, **kw)
        for variant in (1, 5):
            got = run_gpu(gpu, model, st, 25, variant=variant, block_warps=block_warps, **kw)
            assert np.array_equal(got, want), (W, H, geom, variant)


@pytest.mark.parametrize("model", [1, 3])
def test_steps_captured_in_a_cuda_graph(gpu, oracle, model):
    """Steps captured on a caller stream into a CUDA graph (plain launches
    under capture) replay exactly.  A captured call fixes its steps' keys
    and buffers: with an even number of steps per call, every replay repeats
    steps t .. t+k-1 on the current state."""
    torch = pytest.importorskip("torch")
    _captured_replays(gpu, oracle, model, torch, 640, 64, 4, variant=0)
    # a lattice and call the resident kernel would take: under capture the
    # engine steps one step per pass, so the replays chain the same way
    _captured_replays(gpu, oracle, model, torch, 4096, 40, 20, variant=6)


def _captured_replays(gpu, oracle, model, torch, W, H, k, variant):
    types = G.pipe(W, H)
    st = oracle.init_bernoulli(model, W, H, types, seed=5, p_move=0.3, p_rest=0.3)
    L = gpu.GpuLattice(model, W, H, seed=5)
    L.set_cell_types(types)
    L.upload(st)
    L.set_forcing_column(10, 0.3)
    L.set_kernel_variant(variant)
    L.sync()
    s = torch.cuda.Stream()
    L.set_stream(s.cuda_stream)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        assert L.step_plan(k)[0] == 1
        L.collide_and_propagate(k)
    for _ in range(3):
        g.replay()
    torch.cuda.synchronize()
    L.set_stream(None)
    want = st
    for _ in range(3):
        want = oracle.run(model, want, k, types=types, seed=5, t0=0, force_x=10, force_p=0.3)
    assert np.array_equal(L.download(), want)
    L.close()


@pytest.mark.parametrize("model", MODELS)
@pytest.mark.parametrize("p", [0.1, 0.5])
def test_roofline_sweep_kernels_at_1024(gpu, oracle, model, p):
    """Every kernel and depth of the roofline sweep (one-step; register
    wavefront and shared-memory tiles at 2, 4 and 8 steps per pass) on the
    sweep's 1024x1024 check lattice: periodic, Bernoulli p on every channel,
    seed 3, 16 steps -- bit-exact with the oracle."""
    W = H = 1024
    st = oracle.init_bernoulli(model, W, H, None, seed=3, p_move=p, p_rest=p)
    want = oracle.run(model, st, 16, seed=3)
    got = run_gpu(gpu, model, st, 16, seed=3)
    assert np.array_equal(got, want)
    for variant in (2, 3):
        for depth in (2, 4, 8):
            got = run_gpu(gpu, model, st, 16, seed=3, depth=depth, variant=variant)
            assert np.array_equal(got, want), (variant, depth)


def test_step_plan_names_the_kernels_a_call_runs(gpu, oracle):
    """lgca_step_plan reports the kernel family and launches of a call; the
    automatic choice takes the resident form, where it holds the lattice, for
    calls of 16 steps or more from 4 Mi sites (rows of 2048+ sites) and of 64
    or more from 1 Mi sites (rows of 4096+ sites), and passes of several
    steps on lattices far beyond L2."""
    W, H = 8192, 2048
    with gpu.GpuLattice(3, W, H, seed=2) as L:
        assert L.step_plan(100) == (6, 1)
        assert L.step_plan(16) == (6, 1)
        assert L.step_plan(15) == (1, 15)
        L.set_temporal_depth(4)
        assert L.step_plan(10)[0] == 1  # passes of up to 4 steps on the wavefront
        L.set_temporal_depth(1)
        L.set_kernel_variant(4)
        assert L.step_plan(10) == (4, 1)
        L.set_kernel_variant(1)
        assert L.step_plan(10) == (1, 10)
    with gpu.GpuLattice(3, 4160, 64, seed=2) as L:  # odd word count: not held
        assert L.step_plan(100) == (1, 100)
    with gpu.GpuLattice(3, 4096, 256, seed=2) as L:  # 1 Mi sites: long calls only
        assert L.step_plan(100) == (6, 1)
        assert L.step_plan(64) == (6, 1)
        assert L.step_plan(63) == (1, 63)
        L.set_kernel_variant(6)
        assert L.step_plan(16) == (6, 1)
    with gpu.GpuLattice(3, 4096, 128, seed=2) as L:  # held, but too small to pay
        assert L.step_plan(100) == (1, 100)
    with gpu.GpuLattice(3, 2048, 1024, seed=2) as L:  # 2 Mi sites, half of every warp idle
        assert L.step_plan(100) == (1, 100)
    with gpu.GpuLattice(3, 2048, 2048, seed=2) as L:  # 4 Mi sites
        assert L.step_plan(16) == (6, 1)
        assert L.step_plan(15) == (1, 15)
    # far beyond L2: HPP from 64 Mi sites takes 4 steps per pass on the wavefront,
    # with the same bits as one step per pass
    W, H = 8192, 8192
    with gpu.GpuLattice(0, W, H, seed=4) as L, gpu.GpuLattice(0, W, H, seed=4) as R:
        assert L.step_plan(10) == (1, 3)  # passes of 4, 4 and 2 steps
        for X in (L, R):
            X.init_random(0.3)
            X.set_forcing_column(100, 0.2)
        R.set_kernel_variant(5)
        assert R.step_plan(10) == (1, 10)
        L.collide_and_propagate(10)
        R.collide_and_propagate(10)
        assert np.array_equal(L.download(), R.download())
    with gpu.GpuLattice(3, 32768, 4096, seed=2) as L:  # too many rows per SM
        assert L.step_plan(100) == (1, 100)


def test_plan_shape_equals_a_new_lattices_step_plan(gpu):
    """lgca_plan_shape gives, without a lattice, what a new lattice of that
    shape reports; it refuses what lgca_create refuses."""
    for model, W, H in [(3, 8192, 2048), (3, 2048, 1024), (3, 2048, 2048), (3, 4096, 256),
                        (1, 4160, 64), (0, 8192, 8192), (0, 16384, 2048), (2, 320, 100)]:
        with gpu.GpuLattice(model, W, H, seed=1) as L:
            for n in (1, 15, 16, 63, 64, 100, 500):
                assert gpu.plan_shape(model, W, H, n) == L.step_plan(n), (model, W, H, n)
    for args in [(4, 64, 64, 10), (1, 64, 63, 10), (0, 0, 64, 10), (0, 64, 64, -1)]:
        with pytest.raises(gpu.LgcaError):
            gpu.plan_shape(*args)


@pytest.mark.parametrize("model", [0, 1, 3])
def test_run_job_equals_upload_steps_download(gpu, oracle, model):
    """lgca_run_job_async (state in, steps, state out in one call; the
    resident kernel converts the byte-per-cell layout inside its launch) gives
    the oracle's bits, on lattices the resident kernel holds and on others,
    with and without input and output buffers, twice in a row on one handle."""
    import torch
    rng = np.random.default_rng(model + 40)
    for W, H, geom in [(4096, 40, "karman"), (8192, 300, "pipe"), (4160, 40, "periodic"),
                       (2048, 2048, "disc")]:
        types = GEOMS[geom](W, H)
        seed = int(rng.integers(1 << 40))
        st = oracle.init_bernoulli(model, W, H, types, seed=seed, p_move=0.35, p_rest=0.3)
        kw = dict(types=types, seed=seed, force_x=W - 1, force_p=0.5)
        want1 = oracle.run(model, st, 12, **kw)
        want2 = oracle.run(model, want1, 9, t0=12, **kw)
        pin = lambda: torch.empty((H, W), dtype=torch.uint8, pin_memory=True).numpy()
        src, out1, out2 = pin(), pin(), pin()
        B = 32
        sums = torch.empty((3, -(-H // B), -(-W // B)), dtype=torch.int32, pin_memory=True).numpy()
        want_sums = oracle.block_sums(model, want2, B)
        src[:] = st | np.uint8((0xff << oracle.NUM_DIR[model]) & 0xff)  # bits above the channels ignored
        for variant in (0, 6):  # automatic (separate calls here), resident (conversions in the launch)
            out1[:] = 0
            out2[:] = 0
            with gpu.GpuLattice(model, W, H, seed) as L:
                L.set_cell_types(types)
                L.set_forcing_column(W - 1, 0.5)
                L.set_kernel_variant(variant)
                L.run_job_async(src, 12, out1)
                sums[:] = -1
                L.run_job_async(None, 9, out2, B, sums)
                L.sync()
                assert np.array_equal(out1, want1), (W, H, geom, variant)
                assert np.array_equal(out2, want2), (W, H, geom, variant)
                for i in range(3):
                    assert np.array_equal(sums[i], want_sums[i]), (W, H, geom, variant, i)
                assert np.array_equal(L.download(), want2)
                assert L.step_count == 21
                L.set_step(0)
                L.run_job_async(src, 12, None)
                assert np.array_equal(L.download(), want1)


@pytest.mark.parametrize("model", [0, 1, 3])
def test_steps_with_fused_block_sums(gpu, oracle, model):
    """lgca_collide_and_propagate_sums: the steps and the B x B block sums of
    their result equal the oracle's, with the sums inside the resident
    kernel's launch (B = 8, 16, 32, 64) or from the block-sum kernel (other
    B, other kernels), and repeated calls do not accumulate."""
    import torch
    rng = np.random.default_rng(model + 70)
    for W, H, variant in [(4096, 64, 6), (8192, 300, 6), (2048, 2048, 0), (4160, 40, 0)]:
        types = GEOMS["karman"](W, H)
        seed = int(rng.integers(1 << 40))
        st = oracle.init_bernoulli(model, W, H, types, seed=seed, p_move=0.35, p_rest=0.3)
        kw = dict(types=types, seed=seed, force_x=W // 3, force_p=0.5)
        want1 = oracle.run(model, st, 20, **kw)
        want2 = oracle.run(model, want1, 20, t0=20, **kw)
        with gpu.GpuLattice(model, W, H, seed) as L:
            L.set_cell_types(types)
            L.upload(st)
            L.set_forcing_column(W // 3, 0.5)
            L.set_kernel_variant(variant)
            for B in (8, 16, 32, 64, 48):
                L.upload(st)
                L.set_step(0)
                sums = torch.full((3, -(-H // B), -(-W // B)), -1, dtype=torch.int32, device="cuda")
                L.collide_and_propagate_sums(20, B, sums[0].data_ptr(), sums[1].data_ptr(),
                                             sums[2].data_ptr())
                L.collide_and_propagate_sums(20, B, sums[0].data_ptr(), sums[1].data_ptr(),
                                             sums[2].data_ptr())
                L.sync()
                assert np.array_equal(L.download(), want2), (W, H, B)
                got = sums.cpu().numpy()
                for i, w in enumerate(oracle.block_sums(model, want2, B)):
                    assert np.array_equal(got[i], w), (W, H, variant, B, i)
                if B == 32:  # three separate arrays (zeroed one by one)
                    L.upload(want1)
                    L.set_step(20)
                    parts = [torch.full((-(-H // B), -(-W // B)), -1, dtype=torch.int32,
                                        device="cuda") for _ in range(3)]
                    L.collide_and_propagate_sums(20, B, *(p.data_ptr() for p in parts))
                    L.sync()
                    for p, w in zip(parts, oracle.block_sums(model, want2, B)):
                        assert np.array_equal(p.cpu().numpy(), w), (W, H, variant)
