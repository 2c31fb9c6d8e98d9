"""GPU parity of the kernels around the step: layout conversion, init,
geometry, block sums, reference post-processing, reductions and the
random-cell body force.  Bit-exact except the mean velocity, whose reference
is an FP32 sum in thread-dependent order (tolerance stated below)."""
import numpy as np
import pytest

from conftest import load_json, load_npz
from lgca_gb300 import geometry as G

pytestmark = pytest.mark.gpu
MODELS = [0, 1, 2, 3]


@pytest.mark.parametrize("model", MODELS)
@pytest.mark.parametrize("W,H", [(1, 2), (5, 4), (64, 2), (100, 6), (1024, 8), (777, 10)])
def test_upload_download_roundtrip(gpu, model, W, H):
    rng = np.random.default_rng(W * H)
    D = gpu.NUM_DIR[model]
    st = rng.integers(0, 256, (H, W), dtype=np.uint8)
    with gpu.GpuLattice(model, W, H) as L:
        L.upload(st)
        assert np.array_equal(L.download(), st & np.uint8((1 << D) - 1))
        assert L.count_particles() == int(np.unpackbits(st & np.uint8((1 << D) - 1)).sum())


@pytest.mark.parametrize("model", MODELS)
def test_init_random_matches_oracle(gpu, oracle, model):
    for W, H, geom in [(130, 20, G.pipe), (64, 64, G.periodic), (333, 12, G.karman_reference)]:
        types = geom(W, H)
        with gpu.GpuLattice(model, W, H, seed=99) as L:
            L.set_cell_types(types)
            L.init_random(0.37, 0.61)
            got = L.download()
        want = oracle.init_bernoulli(model, W, H, types, seed=99, p_move=0.37, p_rest=0.61)
        assert np.array_equal(got, want)


def test_cell_types_roundtrip_and_validation(gpu):
    W, H = 150, 30
    t = G.reflecting(W, H, "forward")
    t[10:20, 40:60] = G.SOLID_NO_SLIP
    with gpu.GpuLattice(2, W, H) as L:
        L.set_cell_types(t)
        assert np.array_equal(L.get_cell_types(), t)
        bad = t.copy()
        bad[3, 7] = 5
        with pytest.raises(gpu.LgcaError):
            L.set_cell_types(bad)
        assert np.array_equal(L.get_cell_types(), t)  # unchanged by the rejected call


@pytest.mark.parametrize("model", MODELS)
@pytest.mark.parametrize("B", [1, 2, 3, 5, 8, 16, 20, 32, 64, 100, 128, 256])
def test_block_sums_match_oracle(gpu, oracle, model, B):
    W, H = 520, 90
    st = oracle.init_bernoulli(model, W, H, None, seed=B, p_move=0.45, p_rest=0.3)
    with gpu.GpuLattice(model, W, H) as L:
        L.upload(st)
        got = L.block_sums(B)
    want = oracle.block_sums(model, st, B)
    for g, w in zip(got, want):
        assert np.array_equal(g, w)


@pytest.mark.parametrize("B", [1, 16, 37])
def test_block_sums_async_after_steps(gpu, oracle, B):
    """The non-blocking form gives the blocking form's values once the
    handle's stream is synchronised, also when steps were queued before it."""
    import torch
    W, H = 640, 96
    st = oracle.init_bernoulli(3, W, H, None, seed=5, p_move=0.3, p_rest=0.3)
    Hb, Wb = -(-H // B), -(-W // B)
    buf = torch.zeros((3, Hb, Wb), dtype=torch.int32, pin_memory=True).numpy()
    with gpu.GpuLattice(3, W, H, seed=8) as L:
        L.upload(st)
        L.collide_and_propagate(7)
        L.block_sums_async(B, buf[0], buf[1], buf[2])
        L.sync()
        want = oracle.block_sums(3, L.download(), B)
    for g, w in zip(buf, want):
        assert np.array_equal(g, w)


@pytest.mark.parametrize("model", MODELS)
def test_post_process_matches_golden_bitwise(gpu, model):
    npz = load_npz("postprocess.npz")
    keys = sorted({k.rsplit("_", 1)[0] for k in npz.files if k.startswith(f"m{model}_")})
    for k in keys:
        r = int(k.rsplit("_r", 1)[1])
        st = npz[k + "_state"]
        H, W = st.shape
        with gpu.GpuLattice(model, W, H) as L:
            L.upload(st)
            got = L.post_process(r)
        for name, g in zip(("cd", "cm", "md", "mm"), got):
            want = npz[f"{k}_{name}"]
            assert np.array_equal(g.view(np.uint32), want.view(np.uint32)), (k, name)


@pytest.mark.parametrize("model", MODELS)
def test_post_process_matches_oracle_bitwise(gpu, oracle, model):
    for W, H, r in [(200, 60, 10), (1024, 128, 8), (96, 32, 16), (10, 8, 4)]:
        st = oracle.init_bernoulli(model, W, H, None, seed=W, p_move=0.5, p_rest=0.5)
        with gpu.GpuLattice(model, W, H) as L:
            L.upload(st)
            got = L.post_process(r)
        for g, w in zip(got, oracle.post_process(model, st, r)):
            assert np.array_equal(g.view(np.uint32), w.view(np.uint32)), (W, H, r)


def test_mean_velocity(gpu, oracle):
    """Reference: FP32 sum of per-cell u over fluid cells (thread-order
    dependent); here summed in double.  Tolerance: 1e-5 relative + 1e-7."""
    for c in load_json("params.json")["mean_velocity"]:
        m, W, H = c["model"], c["W"], c["H"]
        types = G.pipe(W, H)
        st = oracle.init_bernoulli(m, W, H, types, seed=c["seed"], p_move=0.3, p_rest=0.3)
        st = oracle.run(m, st, c["steps"], types=types, seed=c["seed"], force_x=c["force_x"],
                        force_p=c["force_p"])
        with gpu.GpuLattice(m, W, H) as L:
            L.set_cell_types(types)
            L.upload(st)
            ux, uy = L.mean_velocity()
        assert ux == pytest.approx(c["ux"], rel=1e-5, abs=1e-7)
        assert uy == pytest.approx(c["uy"], rel=1e-5, abs=1e-7)


def test_body_force_matches_golden(gpu):
    meta = load_json("bodyforce.json")
    npz = load_npz("bodyforce.npz")
    geoms = {"pipe": G.pipe, "periodic": G.periodic, "karman": G.karman_reference}
    for i, c in enumerate(meta):
        types = geoms[c["geometry"]](c["W"], c["H"])
        with gpu.GpuLattice(c["model"], c["W"], c["H"], seed=c["seed"]) as L:
            L.set_cell_types(types)
            L.upload(npz[f"b{i}_init"])
            for _ in range(c["call"]):  # advance the handle's call counter
                L.apply_body_force(0, None)
            L.apply_body_force(c["forcing"], c["dir"])
            assert np.array_equal(L.download(), npz[f"b{i}_final"]), c


@pytest.mark.parametrize("model", MODELS)
def test_body_force_matches_oracle_large(gpu, oracle, model):
    """Several chunks of candidates, targets reached mid-chunk and never."""
    W, H = 1000, 700
    types = G.karman_reference(W, H)
    st = oracle.init_bernoulli(model, W, H, types, seed=6, p_move=0.3, p_rest=0.3)
    for call, (forcing, d) in enumerate([(7000, "x"), (150000, "x"), (50000, "y"), (10 ** 9, "x"),
                                         (1, "y")]):
        want, nrev = oracle.apply_body_force(model, st, forcing, types=types, seed=6, call=call,
                                             bf_dir=d)
        with gpu.GpuLattice(model, W, H, seed=6) as L:
            L.set_cell_types(types)
            L.upload(st)
            for _ in range(call):
                L.apply_body_force(0, None)
            n = L.apply_body_force(forcing, d)
            got = L.download()
        assert n == nrev
        assert np.array_equal(got, want), (forcing, d)


@pytest.mark.parametrize("model", MODELS)
def test_body_force_consecutive_calls_match_oracle(gpu, oracle, model):
    """Calls in a row on one handle: each call leaves the first-occurrence
    table all ones for the next (only the drawn entries are reset), across
    targets reached in the first chunk, in a later chunk, never, and the
    minimal target of one draw."""
    W, H = 1536, 1100
    types = G.karman_reference(W, H)
    st = oracle.init_bernoulli(model, W, H, types, seed=8, p_move=0.3, p_rest=0.3)
    calls = [(500, "x"), (120000, "y"), (10 ** 9, "x"), (0, "x"), (30000, "y"), (1, "x"),
             (400000, "x")]
    with gpu.GpuLattice(model, W, H, seed=8) as L:
        L.set_cell_types(types)
        L.upload(st)
        want = st
        for call, (forcing, d) in enumerate(calls):
            want, nrev = oracle.apply_body_force(model, want, forcing, types=types, seed=8, call=call,
                                                 bf_dir=d)
            assert L.apply_body_force(forcing, d) == nrev, call
            assert np.array_equal(L.download(), want), call


@pytest.mark.parametrize("model", MODELS)
def test_checkpoint_resume_is_bit_exact(gpu, oracle, model):
    """Stop after 17 steps, save, restore into a fresh handle, run 23 more:
    identical to 40 uninterrupted steps (geometry, forcing, chirality,
    body-force counter and step counter all carried)."""
    W, H = 320, 40
    types = G.reflecting(W, H, "forward")
    types[10:20, 100:120] = G.SOLID_NO_SLIP
    rng = np.random.default_rng(model)
    chir = rng.integers(0, 2, (H, W), dtype=np.uint8) if model == 2 else None

    def fresh():
        L = gpu.GpuLattice(model, W, H, seed=77)
        L.set_cell_types(types)
        L.init_random(0.3, 0.2)
        L.set_forcing_column(5, 0.4)
        if chir is not None:
            L.set_chirality(chir)
        return L

    with fresh() as A:
        A.collide_and_propagate(17)
        A.apply_body_force(50, "x")
        blob = A.checkpoint()
        A.collide_and_propagate(23)
        A.apply_body_force(30, "y")
        want = A.download()
    with gpu.GpuLattice(model, W, H, seed=0) as B:
        B.restore(blob)
        assert B.step_count == 17
        B.collide_and_propagate(23)
        B.apply_body_force(30, "y")
        assert np.array_equal(B.download(), want)
        assert np.array_equal(B.get_cell_types(), types)
    with gpu.GpuLattice(model, W + 64, H) as C_:
        with pytest.raises(gpu.LgcaError):
            C_.restore(blob)


@pytest.mark.parametrize("W,H", [(64, 8), (130, 20), (777, 96), (1024, 512), (8192, 2048)])
def test_paint_reference_geometries(gpu, W, H):
    """Device painting gives the reference setters' cell maps exactly."""
    with gpu.GpuLattice(2, W, H) as L:
        L.apply_bc_pipe()
        assert np.array_equal(L.get_cell_types(), G.pipe(W, H))
        L.apply_bc_karman_vortex_street()
        assert np.array_equal(L.get_cell_types(), G.karman_reference(W, H))
        for bt in ("back", "forward"):
            L.apply_bc_reflecting(bt)
            assert np.array_equal(L.get_cell_types(), G.reflecting(W, H, bt))
        L.apply_bc_periodic()
        assert np.array_equal(L.get_cell_types(), G.periodic(W, H))


@pytest.mark.parametrize("W,H", [(100, 40), (777, 96), (2048, 1024)])
def test_paint_shapes_against_numpy(gpu, W, H):
    rng = np.random.default_rng(W + H)
    want = G.periodic(W, H)
    y, x = np.mgrid[0:H, 0:W]
    with gpu.GpuLattice(3, W, H) as L:
        for k in range(12):
            shape = int(rng.integers(3))
            t = int(rng.integers(3))
            a, b = int(rng.integers(-W // 4, W + W // 4)), int(rng.integers(-H // 4, H + H // 4))
            if shape == 0:
                c, d = a + int(rng.integers(0, W)), b + int(rng.integers(0, H))
                m = (x >= a) & (x < c) & (y >= b) & (y < d)
            elif shape == 1:
                c, d = int(rng.integers(0, H)), 0
                m = (x - a) ** 2 + (y - b) ** 2 < c * c
            else:
                c, d = int(rng.integers(0, H)), 0
                dist = np.sqrt(((x - a) ** 2 + (y - b) ** 2).astype(np.float64)).astype(np.float32)
                m = dist.astype(np.float64) < np.float64(np.float32(c)) / 2.0
            want[m] = t
            L.paint_cells(shape, t, a, b, c, d)
            assert np.array_equal(L.get_cell_types(), want), (k, shape, t, a, b, c, d)


def test_paint_then_step_matches_uploaded_map(gpu, oracle):
    """A painted lattice steps exactly like one given the same map from the
    host, and like the oracle."""
    W, H, model = 640, 128, 3
    types = G.disc(W, H, W // 8, H // 2, H // 8)
    st = oracle.init_bernoulli(model, W, H, types, seed=4, p_move=0.3, p_rest=0.3)
    out = []
    for painted in (True, False):
        with gpu.GpuLattice(model, W, H, seed=6) as L:
            if painted:
                L.apply_bc_pipe()
                L.paint_cells(gpu.SHAPE_DISC, gpu.SOLID_NO_SLIP, W // 8, H // 2, H // 8)
            else:
                L.set_cell_types(types)
            L.upload(st)
            L.set_forcing_column(16, 0.05)
            L.collide_and_propagate(40)
            out.append(L.download())
    assert np.array_equal(out[0], out[1])
    want = oracle.run(model, st, 40, types=types, seed=6, force_x=16, force_p=0.05)
    assert np.array_equal(out[0], want)


def test_paint_rejects_bad_arguments(gpu):
    with gpu.GpuLattice(1, 64, 8) as L:
        for args in [(3, 1, 0, 0, 1, 1), (0, 3, 0, 0, 1, 1), (0, -1, 0, 0, 1, 1),
                     (1, 1, 0, 0, -2, 0), (0, 1, 1 << 29, 0, 1, 1)]:
            with pytest.raises(gpu.LgcaError):
                L.paint_cells(*args)
        L.paint_cells(gpu.SHAPE_RECT, gpu.FLUID, 0, 0, 64, 8)  # no planes yet: nothing to do
        assert not L.get_cell_types().any()


@pytest.mark.parametrize("variant,W,H", [(4, 512, 256), (6, 512, 256), (6, 4096, 3648)])
def test_persistent_wait_timeout_marks_handle_failed_until_cleared(gpu, oracle, variant, W, H):
    """One block of the persistent (4) or resident (6) kernel withholds its
    progress (test hook),
    so its neighbours' bounded waits run out after the 1 ms limit.  Every call
    that waits for the handle then reports LGCA_ERR_TIMEOUT, and persistent
    calls queued behind the failure do not step, until lgca_clear_error; after
    a state is reloaded the handle steps correctly again.  4096 x 3648 runs
    the resident kernel with row barriers (FHP-III, bands of 24 warps), whose
    row waits give up once the edge warps' halo waits have."""
    model = 3
    st = oracle.init_bernoulli(model, W, H, None, seed=4, p_move=0.3, p_rest=0.3)
    with gpu.GpuLattice(model, W, H, seed=4) as L:
        L.upload(st)
        L.set_kernel_variant(variant)
        L.set_wait_limit(1_000_000)
        L.test_withhold_progress(1)
        L.collide_and_propagate(10)
        for call in (L.sync, L.download, L.count_particles, lambda: L.block_sums(16), L.checkpoint):
            with pytest.raises(gpu.LgcaError) as e:
                call()
            assert e.value.status == 4  # LGCA_ERR_TIMEOUT
        L.test_withhold_progress(-1)
        L.collide_and_propagate(10)  # a launch behind the failure returns without stepping
        with pytest.raises(gpu.LgcaError) as e:
            L.sync()
        assert e.value.status == 4
        L.clear_error()
        L.sync()
        L.upload(st)
        L.set_step(0)
        L.collide_and_propagate(10)
        assert np.array_equal(L.download(), oracle.run(model, st, 10, seed=4))
        with pytest.raises(gpu.LgcaError):
            L.set_wait_limit(10)  # below 1 us


def test_checkpoint_load_rejects_invalid_settings(gpu):
    """A damaged checkpoint header is refused before anything changes."""
    import struct
    with gpu.GpuLattice(1, 128, 16, seed=3) as L:
        L.init_random(0.3)
        blob = bytearray(L.checkpoint())
        want = L.download()
        # header: magic[8], model, dim_x, dim_y, flags (int32), seed, step,
        # fcall (uint64), force_x, depth (int32), force_thr (uint64), variant, wpt
        offsets = {"flags": 20, "force_x": 48, "depth": 52, "variant": 64, "wpt": 68}
        for field, bad in [("flags", 16), ("variant", 9), ("wpt", 3), ("depth", 0), ("depth", 9),
                           ("force_x", 128), ("force_x", 5)]:
            b = bytearray(blob)
            struct.pack_into("<i", b, offsets[field], bad)
            with pytest.raises(gpu.LgcaError):
                L.restore(bytes(b))
        assert np.array_equal(L.download(), want)
        L.restore(bytes(blob))
        assert np.array_equal(L.download(), want)


def test_job_and_fused_sum_calls_reject_bad_arguments(gpu):
    """The one-call job, the steps-with-sums call and the step plan refuse
    invalid arguments with a status, before queueing anything."""
    import ctypes as C
    lib = gpu.lib()
    with gpu.GpuLattice(3, 4096, 64, seed=1) as L:
        L.init_random(0.3)
        want = L.download()
        h = L._h
        assert lib.lgca_run_job_async(h, None, -1, None, 0, None, None, None) != 0
        assert lib.lgca_run_job_async(h, None, 4, None, -2, None, None, None) != 0
        assert lib.lgca_run_job_async(h, None, 4, None, 32, None, None, None) != 0  # sums NULL
        assert lib.lgca_collide_and_propagate_sums(h, 4, 0, None, None, None) != 0
        assert lib.lgca_collide_and_propagate_sums(h, -1, 32, None, None, None) != 0
        fam, n = C.c_int(), C.c_int()
        assert lib.lgca_step_plan(h, -3, C.byref(fam), C.byref(n)) != 0
        assert np.array_equal(L.download(), want) and L.step_count == 0
