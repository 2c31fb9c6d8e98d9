"""Batched lattices (lgca_batch_*): every member of a mixed batch -- models,
sizes (ragged widths included), geometries, forcing, frozen chirality and
different step counts -- ends with exactly the bits it reaches when stepped
alone, with and without CUDA graphs."""
import numpy as np
import pytest

from lgca_gb300 import geometry as G

pytestmark = pytest.mark.gpu

GEOMS = [lambda w, h: G.periodic(w, h), G.pipe, G.karman_reference,
         lambda w, h: G.reflecting(w, h, "forward"),
         lambda w, h: G.disc(w, h, w // 8, h // 2, max(1, h // 16))]


def make_jobs(gpu, n, rng, max_side=700):
    jobs = []
    for i in range(n):
        model = int(rng.integers(4))
        W = int(rng.choice([64, 100, 128, 192, 256, 300, 320, 512, 640, max_side]))
        H = 2 * int(rng.integers(2, max_side // 2))
        types = GEOMS[int(rng.integers(len(GEOMS)))](W, H)
        L = gpu.GpuLattice(model, W, H, seed=1000 + i)
        L.set_cell_types(types)
        L.init_random(float(rng.uniform(0.1, 0.4)), float(rng.uniform(0.1, 0.4)))
        if rng.random() < 0.5:
            L.set_forcing_column(int(rng.integers(W)), 0.05)
        if model > 0 and rng.random() < 0.2:
            L.set_chirality(rng.integers(0, 2, (H, W), dtype=np.uint8))
        L.set_step(int(rng.integers(0, 1000)))
        jobs.append(L)
    return jobs


@pytest.mark.parametrize("graph_steps,warp_tasks", [(0, 4), (8, 4), (32, 4), (0, 1), (32, 2),
                                                    (8, 8), (32, 0)])
def test_mixed_batch_equals_alone(gpu, graph_steps, warp_tasks):
    rng = np.random.default_rng(graph_steps + 1)
    jobs = make_jobs(gpu, 24, rng)
    steps = [int(x) for x in rng.integers(0, 90, len(jobs))]
    steps[0] = 90
    # reference: each lattice alone (its checkpoint restored into a twin)
    want = []
    for L, n in zip(jobs, steps):
        twin = gpu.GpuLattice(L.model, L.dim_x, L.dim_y)
        twin.restore(L.checkpoint())
        twin.collide_and_propagate(n)
        want.append((twin.download(), twin.step_count))
        twin.close()
    with gpu.GpuBatch(graph_steps=graph_steps) as B:
        B.set_persistent(graph_steps == 0)  # graphs belong to the one-launch-per-step form
        B.set_warp_tasks(warp_tasks)
        for L in jobs:
            B.add(L)
        B.step_each(steps)
        for L, (w, t) in zip(jobs, want):
            assert L.step_count == t
            assert np.array_equal(L.download(), w), (L.model, L.dim_x, L.dim_y)
    for L in jobs:
        L.close()


def test_batch_calls_interleave_with_member_calls(gpu, oracle):
    """Work queued on a member before a batch call runs first, and the member
    continues after it; several batch calls in a row; members removed."""
    W, H = 256, 48
    types = G.pipe(W, H)
    A = gpu.GpuLattice(3, W, H, seed=5)
    Bl = gpu.GpuLattice(1, 192, 30, seed=6)
    A.set_cell_types(types)
    st = oracle.init_bernoulli(3, W, H, types, seed=5, p_move=0.3, p_rest=0.3)
    A.upload(st)  # queued on A's stream, not yet synchronised
    A.set_forcing_column(9, 0.3)
    Bl.init_random(0.3)
    with gpu.GpuBatch(graph_steps=4) as B:
        B.add(A)
        B.add(Bl)
        B.step_each([10, 3])
        A.collide_and_propagate(5)  # member's own call after the batch
        B.step(12)
        B.remove(Bl)
        B.step(7)
    want = oracle.run(3, st, 34, types=types, seed=5, force_x=9, force_p=0.3)
    assert A.step_count == 34 and Bl.step_count == 15
    assert np.array_equal(A.download(), want)
    A.close()
    Bl.close()


def test_batch_ordering_with_long_queues(gpu):
    """Ordering between a member's own stream and batch calls with enough
    queued work on both sides that a missing dependency would show: a long
    run queued on a member before the batch call, block sums queued on it
    right after (they must see the batch's steps), more own steps, another
    batch call, and a stream fetched by the caller after a batch call."""
    import torch
    W, H = 4096, 2048
    A = gpu.GpuLattice(3, W, H, seed=21)
    S = gpu.GpuLattice(0, 512, 64, seed=22)
    A.init_random(0.3, 0.3)
    S.init_random(0.2)
    twin = gpu.GpuLattice(3, W, H, seed=21)
    twin.init_random(0.3, 0.3)
    A.collide_and_propagate(60)  # queued on A's stream, not synchronised
    n = np.zeros((3, H // 32, W // 32), dtype=np.int32)
    with gpu.GpuBatch(graph_steps=0) as B:
        B.add(A)
        B.add(S)
        B.step_each([40, 40])
        A.block_sums_async(32, n[0], n[1], n[2])  # after the batch's 40 steps
        A.collide_and_propagate(7)
        B.step(3)
        ev = torch.cuda.Event()
        ev.record(torch.cuda.ExternalStream(A.stream_ptr()))  # after the second call
        ev.synchronize()
        # the fetched stream waited for the whole second call
        assert torch.cuda.ExternalStream(B.stream_ptr()).query()
        got = A.download()
    twin.collide_and_propagate(100)
    n_want = twin.block_sums(32)
    twin.collide_and_propagate(10)
    assert np.array_equal(got, twin.download())
    for a, b in zip(n, n_want):
        assert np.array_equal(a, b)
    assert A.step_count == 110 and S.step_count == 43
    for L in (A, S, twin):
        L.close()


def test_batched_config_small_is_bit_exact_and_faster(gpu):
    """The batched workload generator at reduced scale: batched and
    one-at-a-time runs agree bit for bit (the full 512 x 1000 run is in the
    benchmark)."""
    from lgca_gb300 import batched
    r = batched.compare(n_jobs=24, steps=60, tune=True)
    assert r["bit_exact"]
    assert r["batched_gsite_updates_s"] > 0


def test_autotuner_single_lattice_choice_keeps_results(gpu, oracle):
    from lgca_gb300.autotune import Autotuner
    W, H = 1024, 96
    types = G.pipe(W, H)
    st = oracle.init_bernoulli(0, W, H, types, seed=2, p_move=0.3)
    L = gpu.GpuLattice(0, W, H, seed=2)
    L.set_cell_types(types)
    L.upload(st)
    L.set_forcing_column(8, 0.2)
    choice = Autotuner().tune_lattice(L, steps=8)
    assert choice[0] in (1, 2, 3, 5, 6)
    L.collide_and_propagate(40)
    want = oracle.run(0, st, 40, types=types, seed=2, force_x=8, force_p=0.2)
    assert np.array_equal(L.download(), want) and L.step_count == 40
    L.close()


def test_membership_rules(gpu):
    """A lattice joins at most one batch; closing a member removes it from
    its batch, whose other members keep stepping correctly."""
    a = gpu.GpuLattice(1, 128, 8, seed=1)
    b = gpu.GpuLattice(1, 128, 8, seed=2)
    for L in (a, b):
        L.init_random(0.3, 0.3)
    want = []
    twin = gpu.GpuLattice(1, 128, 8, seed=2)
    twin.restore(b.checkpoint())
    twin.collide_and_propagate(5)
    want = twin.download()
    twin.close()
    with gpu.GpuBatch() as B1, gpu.GpuBatch() as B2:
        B1.add(a)
        B1.add(b)
        with pytest.raises(gpu.LgcaError):
            B2.add(a)  # already in B1
        with pytest.raises(gpu.LgcaError):
            B1.add(a)  # twice
        a.close()  # leaves B1
        assert B1.members == [b]
        B1.step(5)
        assert np.array_equal(b.download(), want)
    b.close()


@pytest.mark.parametrize("graph_steps", [0, 32])
def test_batch_with_wavefront_members_equals_alone(gpu, graph_steps):
    """Members on the register wavefront (kernel variant 2, depth 2, 4 or 8)
    run their single steps with the others and then passes of K steps; mixed
    with one-step members, every member equals its lone run."""
    rng = np.random.default_rng(100 + graph_steps)
    jobs = make_jobs(gpu, 20, rng, max_side=900)
    for i, (model, W, H) in enumerate([(0, 3200, 200), (1, 2048, 130), (3, 1984, 96)]):
        # several strips of 30 words per row, several slabs
        L = gpu.GpuLattice(model, W, H, seed=77 + i)
        L.set_cell_types(GEOMS[i](W, H))
        L.init_random(0.3, 0.3)
        L.set_forcing_column(int(rng.integers(W)), 0.05)
        jobs.append(L)
    depths = []
    for L in jobs:
        K = int(rng.choice([1, 2, 4, 8]))
        if K > 1:
            L.set_kernel_variant(2)
            L.set_temporal_depth(K)
        depths.append(K)
    steps = [int(x) for x in rng.integers(0, 150, len(jobs))]
    steps[0] = 150
    want = []
    for L, n in zip(jobs, steps):
        twin = gpu.GpuLattice(L.model, L.dim_x, L.dim_y)
        twin.restore(L.checkpoint())
        twin.set_kernel_variant(1)  # one step per pass, one word per lane
        twin.collide_and_propagate(n)
        want.append((twin.download(), twin.step_count))
        twin.close()
    with gpu.GpuBatch(graph_steps=graph_steps) as B:
        for L in jobs:
            B.add(L)
        B.step_each(steps)
        for L, (w, t), K in zip(jobs, want, depths):
            assert L.step_count == t
            assert np.array_equal(L.download(), w), (L.model, L.dim_x, L.dim_y, K)
        # a second call continues from the first on every path
        B.step_each([7] * len(jobs))
    for L in jobs:
        L.close()


@pytest.mark.parametrize("warp_tasks", [1, 2, 4])
def test_persistent_batch_equals_alone(gpu, warp_tasks):
    """The persistent form (one cooperative launch per stretch of steps with
    an unchanged member set, a grid barrier between steps) gives every member
    the bits of its lone run, also when members leave part way."""
    rng = np.random.default_rng(200 + warp_tasks)
    jobs = make_jobs(gpu, 24, rng)
    steps = [int(x) for x in rng.integers(0, 90, len(jobs))]
    steps[0] = 90
    want = []
    for L, n in zip(jobs, steps):
        twin = gpu.GpuLattice(L.model, L.dim_x, L.dim_y)
        twin.restore(L.checkpoint())
        twin.collide_and_propagate(n)
        want.append(twin.download())
        twin.close()
    with gpu.GpuBatch() as B:
        B.set_persistent(True)
        B.set_warp_tasks(warp_tasks)
        for L in jobs:
            B.add(L)
        B.step_each(steps)
        B.sync()
        for L, w in zip(jobs, want):
            assert np.array_equal(L.download(), w), (L.model, L.dim_x, L.dim_y)
    for L in jobs:
        L.close()


def test_batched_workload_equals_oracle(gpu):
    """The batched workload at full size -- 512 lattices of 256..4096 x
    256..4096 sites, the four models, periodic / pipe with forcing / disc,
    1000 steps -- run as one batch with the autotuned kernels: every job's
    final state equals its lone oracle run (hashes in the fixture)."""
    from conftest import load_json
    from lgca_gb300 import batched as BT
    g = load_json("batched_512.json")
    assert g["engine"] == "port"
    jobs = BT.make_jobs(512)
    assert jobs == g["jobs"] and g["steps"] == 1000
    _, hashes, _ = BT.run_batched(jobs, 1000, tune=True)
    bad = [i for i, (a, b) in enumerate(zip(hashes, g["final_sha"])) if a != b]
    assert len(hashes) == 512 and not bad, bad[:10]
