"""CPU tests of the oracle: the C restatement (oracle/lgca_oracle.c) against
the golden fixtures generated from the reference, and -- where the reference
sources are present -- against the compiled reference itself."""
import hashlib

import numpy as np
import pytest

from conftest import load_json, load_npz
from lgca_gb300 import geometry as G
from lgca_gb300 import params as P

MODELS = [0, 1, 2, 3]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("model", MODELS)
def test_collide_tables_match_golden(oracle, model):
    t = load_npz("collide_tables.npz")[f"m{model}"]
    D = oracle.NUM_DIR[model]
    mine = np.array([[oracle.collide(model, s, p) & ((1 << D) - 1) for s in range(1 << D)]
                     for p in (0, 1)], np.uint8)
    assert np.array_equal(mine, t)


def test_fhp3_equals_fhp2(oracle):
    for s in range(128):
        for p in (0, 1):
            assert oracle.collide(2, s, p) == oracle.collide(3, s, p)


def test_collisions_conserve_mass_and_momentum(oracle):
    vx = {0: [2, 0, -2, 0], 1: [2, 1, -1, -2, -1, 1]}
    vy = {0: [0, 1, 0, -1], 1: [0, 1, 1, 0, -1, -1]}
    for m in MODELS:
        D = oracle.NUM_DIR[m]
        k = 0 if m == 0 else 1
        for s in range(1 << D):
            for p in (0, 1):
                o = oracle.collide(m, s, p)
                bits = lambda v: [(v >> d) & 1 for d in range(D)]
                assert sum(bits(s)) == sum(bits(o))
                for v in (vx[k], vy[k]):
                    assert sum(a * b for a, b in zip(bits(s)[:len(v)], v)) == \
                           sum(a * b for a, b in zip(bits(o)[:len(v)], v))


def _traj_case(i, c, npz):
    types = npz[f"c{i}_types"].astype(np.int32)
    init = npz[f"c{i}_init"]
    final = npz[f"c{i}_final"]
    chir = npz[f"c{i}_chir"] if f"c{i}_chir" in npz.files else None
    return types, init, final, chir


def test_trajectories_match_golden(oracle):
    meta = load_json("trajectories.json")
    npz = load_npz("trajectories.npz")
    for i, c in enumerate(meta):
        types, init, final, chir = _traj_case(i, c, npz)
        # the initial states were drawn by the oracle's INIT stream
        again = oracle.init_bernoulli(c["model"], c["W"], c["H"], types, seed=c["seed"],
                                      p_move=c["p_move"], p_rest=c["p_rest"])
        assert np.array_equal(again, init), c
        out = oracle.run(c["model"], init, c["steps"], types=types, seed=c["seed"], chir=chir,
                         force_x=c["force_x"], force_p=c["force_p"])
        assert np.array_equal(out, final), c


def test_postprocess_match_golden(oracle):
    npz = load_npz("postprocess.npz")
    keys = sorted({k.rsplit("_", 1)[0] for k in npz.files})
    assert keys
    for k in keys:
        m = int(k[1])
        r = int(k.rsplit("_r", 1)[1])
        got = oracle.post_process(m, npz[k + "_state"], r)
        for name, g in zip(("cd", "cm", "md", "mm"), got):
            want = npz[f"{k}_{name}"]
            assert g.shape == want.shape
            assert np.array_equal(g.view(np.uint32), want.view(np.uint32)), (k, name)


def test_bodyforce_match_golden(oracle):
    meta = load_json("bodyforce.json")
    npz = load_npz("bodyforce.npz")
    for i, c in enumerate(meta):
        types = {"pipe": G.pipe, "periodic": G.periodic, "karman": G.karman_reference}[c["geometry"]](
            c["W"], c["H"])
        out, n = oracle.apply_body_force(c["model"], npz[f"b{i}_init"], c["forcing"], types=types,
                                         seed=c["seed"], call=c["call"], bf_dir=c["dir"])
        assert np.array_equal(out, npz[f"b{i}_final"]), c
        assert oracle.count_particles(out) == oracle.count_particles(npz[f"b{i}_init"])


def test_mean_velocity_matches_single_thread_reference(oracle):
    for c in load_json("params.json")["mean_velocity"]:
        types = G.pipe(c["W"], c["H"])
        st = oracle.init_bernoulli(c["model"], c["W"], c["H"], types, seed=c["seed"], p_move=0.3,
                                   p_rest=0.3)
        st = oracle.run(c["model"], st, c["steps"], types=types, seed=c["seed"],
                        force_x=c["force_x"], force_p=c["force_p"])
        assert sha(st) == c["state_sha"]
        ux, uy = oracle.mean_velocity(c["model"], st, types)
        assert ux == pytest.approx(c["ux"], rel=1e-5, abs=1e-7)
        assert uy == pytest.approx(c["uy"], rel=1e-5, abs=1e-7)


def test_lattice_parameters_match_reference_constructor():
    for d in load_json("params.json")["dims"]:
        p = P.lattice_parameters(d["model"], d["test_case"], d["Re"], d["Ma"], d["r"])
        for k in ("dim_x", "dim_y", "coarse_dim_x", "coarse_dim_y", "initial_forcing",
                  "equilibrium_forcing", "bf_dir"):
            assert p[k] == d[k], (k, d, p)
        for k in ("nu_s", "c_s", "u"):
            assert np.float32(p[k]) == np.float32(d[k]), (k, d, p)


def test_single_collision_matches_reference():
    npz = load_npz("single_collision.npz")
    for m in MODELS:
        assert np.array_equal(P.init_single_collision(m, 34, 8), npz[f"m{m}"])


def test_mass_conservation_without_forcing(oracle):
    for m in MODELS:
        for geom in (G.periodic, G.pipe, lambda W, H: G.reflecting(W, H, "forward")):
            W, H = 96, 40
            types = geom(W, H)
            st = oracle.init_bernoulli(m, W, H, types, seed=3, p_move=0.35, p_rest=0.2)
            out = oracle.run(m, st, 30, types=types, seed=3)
            assert oracle.count_particles(out) == oracle.count_particles(st)


def test_block_sums_totals(oracle):
    st = oracle.init_bernoulli(2, 100, 50, None, seed=9, p_move=0.4)
    N, Jx2, Jy = oracle.block_sums(2, st, 16)
    assert N.shape == (4, 7)
    assert int(N.sum()) == oracle.count_particles(st)


def test_config_pipe_pin(oracle):
    pins = load_json("config_pins.json")["pipe_fhp1_1024x512"]
    W, H = 1024, 512
    types = G.pipe(W, H)
    st = oracle.init_bernoulli(1, W, H, types, seed=1, p_move=0.2, p_rest=0.2)
    assert sha(st) == pins["init_sha"]
    fin = oracle.run(1, st, pins["steps"], types=types, seed=1, force_x=8, force_p=0.01)
    assert sha(fin) == pins["final_sha"]
    N, Jx2, Jy = oracle.block_sums(1, fin, 16)
    g = load_npz("config_pipe_blocksums.npz")
    assert np.array_equal(N, g["N"]) and np.array_equal(Jx2, g["Jx2"]) and np.array_equal(Jy, g["Jy"])


def test_batched_fixture_matches_workload_and_oracle(oracle):
    """The batched-workload fixture lists exactly the jobs the batched form
    builds, and its hashes are the oracle's: the smallest job of each model
    and geometry is re-run here for the full 1000 steps."""
    from lgca_gb300 import batched as BT
    g = load_json("batched_512.json")
    jobs = BT.make_jobs(512)
    assert g["jobs"] == jobs and g["steps"] == 1000 and len(g["final_sha"]) == 512
    smallest = {}
    for j in jobs:
        k = (j["model"], j["geometry"])
        if k not in smallest or j["W"] * j["H"] < smallest[k]["W"] * smallest[k]["H"]:
            smallest[k] = j
    assert len(smallest) >= 8
    for j in sorted(smallest.values(), key=lambda j: j["W"] * j["H"])[:8]:
        W, H = j["W"], j["H"]
        types = (G.pipe(W, H) if j["geometry"] == "pipe" else
                 G.disc(W, H, W // 8, H // 2, max(1, H // 16), walls=False)
                 if j["geometry"] == "disc" else G.periodic(W, H))
        st = oracle.init_bernoulli(j["model"], j["W"], j["H"], types, seed=j["seed"],
                                   p_move=j["p"], p_rest=j["p"])
        assert sha(st) == g["init_sha"][j["index"]]
        pipe = j["geometry"] == "pipe"
        fin = oracle.run(j["model"], st, 1000, types=types, seed=j["seed"],
                         force_x=8 if pipe else -1, force_p=0.01 if pipe else 0.0)
        assert sha(fin) == g["final_sha"][j["index"]], j


# ----------------------------------------------- against the compiled reference
@pytest.mark.parametrize("model", MODELS)
def test_restatement_equals_reference_random_cases(ref, model):
    rng = np.random.default_rng(100 + model)
    for _ in range(6):
        W = int(rng.integers(2, 150))
        H = 2 * int(rng.integers(1, 20))
        geom = rng.choice(["periodic", "pipe", "karman", "reflecting_back", "reflecting_forward"])
        types = ref.ref_geometry(model, W, H, str(geom))
        st = ref.init_bernoulli(model, W, H, types, seed=int(rng.integers(1 << 30)),
                                p_move=float(rng.uniform(0.05, 0.6)), p_rest=float(rng.uniform(0, 1)))
        fx = int(rng.integers(-1, W))
        kw = dict(types=types, seed=int(rng.integers(1 << 40)), t0=int(rng.integers(0, 1000)),
                  force_x=fx, force_p=float(rng.uniform(0, 1)))
        steps = int(rng.integers(1, 30))
        assert np.array_equal(ref.run(model, st, steps, **kw), ref.ref_run(model, st, steps, **kw))


def test_geometry_setters_equal_reference(ref):
    for m in MODELS:
        for (W, H) in [(64, 32), (90, 30), (7, 6)]:
            assert np.array_equal(G.periodic(W, H), ref.ref_geometry(m, W, H, "periodic"))
            assert np.array_equal(G.pipe(W, H), ref.ref_geometry(m, W, H, "pipe"))
            assert np.array_equal(G.karman_reference(W, H), ref.ref_geometry(m, W, H, "karman"))
            assert np.array_equal(G.reflecting(W, H, "back"), ref.ref_geometry(m, W, H, "reflecting_back"))
            assert np.array_equal(G.reflecting(W, H, "forward"),
                                  ref.ref_geometry(m, W, H, "reflecting_forward"))


def test_postprocess_and_bodyforce_equal_reference(ref):
    rng = np.random.default_rng(7)
    for m in MODELS:
        W, H, r = 60, 30, 3
        st = ref.init_bernoulli(m, W, H, None, seed=5, p_move=0.45)
        for a, b in zip(ref.post_process(m, st, r), ref.ref_post_process(m, st, r)):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
        types = G.pipe(W, H)
        for d in ("x", "y", None):
            f = int(rng.integers(-2, 200))
            call = int(rng.integers(9))
            a, _ = ref.apply_body_force(m, st, f, types=types, seed=3, call=call, bf_dir=d)
            b = ref.ref_apply_body_force(m, st, f, types=types, seed=3, call=call, bf_dir=d)
            assert np.array_equal(a, b)


def test_karman_long_run_port_equals_reference():
    """The oracle's restatement and the compiled reference, each run over the
    whole Karman workload (FHP-III 8192x2048, 10000 steps; tests/golden/
    gen_golden.py --karman-long ref|port), agree on every 32x32 block-sum set
    (every 100 steps) and every state hash (every 1000 steps)."""
    ref = load_json("config_karman_long.json")
    port = load_json("config_karman_long_port.json")
    assert ref["engine"] == "ref" and port["engine"] == "port"
    assert len(ref["blocksum_sha"]) == 100 and len(ref["state_sha"]) == 10
    for k in ("W", "H", "steps", "block", "init_sha", "blocksum_sha", "blocksum_total", "state_sha"):
        assert port[k] == ref[k], k
