"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs the unmodified reference OMP_Lattice (keva92/lgca src/lattice.cpp,
src/omp_lattice.cpp) through the hook harness oracle/ref_harness.cpp, built
from the reference sources by `make -C oracle ref`.  Needs the reference
checkout that oracle/oracle.py names (LGCA_REFERENCE_DIR); the fixtures it
writes are committed so that the tests run without it.

    python tests/golden/gen_golden.py            # small fixtures (seconds)
    python tests/golden/gen_golden.py --configs  # + full-size workload pins (minutes)
    python tests/golden/gen_golden.py --karman-long ref  # Karman workload, 10000 steps (about 50 min)
    python tests/golden/gen_golden.py --batched  # batched workload, 512 jobs x 1000 steps (about 90 min)
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from lgca_gb300 import geometry as G  # noqa: E402

MODELS = [O.HPP, O.FHP_I, O.FHP_II, O.FHP_III]


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def geometry(name, W, H):
    if name == "periodic":
        return G.periodic(W, H)
    if name == "pipe":
        return G.pipe(W, H)
    if name == "karman":
        return G.karman_reference(W, H)
    if name == "reflecting_back":
        return G.reflecting(W, H, "back")
    if name == "reflecting_forward":
        return G.reflecting(W, H, "forward")
    if name.startswith("disc"):
        return G.disc(W, H, W // 4, H // 2, max(2, H // 5))
    raise ValueError(name)


# (model, W, H, geometry, seed, p_move, p_rest, force_x, force_p, steps, chirality)
TRAJ_CASES = []
for m in MODELS:
    TRAJ_CASES += [
        (m, 64, 32, "periodic", 11, 0.3, 0.3, -1, 0.0, 40, "counter"),
        (m, 128, 64, "pipe", 12, 0.2, 0.25, 8, 0.05, 60, "counter"),
        (m, 96, 48, "karman", 13, 0.3, 0.3, 16, 0.1, 50, "counter"),
        (m, 70, 20, "reflecting_forward", 14, 0.35, 0.2, 0, 0.3, 45, "counter"),
        (m, 130, 18, "reflecting_back", 15, 0.25, 0.5, 129, 0.5, 45, "counter"),
        (m, 200, 22, "disc", 16, 0.3, 0.1, 63, 0.2, 30, "counter"),
        (m, 66, 16, "periodic", 17, 0.5, 0.5, -1, 0.0, 25, "frozen"),
        (m, 3, 4, "periodic", 18, 0.5, 0.5, 1, 0.5, 20, "counter"),
    ]


def gen_small():
    # exhaustive collision tables
    tables = {}
    for m in MODELS:
        D = O.NUM_DIR[m]
        tables[f"m{m}"] = np.array([[O.ref_collide(m, s, p) for s in range(1 << D)] for p in (0, 1)],
                                   np.uint8)
    np.savez_compressed(os.path.join(HERE, "collide_tables.npz"), **tables)

    # trajectories
    traj = {}
    meta = []
    rng = np.random.default_rng(2024)
    for i, (m, W, H, geom, seed, pm, pr, fx, fp, steps, chmode) in enumerate(TRAJ_CASES):
        types = geometry(geom, W, H)
        state = O.init_bernoulli(m, W, H, types, seed=seed, p_move=pm, p_rest=pr)
        chir = rng.integers(0, 2, (H, W), dtype=np.uint8) if chmode == "frozen" else None
        final = O.ref_run(m, state, steps, types=types, seed=seed, t0=0, chir=chir, force_x=fx,
                          force_p=fp)
        traj[f"c{i}_types"] = types.astype(np.int8)
        traj[f"c{i}_init"] = state
        traj[f"c{i}_final"] = final
        if chir is not None:
            traj[f"c{i}_chir"] = chir
        meta.append(dict(model=m, W=W, H=H, geometry=geom, seed=seed, p_move=pm, p_rest=pr,
                         force_x=fx, force_p=fp, steps=steps, chirality=chmode))
    np.savez_compressed(os.path.join(HERE, "trajectories.npz"), **traj)
    with open(os.path.join(HERE, "trajectories.json"), "w") as f:
        json.dump(meta, f, indent=1)

    # post-processing (cell + coarse, reference FP32 arithmetic)
    pp = {}
    for m in MODELS:
        for (W, H, r) in [(64, 32, 4), (80, 40, 5), (48, 24, 8), (24, 16, 8)]:
            st = O.init_bernoulli(m, W, H, None, seed=21 + W, p_move=0.4, p_rest=0.3)
            cd, cm, md, mm = O.ref_post_process(m, st, r)
            k = f"m{m}_{W}x{H}_r{r}"
            pp[k + "_state"] = st
            pp[k + "_cd"], pp[k + "_cm"], pp[k + "_md"], pp[k + "_mm"] = cd, cm, md, mm
    np.savez_compressed(os.path.join(HERE, "postprocess.npz"), **pp)

    # random-cell body force
    bf = {}
    bmeta = []
    for m in MODELS:
        for (geom, direction, forcing) in [("pipe", "x", 40), ("pipe", "x", 0), ("periodic", "y", 25),
                                           ("karman", "x", 100000), ("pipe", "y", -1)]:
            W, H = 96, 48
            types = geometry(geom, W, H)
            st = O.init_bernoulli(m, W, H, types, seed=31, p_move=0.3, p_rest=0.3)
            out = O.ref_apply_body_force(m, st, forcing, types=types, seed=5, call=7, bf_dir=direction)
            k = f"b{len(bmeta)}"
            bf[k + "_init"], bf[k + "_final"] = st, out
            bmeta.append(dict(model=m, geometry=geom, dir=direction, forcing=forcing, seed=5, call=7,
                              W=W, H=H))
    np.savez_compressed(os.path.join(HERE, "bodyforce.npz"), **bf)
    with open(os.path.join(HERE, "bodyforce.json"), "w") as f:
        json.dump(bmeta, f, indent=1)

    # lattice parameters derived by the reference constructor
    dims = []
    for m in MODELS:
        for (tc, Re, Ma, r) in [("pipe", 80.0, 0.3, 10), ("karman", 80.0, 0.3, 10),
                                ("diffusion", 500.0, 0.2, 8), ("periodic", 1020.0, 0.3, 8),
                                ("periodic", 1024.0, 0.3, 8), ("box", 200.0, 0.3, 1),
                                ("pipe", 250.0, 0.25, 8)]:
            d = O.ref_dims(m, tc, Re, Ma, r)
            d.update(model=m, test_case=tc, Re=Re, Ma=Ma, r=r)
            dims.append(d)
    # init_single_collision (src/lattice.cpp:283-294)
    sc = {f"m{m}": O.ref_init(m, 34, 8, "single_collision") for m in MODELS}
    np.savez_compressed(os.path.join(HERE, "single_collision.npz"), **sc)
    # get_mean_velocity of the reference, one thread (its fluid-cell counter is
    # incremented inside a parallel loop without being a reduction variable)
    mv = subprocess.run([sys.executable, __file__, "--mean-velocity"], capture_output=True,
                        text=True, env={**os.environ, "OMP_NUM_THREADS": "1"}, check=True)
    with open(os.path.join(HERE, "params.json"), "w") as f:
        json.dump({"dims": dims, "mean_velocity": json.loads(mv.stdout)}, f, indent=1)


def mean_velocity_cases():
    out = []
    for m in MODELS:
        W, H = 64, 32
        types = G.pipe(W, H)
        st = O.init_bernoulli(m, W, H, types, seed=41, p_move=0.3, p_rest=0.3)
        st = O.ref_run(m, st, 10, types=types, seed=41, force_x=5, force_p=0.5)
        ux, uy = O.ref_mean_velocity(m, st, types)
        out.append(dict(model=m, W=W, H=H, seed=41, steps=10, force_x=5, force_p=0.5, ux=ux, uy=uy,
                        state_sha=sha(st)))
    return out


def gen_configs():
    """Pins of the two full-size workloads (reference run, minutes)."""
    pins = {}
    # FHP-I pipe 1024x512, Bernoulli 0.2 seed 1, forcing x=8 p=0.01, 1000 steps, 16x16 sums
    W, H = 1024, 512
    types = G.pipe(W, H)
    st = O.init_bernoulli(O.FHP_I, W, H, types, seed=1, p_move=0.2, p_rest=0.2)
    fin = O.ref_run(O.FHP_I, st, 1000, types=types, seed=1, force_x=8, force_p=0.01)
    N, Jx2, Jy = O.block_sums(O.FHP_I, fin, 16)
    pins["pipe_fhp1_1024x512"] = dict(init_sha=sha(st), final_sha=sha(fin), steps=1000,
                                      particles=int(O.count_particles(fin)))
    np.savez_compressed(os.path.join(HERE, "config_pipe_blocksums.npz"), N=N, Jx2=Jx2, Jy=Jy)
    # FHP-III Karman 8192x2048, disc r=128 at (1024,1024), forcing x=16 p=0.02,
    # Bernoulli 0.3 seed 2; reference run for 200 steps, 32x32 sums at 100 and 200
    W, H = 8192, 2048
    types = G.disc(W, H, 1024, 1024, 128)
    st = O.init_bernoulli(O.FHP_III, W, H, types, seed=2, p_move=0.3, p_rest=0.3)
    s100 = O.ref_run(O.FHP_III, st, 100, types=types, seed=2, t0=0, force_x=16, force_p=0.02)
    s200 = O.ref_run(O.FHP_III, s100, 100, types=types, seed=2, t0=100, force_x=16, force_p=0.02)
    sums = {}
    for tag, s in (("t100", s100), ("t200", s200)):
        N, Jx2, Jy = O.block_sums(O.FHP_III, s, 32)
        sums[f"{tag}_N"], sums[f"{tag}_Jx2"], sums[f"{tag}_Jy"] = N, Jx2, Jy
    np.savez_compressed(os.path.join(HERE, "config_karman_blocksums.npz"), **sums)
    pins["karman_fhp3_8192x2048"] = dict(init_sha=sha(st), t100_sha=sha(s100), t200_sha=sha(s200),
                                         types_sha=sha(types))
    with open(os.path.join(HERE, "config_pins.json"), "w") as f:
        json.dump(pins, f, indent=1)


def blocksum_sha(N, Jx2, Jy) -> str:
    """One hash over the three int32 block-sum arrays, in the order N, Jx2, Jy."""
    return sha(np.stack([np.asarray(N, np.int32), np.asarray(Jx2, np.int32),
                         np.asarray(Jy, np.int32)]))


def gen_karman_long(engine: str = "ref", steps: int = 10000):
    """The Karman workload over its whole run: FHP-III 8192x2048, disc r=128 at
    (1024,1024), forcing column x=16 p=0.02, Bernoulli 0.3 seed 2.  Records the
    hash of the 32x32 block sums every 100 steps and of the state every 1000
    steps.  engine "ref" steps the reference OMP_Lattice (about 50 minutes on 8
    cores), "port" the restatement (about 8 minutes)."""
    import time
    W, H = 8192, 2048
    types = G.disc(W, H, 1024, 1024, 128)
    st = O.init_bernoulli(O.FHP_III, W, H, types, seed=2, p_move=0.3, p_rest=0.3)
    run = O.ref_run if engine == "ref" else O.run
    out = dict(engine=engine, W=W, H=H, steps=steps, block=32, init_sha=sha(st),
               blocksum_sha={}, blocksum_total=[], state_sha={})
    s = st
    t_start = time.time()
    for t in range(0, steps, 100):
        s = run(O.FHP_III, s, 100, types=types, seed=2, t0=t, force_x=16, force_p=0.02)
        N, Jx2, Jy = O.block_sums(O.FHP_III, s, 32)
        out["blocksum_sha"][str(t + 100)] = blocksum_sha(N, Jx2, Jy)
        out["blocksum_total"].append([int(N.sum()), int(Jx2.sum()), int(Jy.sum())])
        if (t + 100) % 1000 == 0:
            out["state_sha"][str(t + 100)] = sha(s)
        print(f"step {t + 100}: {time.time() - t_start:.0f} s", flush=True)
    name = "config_karman_long.json" if engine == "ref" else "config_karman_long_port.json"
    with open(os.path.join(HERE, name), "w") as f:
        json.dump(out, f, indent=1)
    return out


def batched_job_types(job):
    """Cell map of a batched-workload job, as lgca_gb300.batched.build paints it."""
    W, H = job["W"], job["H"]
    if job["geometry"] == "pipe":
        return G.pipe(W, H)
    if job["geometry"] == "disc":
        return G.disc(W, H, W // 8, H // 2, max(1, H // 16), walls=False)
    return G.periodic(W, H)


def gen_batched(n_jobs: int = 512, steps: int = 1000):
    """Final-state hashes of every job of the batched workload (512 lattices,
    1000 steps each), stepped one by one through the restatement (pinned to
    the reference by the other fixtures).  About an hour on 8 cores."""
    import time
    from lgca_gb300.batched import make_jobs
    jobs = make_jobs(n_jobs)
    out = dict(engine="port", steps=steps, jobs=jobs, init_sha=[], final_sha=[])
    t_start = time.time()
    for j in jobs:
        types = batched_job_types(j)
        st = O.init_bernoulli(j["model"], j["W"], j["H"], types, seed=j["seed"], p_move=j["p"],
                              p_rest=j["p"])
        pipe = j["geometry"] == "pipe"
        fin = O.run(j["model"], st, steps, types=types, seed=j["seed"],
                    force_x=8 if pipe else -1, force_p=0.01 if pipe else 0.0)
        out["init_sha"].append(sha(st))
        out["final_sha"].append(sha(fin))
        print(f"job {j['index']} ({j['W']}x{j['H']}): {time.time() - t_start:.0f} s", flush=True)
    with open(os.path.join(HERE, "batched_512.json"), "w") as f:
        json.dump(out, f, indent=0)
    return out


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--configs", action="store_true")
    ap.add_argument("--batched", action="store_true")
    ap.add_argument("--karman-long", choices=["ref", "port"])
    ap.add_argument("--mean-velocity", action="store_true")
    args = ap.parse_args()
    O.build(ref=True)
    if args.mean_velocity:
        print(json.dumps(mean_velocity_cases()))
        sys.exit(0)
    if args.karman_long:
        gen_karman_long(args.karman_long)
        sys.exit(0)
    if args.batched:
        gen_batched()
        sys.exit(0)
    gen_small()
    if args.configs:
        gen_configs()
    print("fixtures written to", HERE)
