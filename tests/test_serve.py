"""Serving loop.  CPU tests drive the scheduler with a fake backend and a
simulated clock: admission against the memory budget, rejection of jobs that
can never fit, a failing allocation (host-side fault injection), output
cadence, latency accounting and the FCFS baseline.  The GPU test runs a short
served stream and checks that sampled jobs give the same fields alone."""
import numpy as np
import pytest

from lgca_gb300 import serve as S


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def sleep(self, dt):
        self.t += dt


class FakeBackend:
    """Counts steps; each step call costs 1 ms of simulated time per 1e6
    site-steps; create can be made to fail."""

    def __init__(self, clock, fail_first=()):
        self.clock, self.fail = clock, set(fail_first)
        self.live, self.peak_live, self.created = set(), 0, []

    def create(self, job):
        if job.index in self.fail:
            self.fail.discard(job.index)
            raise MemoryError("injected allocation failure")
        h = {"job": job.index, "steps": 0, "sites": job.sites}
        self.live.add(job.index)
        self.peak_live = max(self.peak_live, len(self.live))
        self.created.append(job.index)
        return h

    def step(self, handles, nsteps):
        work = 0
        for h, n in zip(handles, nsteps):
            h["steps"] += n
            work += n * h["sites"]
        self.clock.t += 1e-3 * work / 1e6 + 1e-4

    def fields(self, h):
        return (h["steps"],)

    def destroy(self, h):
        self.live.discard(h["job"])

    def evict(self, h):
        self.destroy(h)
        return dict(h)  # the "checkpoint": the handle's state

    def resume(self, job, blob):
        h = dict(blob)
        self.live.add(job.index)
        return h


def jobs_small(n=40, rate=200.0, seed=1):
    return S.make_jobs(rate, 10.0, rng_seed=seed, w_range=(64, 512), h_range=(64, 512),
                       steps_range=(10, 3000), max_jobs=n)


def test_budget_admission_and_completion():
    clock = FakeClock()
    be = FakeBackend(clock)
    jobs = jobs_small()
    budget = 3 * max(S.lattice_bytes(j.model, j.W, j.H, j.geometry) for j in jobs)
    srv = S.Server(be, budget=budget, clock=clock, sleep=clock.sleep)
    used_max = [0]
    orig = srv._admit

    def admit(now):
        orig(now)
        used_max[0] = max(used_max[0], srv.used)
        assert srv.used <= budget

    srv._admit = admit
    rep = srv.run(jobs)
    assert rep["completed"] == len(jobs) and rep["rejected"] == 0 and rep["backlog"] == 0
    assert used_max[0] <= budget and srv.used == 0 and not be.live
    for j in jobs:
        assert j.done_steps == j.steps
        assert j.outputs == -(-j.steps // 500)  # every 500 steps and at the end
        assert j.last_fields == (j.steps,)
        assert j.finished >= j.arrival and j.admitted >= j.arrival
    assert rep["p99_latency_s"] >= rep["p50_latency_s"] > 0


def test_site_slots_bound_the_resident_set():
    clock = FakeClock()
    jobs = jobs_small(40)
    cap = 2 * max(j.sites for j in jobs)
    srv = S.Server(FakeBackend(clock), budget=1e12, clock=clock, sleep=clock.sleep,
                   max_sites=cap)
    seen = [0]
    orig = srv._admit

    def admit(now):
        orig(now)
        assert srv.sites == sum(j.sites for j in srv.active)
        assert len(srv.active) <= 1 or srv.sites <= cap
        seen[0] = max(seen[0], len(srv.active))

    srv._admit = admit
    rep = srv.run(jobs)
    assert rep["completed"] == len(jobs) and seen[0] >= 2 and srv.sites == 0


def test_srpt_evicts_and_resumes_without_losing_steps():
    """Least-remaining-work admission with eviction: big residents are
    checkpointed out when much smaller jobs wait, and come back later; every
    job still does exactly its steps, and small jobs finish sooner."""
    def run(policy):
        clock = FakeClock()
        jobs = S.make_jobs(400.0, 2.0, rng_seed=9, w_range=(64, 1024), h_range=(64, 512),
                           steps_range=(10, 5000), max_jobs=120)
        cap = 3 * max(j.sites for j in jobs)
        srv = S.Server(FakeBackend(clock), budget=1e12, clock=clock, sleep=clock.sleep,
                       max_sites=cap, policy=policy)
        return srv.run(jobs), jobs, srv
    rep_f, jobs_f, _ = run("fcfs")
    rep_s, jobs_s, srv = run("srpt")
    assert rep_s["completed"] == len(jobs_s) and srv.evictions > 0 and srv.sites == 0
    for j in jobs_s:
        assert j.done_steps == j.steps and j.last_fields == (j.steps,)
        assert j.outputs >= -(-j.steps // 500) and j.ckpt is None
    assert rep_s["p50_latency_s"] < rep_f["p50_latency_s"]


def test_sampled_jobs_log_every_output():
    """Jobs marked before the run keep the hash of every field they stream,
    in step order; unmarked jobs keep none."""
    jobs = jobs_small(20, seed=9)
    pick = S.mark_sample(jobs, 6, seed=3)
    assert len(pick) == 6 and all(j.record for j in pick)
    assert all(j.arrival <= 0.5 * max(x.arrival for x in jobs) for j in pick)
    clock = FakeClock()
    S.Server(FakeBackend(clock), budget=1e12, clock=clock, sleep=clock.sleep).run(jobs)
    for j in jobs:
        if j.record:
            steps = [at for at, _ in j.field_log]
            assert steps == sorted(steps) and steps[-1] == j.steps and len(steps) == j.outputs
            assert all(h == S.fields_sha((at,)) for at, h in j.field_log)
        else:
            assert j.field_log == []


def test_unknown_policy_is_rejected():
    with pytest.raises(ValueError):
        S.Server(FakeBackend(FakeClock()), policy="lifo")


def test_job_larger_than_budget_is_rejected():
    clock = FakeClock()
    jobs = jobs_small(5)
    big = max(jobs, key=lambda j: j.sites)
    budget = S.lattice_bytes(big.model, big.W, big.H, big.geometry) - 1
    rep = S.Server(FakeBackend(clock), budget=budget, clock=clock, sleep=clock.sleep).run(jobs)
    assert rep["rejected"] >= 1 and rep["completed"] + rep["rejected"] == len(jobs)


def test_failed_allocation_is_retried():
    clock = FakeClock()
    jobs = jobs_small(12)
    be = FakeBackend(clock, fail_first={3, 7})
    rep = S.Server(be, budget=1e12, clock=clock, sleep=clock.sleep).run(jobs)
    assert rep["completed"] + rep["rejected"] == len(jobs)
    assert be.created.count(3) <= 1 and be.created.count(7) <= 1


def test_fcfs_baseline_queueing():
    jobs = [S.Job(index=i, arrival=float(i), model=0, W=64, H=64, geometry="periodic", p=0.2,
                  steps=100, seed=i) for i in range(3)]
    base = S.fcfs_baseline(jobs, lambda j: 0.02)  # 2 s per job, arrivals 1 s apart
    assert base["makespan_s"] == pytest.approx(6.0)
    assert base["p50_latency_s"] == pytest.approx(3.0)


def test_step_time_table_statistics():
    """A job's per-step time: the median (or fastest) repeat of the grid
    points of its model, geometry class, word-count parity and kernel family, as time per
    site interpolated in (log W, log H) by inverse squared distance (the
    table's points are set by hand; measuring them needs a GPU)."""
    t = object.__new__(S.StepTimeTable)
    t.stat = "median"
    fam = {}
    t.plan = lambda m, W, H, n: (fam.get((W, H), 1), n)
    pts = [(256, 256, 1, "periodic", [3e-6, 1e-6, 2e-6]),     # 2e-6 s per step at 65536 sites
           (1024, 256, 1, "periodic", [8e-6, 16e-6, 32e-6]),  # 16e-6 at 262144
           (320, 256, 1, "periodic", [1.0, 1.0, 1.0]),        # odd word count: other points
           (1024, 1024, 6, "periodic", [4e-6, 4e-6, 4e-6]),   # another kernel family
           (256, 256, 1, "walls", [5.0, 5.0, 5.0])]           # pipe and disc jobs
    t.samples = {m: pts for m in range(4)}
    job = lambda W, H: S.Job(index=0, arrival=0.0, model=2, W=W, H=H, geometry="periodic", p=0.2,
                             steps=10, seed=0)
    assert t(job(256, 256)) == pytest.approx(2e-6)  # on a point: that point
    assert t.with_stat("best")(job(256, 256)) == pytest.approx(1e-6)
    assert t.stat == "median"
    # halfway in log W between the two family-1 points of even word count:
    # the per-site times' geometric mean (2e-6/65536 and 16e-6/262144)
    want = ((2e-6 / 65536) * (16e-6 / 262144)) ** 0.5 * 512 * 256
    assert t(job(512, 256)) == pytest.approx(want)
    # the same shape on the resident path reads only family-6 points
    fam[(512, 256)] = 6
    t._families = {}
    assert t(job(512, 256)) == pytest.approx(4e-6 / (1024 * 1024) * 512 * 256)
    # an odd word count reads only the odd-width points
    assert t(job(320, 256)) == pytest.approx(1.0)
    # a job with walls or an obstacle reads the points with walls
    disc = S.Job(index=1, arrival=0.0, model=2, W=256, H=256, geometry="disc", p=0.2, steps=10,
                 seed=1)
    assert t(disc) == pytest.approx(5.0)
    # per-job costs: set-up plus one field copy per output, interpolated by sites
    j = job(100, 100)
    assert t.job_overhead(j, 3) == 0.0  # no measured costs
    t.costs = {m: [(1000, 1e-3, 1e-5), (100000, 1e-1, 1e-3)] for m in range(4)}
    assert t.job_overhead(j, 3) == pytest.approx(1e-2 + 3 * 1e-4)
    base = S.fcfs_baseline([job(256, 256)], t)  # 10 steps + set-up + one output
    assert base["makespan_s"] == pytest.approx(10 * 2e-6 + t.job_overhead(job(256, 256), 1))


def test_job_stream_shapes():
    jobs = S.make_jobs(100.0, 5.0, rng_seed=3)
    assert all(j.W % 64 == 0 and j.H % 64 == 0 and 256 <= j.W <= 8192 and 256 <= j.H <= 4096
               for j in jobs)
    assert all(100 <= j.steps <= 20000 for j in jobs)
    assert [j.seed for j in jobs] == list(range(len(jobs)))
    assert 300 < len(jobs) < 700


class PipelinedFake(FakeBackend):
    """Field requests return tokens collected later, as on the GPU; logs the
    order of step calls and collections."""

    def __init__(self, clock):
        super().__init__(clock)
        self.log = []

    def step(self, handles, nsteps):
        super().step(handles, nsteps)
        self.log.append("step")

    def request_fields(self, handles):
        return [(h["steps"],) for h in handles]  # values as of the request

    def collect(self, token):
        self.log.append("collect")
        return token


def test_pipelined_backend_overlaps_and_gives_same_results():
    jobs_a, jobs_b = jobs_small(30, seed=4), jobs_small(30, seed=4)
    clock = FakeClock()
    plain = S.Server(FakeBackend(clock), budget=1e12, clock=clock, sleep=clock.sleep).run(jobs_a)
    clock2 = FakeClock()
    be = PipelinedFake(clock2)
    piped = S.Server(be, budget=1e12, clock=clock2, sleep=clock2.sleep).run(jobs_b)
    assert piped["completed"] == plain["completed"] == len(jobs_a)
    for a, b in zip(jobs_a, jobs_b):
        assert a.last_fields == b.last_fields == (a.steps,)
        assert a.outputs == b.outputs
    # a call's fields are collected after the next call was queued (two calls
    # outstanding), except when nothing else was runnable
    outstanding, two = 0, 0
    for e in be.log:
        if e == "step":
            outstanding += 1
        else:
            assert outstanding in (1, 2)
            two += outstanding == 2
            outstanding -= 1
    assert two >= 0.8 * be.log.count("collect")


@pytest.mark.gpu
def test_short_served_stream_is_bit_exact(gpu):
    jobs = S.make_jobs(40.0, 1.5, rng_seed=11, w_range=(256, 1024), h_range=(256, 512),
                       steps_range=(100, 1500))
    for j in jobs:
        j.record = True  # log every streamed field
    backend = S.GpuBackend()
    srv = S.Server(backend, budget=20e9)
    rep = srv.run(jobs)
    backend.close()
    assert rep["completed"] == len(jobs)
    assert all(j.outputs == -(-j.steps // 500) == len(j.field_log) for j in jobs)
    # every job rebuilt from a host map, every one of its outputs compared
    v = S.verify_sample(srv.done, n=len(srv.done))
    assert v["bit_exact"] and v["jobs"] == len(jobs)
    assert v["fields"] == sum(j.outputs for j in jobs)


@pytest.mark.gpu
def test_evicted_and_resumed_jobs_are_bit_exact(gpu):
    """With least-remaining-work admission and a small site cap, residents
    are checkpointed out and resumed; every job's final fields still equal
    its lone run."""
    # arrivals far above capacity with room for one lattice at a time: small
    # newcomers displace big residents while the stream arrives
    jobs = S.make_jobs(2000.0, 0.15, rng_seed=12, w_range=(256, 1024), h_range=(256, 512),
                       steps_range=(100, 3000))
    for j in jobs:
        j.record = True
    backend = S.GpuBackend()
    srv = S.Server(backend, budget=20e9, max_sites=1024 * 512, policy="srpt", preempt_ratio=0.5)
    rep = srv.run(jobs)
    backend.close()
    assert rep["completed"] == len(jobs) and srv.evictions > 0
    # the outputs streamed before and after each eviction, all compared
    v = S.verify_sample(srv.done, n=len(srv.done))
    assert v["bit_exact"] and v["fields"] == sum(j.outputs for j in jobs)


@pytest.mark.gpu
def test_backend_evict_resume_round_trip(gpu):
    """Evict mid-run (checkpoint to host, lattice freed), resume into a new
    lattice, finish: the fields equal an uninterrupted run."""
    job = S.Job(index=7, arrival=0.0, model=3, W=640, H=384, geometry="disc", p=0.3, steps=700,
                seed=7)
    backend = S.GpuBackend()
    h = backend.create(job)
    backend.step([h], [300])
    blob = backend.evict(h)
    h2 = backend.resume(job, blob)
    backend.step([h2], [400])
    got = backend.fields(h2)
    backend.destroy(h2)
    backend.close()
    L = S.build_alone(job)
    L.collide_and_propagate(700)
    want = L.block_sums(16)
    L.close()
    assert all(np.array_equal(a, b) for a, b in zip(got, want))
