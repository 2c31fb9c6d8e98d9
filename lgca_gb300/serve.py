"""Serving loop: simulation jobs arrive over time, are admitted as device
memory frees up, run together (continuous batching: every resident lattice
advances in the same batched launches, jobs join and leave between batch
calls), stream back coarse-grained fields, and report latency.

Job stream (defaults): Poisson arrivals at `rate` jobs/s for `duration` s;
model, geometry and occupation as the batched workload; width log-uniform in
[256, 8192] and height in [256, 4096] (multiples of 64); steps log-uniform in
[100, 20000]; seed = arrival index.  Every `out_every` steps (and at the end)
a job returns its 16 x 16 integer block sums (N, Jx2, Jy).  Admission keeps
the resident lattices' device bytes within `budget` (150 GB) and their sites
within `max_sites` (slots), in one of two orders: first come, first served
("fcfs"), or least remaining work first ("srpt"), where a waiting job with a
small fraction of a resident's remaining work evicts that resident -- its
state is checkpointed to host memory and restored later, bit-exactly.

The scheduler (Server) talks to a backend: GpuBackend runs the engine;
tests substitute a CPU fake to exercise admission, budgets and failures.

    python -m lgca_gb300.serve --rate 50 --duration 60
"""
from __future__ import annotations

import argparse
import hashlib
import heapq
import json
import math
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

GEOMETRIES = ("periodic", "pipe", "disc")


@dataclass
class Job:
    index: int
    arrival: float
    model: int
    W: int
    H: int
    geometry: str
    p: float
    steps: int
    seed: int
    done_steps: int = 0
    admitted: float | None = None
    finished: float | None = None
    outputs: int = 0
    last_fields: tuple | None = None
    handle: object = None
    error: str | None = None
    bytes: int = 0
    ckpt: bytes | None = None  # state of an evicted job, restored on resume
    evictions: int = 0
    # sampled jobs keep (step, hash of the fields) of every output they stream
    record: bool = False
    field_log: list = field(default_factory=list)

    @property
    def sites(self) -> int:
        return self.W * self.H

    @property
    def remaining(self) -> int:
        """Site updates still to do."""
        return (self.steps - self.done_steps) * self.sites

    def next_event(self, out_every: int) -> int:
        """Steps to the next output or the end."""
        to_out = out_every - (self.done_steps % out_every)
        return min(to_out, self.steps - self.done_steps)


def fields_sha(fields) -> str:
    """Hash of one streamed output: the N, Jx2, Jy block-sum arrays in order."""
    h = hashlib.sha256()
    for a in fields:
        h.update(np.ascontiguousarray(a, dtype=np.int32).tobytes())
    return h.hexdigest()


def _round64(v: float) -> int:
    return max(64, int(round(v / 64.0)) * 64)


def make_jobs(rate: float, duration: float, rng_seed: int = 5, w_range=(256, 8192),
              h_range=(256, 4096), steps_range=(100, 20000), max_jobs: int | None = None):
    rng = np.random.default_rng(rng_seed)
    t, jobs = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration or (max_jobs is not None and len(jobs) >= max_jobs):
            break
        i = len(jobs)
        lu = lambda lo, hi: math.exp(rng.uniform(math.log(lo), math.log(hi)))
        jobs.append(Job(index=i, arrival=t, model=int(rng.integers(4)),
                        W=_round64(lu(*w_range)), H=_round64(lu(*h_range)),
                        geometry=GEOMETRIES[int(rng.integers(3))],
                        p=float(rng.uniform(0.1, 0.4)),
                        steps=int(round(lu(*steps_range))), seed=i))
    return jobs


def lattice_bytes(model: int, W: int, H: int, geometry: str, block: int = 16) -> int:
    """Device bytes of a served lattice: two state buffers, the geometry planes
    when there are walls or obstacles, and the block-sum outputs (geometry is
    painted on the device, so there is no cell-map staging)."""
    D = {0: 4, 1: 6, 2: 7, 3: 7}[model]
    nw = (W + 63) // 64
    pitch = nw + (nw & 1)
    plane = H * pitch * 8
    geo = 2 * plane if geometry != "periodic" else 0
    sums = 3 * 4 * (-(-W // block)) * (-(-H // block))
    return 2 * D * plane + geo + sums + 4096


class GpuBackend:
    """Runs jobs on the GPU through the C ABI (one batch for all residents).

    Nothing here waits for the device except `collect`: geometry is painted
    on the device, lattice memory comes from the engine's stream-ordered pool,
    batch steps and field copies are queued, and a field request is tracked
    by one event per job, so the host prepares the next batch call while the
    device runs the current one."""

    def __init__(self, block: int = 16):
        import torch
        import lgca_gb300 as gpu
        self.gpu, self.torch, self.block = gpu, torch, block
        self.batch = gpu.GpuBatch()
        self.out = {}  # (handle id, parity) -> pinned (3, Hb, Wb) int32 buffers
        self.parity = {}

    def create(self, job: Job):
        gpu = self.gpu
        L = gpu.GpuLattice(job.model, job.W, job.H, seed=job.seed)
        if job.geometry == "pipe":
            L.apply_bc_pipe()
            L.set_forcing_column(8, 0.01)
        elif job.geometry == "disc":
            L.paint_cells(gpu.SHAPE_DISC, gpu.SOLID_NO_SLIP, job.W // 8, job.H // 2,
                          max(1, job.H // 16))
        L.init_random(job.p, job.p)
        self.batch.add(L)
        return L

    def step(self, handles, nsteps):
        # members not in `handles` do not step
        counts = {id(h): n for h, n in zip(handles, nsteps)}
        self.batch.step_each([counts.get(id(m), 0) for m in self.batch.members])

    def _buffers(self, handle):
        par = self.parity.get(id(handle), 0)
        self.parity[id(handle)] = par ^ 1  # consecutive requests use different buffers
        key = (id(handle), par)
        if key not in self.out:
            Hb, Wb = -(-handle.dim_y // self.block), -(-handle.dim_x // self.block)
            self.out[key] = self.torch.empty((3, Hb, Wb), dtype=self.torch.int32,
                                             pin_memory=True).numpy()
        return self.out[key]

    def request_fields(self, handles):
        """Queue every job's block sums into pinned buffers; returns a token."""
        token = []
        for h in handles:
            b = self._buffers(h)
            h.block_sums_async(self.block, b[0], b[1], b[2])
            ev = self.torch.cuda.Event()
            ev.record(self.torch.cuda.ExternalStream(h.stream_ptr()))
            token.append((ev, b))
        return token

    def collect(self, token):
        out = []
        for ev, b in token:
            ev.synchronize()
            out.append((b[0].copy(), b[1].copy(), b[2].copy()))
        return out

    def fields(self, handle):
        return self.collect(self.request_fields([handle]))[0]

    def destroy(self, handle):
        self.batch.remove(handle)
        self.out.pop((id(handle), 0), None)
        self.out.pop((id(handle), 1), None)
        self.parity.pop(id(handle), None)
        handle.close()

    def evict(self, handle) -> bytes:
        """Checkpoint a resident lattice to host memory and free it (its
        queued steps and field copies complete first, in stream order)."""
        blob = handle.checkpoint()
        self.destroy(handle)
        return blob

    def resume(self, job: Job, blob: bytes):
        L = self.gpu.GpuLattice(job.model, job.W, job.H, seed=job.seed)
        L.restore(blob)
        self.batch.add(L)
        return L

    def close(self):
        self.batch.close()


class _Queue:
    """Waiting jobs: first come, first served ("fcfs"), or least remaining
    work first ("srpt", ties by arrival)."""

    def __init__(self, policy: str):
        if policy not in ("fcfs", "srpt"):
            raise ValueError(f"unknown policy {policy!r}")
        self.policy = policy
        self.q = deque() if policy == "fcfs" else []

    def push(self, job: Job) -> None:
        if self.policy == "fcfs":
            self.q.append(job)
        else:
            heapq.heappush(self.q, (job.remaining, job.arrival, job.index, job))

    def push_front(self, job: Job) -> None:
        if self.policy == "fcfs":
            self.q.appendleft(job)
        else:
            self.push(job)

    def peek(self) -> Job:
        return self.q[0] if self.policy == "fcfs" else self.q[0][3]

    def pop(self) -> Job:
        return self.q.popleft() if self.policy == "fcfs" else heapq.heappop(self.q)[3]

    def jobs(self):
        return list(self.q) if self.policy == "fcfs" else [e[3] for e in self.q]

    def clear(self) -> None:
        self.q.clear()

    def __len__(self) -> int:
        return len(self.q)


class Server:
    def __init__(self, backend, budget: float = 150e9, out_every: int = 500,
                 clock=time.perf_counter, sleep=time.sleep, max_quantum: int = 100,
                 max_sites: float = float("inf"), policy: str = "fcfs",
                 preempt_ratio: float = 0.25, max_evictions: int = 4):
        self.backend, self.budget, self.out_every = backend, budget, out_every
        self.clock, self.sleep, self.max_quantum = clock, sleep, max_quantum
        # slots: residents' total sites; beyond what fills the device, more
        # residents only share it more thinly (longer latency, same throughput)
        self.max_sites = max_sites
        # "srpt": admit the least remaining work first, and when a waiting
        # job has under preempt_ratio of a resident's remaining work and no
        # slot is free, evict that resident (checkpoint to host, resume later
        # bit-exactly); at most max_evictions per admission pass
        self.policy, self.preempt_ratio, self.max_evictions = policy, preempt_ratio, max_evictions
        self.used = 0
        self.sites = 0
        self.evictions = 0
        self.active: list[Job] = []
        self.waiting = _Queue(policy)
        self.done: list[Job] = []
        self.rejected: list[Job] = []
        self.site_updates = 0
        self.batch_calls = 0

    def _admit(self, now: float) -> None:
        # in queue order; a job that never fits is rejected
        evicted = 0
        while self.waiting:
            job = self.waiting.peek()
            need = lattice_bytes(job.model, job.W, job.H, job.geometry)
            if need > self.budget:
                self.waiting.pop()
                job.error = "larger than the memory budget"
                self.rejected.append(job)
                continue
            fits = self.used + need <= self.budget and not (
                self.active and self.sites + job.sites > self.max_sites)
            if not fits:
                if self.policy == "srpt" and evicted < self.max_evictions and self.active:
                    victim = max(self.active, key=lambda j: j.remaining)
                    if victim.remaining * self.preempt_ratio > job.remaining:
                        self._evict(victim)
                        evicted += 1
                        continue
                return
            self.waiting.pop()
            try:
                if job.ckpt is not None:
                    job.handle = self.backend.resume(job, job.ckpt)
                else:
                    job.handle = self.backend.create(job)
            except Exception as e:  # allocation failure: retry once memory frees
                job.error = f"create failed: {e}"
                if not self.active:
                    self.rejected.append(job)
                else:
                    self.waiting.push_front(job)
                return
            job.ckpt = None
            job.error = None
            job.bytes = need
            if job.admitted is None:
                job.admitted = now
            self.used += need
            self.sites += job.sites
            self.active.append(job)

    def _evict(self, job: Job) -> None:
        job.ckpt = self.backend.evict(job.handle)
        job.handle = None
        job.evictions += 1
        self.evictions += 1
        self.used -= job.bytes
        self.sites -= job.sites
        self.active.remove(job)
        self.waiting.push(job)

    def _finish(self, job: Job, now: float) -> None:
        job.finished = now
        self.backend.destroy(job.handle)
        job.handle = None
        self.used -= job.bytes
        self.sites -= job.sites
        self.active.remove(job)
        self.done.append(job)

    def _request(self, handles):
        req = getattr(self.backend, "request_fields", None)
        return req(handles) if req else [self.backend.fields(h) for h in handles]

    def _collect(self, token):
        col = getattr(self.backend, "collect", None)
        return col(token) if col else token

    def run(self, jobs, drain_limit: float = float("inf")) -> dict:
        """Continuous batching, pipelined one call deep: call k's steps and
        field copies are queued before call k-1's fields are collected, so
        the device does not idle while the host admits, finishes and plans."""
        pending = sorted(jobs, key=lambda j: j.arrival)
        t0 = self.clock()
        k = 0
        last_arrival = pending[-1].arrival if pending else 0.0
        inflight = None  # (token, jobs whose fields it carries)
        while k < len(pending) or self.waiting or self.active or inflight:
            now = self.clock() - t0
            while k < len(pending) and pending[k].arrival <= now:
                self.waiting.push(pending[k])
                k += 1
            self._admit(now)
            if now > last_arrival + drain_limit and inflight is None:
                break
            launched = None
            run = [j for j in self.active if j.done_steps < j.steps]
            if run and now <= last_arrival + drain_limit:
                # every runnable job advances to its next output, its end or a quantum
                n = [min(j.next_event(self.out_every), self.max_quantum) for j in run]
                self.backend.step([j.handle for j in run], n)
                self.batch_calls += 1
                emit = []
                for j, s in zip(run, n):
                    j.done_steps += s
                    self.site_updates += s * j.sites
                    if j.done_steps % self.out_every == 0 or j.done_steps == j.steps:
                        emit.append((j, j.done_steps))
                launched = (self._request([j.handle for j, _ in emit]), emit)
            if inflight is not None:
                token, emit = inflight
                got = self._collect(token)
                now = self.clock() - t0
                for (j, at), f in zip(emit, got):
                    j.last_fields = f
                    j.outputs += 1
                    if j.record:
                        j.field_log.append((at, fields_sha(f)))
                    if at == j.steps:
                        self._finish(j, now)
            inflight = launched
            if inflight is None and not self.active:
                self._admit(now)  # the jobs just finished freed their slots
                if self.active:
                    continue
                if k < len(pending):  # idle until the next arrival
                    self.sleep(max(0.0, pending[k].arrival - now))
                elif self.waiting:  # nothing resident and nothing admissible
                    left = self.waiting.jobs()
                    for j in left:
                        j.error = j.error or "could not be admitted"
                    self.rejected.extend(left)
                    self.waiting.clear()
        elapsed = self.clock() - t0
        return self.report(jobs, elapsed)

    def report(self, jobs, elapsed: float) -> dict:
        lat = np.array([j.finished - j.arrival for j in self.done]) if self.done else np.zeros(0)
        return {
            "jobs": len(jobs), "completed": len(self.done), "rejected": len(self.rejected),
            "backlog": len(jobs) - len(self.done) - len(self.rejected),
            "elapsed_s": elapsed, "site_updates": self.site_updates,
            "sustained_gsite_updates_s": self.site_updates / elapsed / 1e9 if elapsed else 0.0,
            "p50_latency_s": float(np.percentile(lat, 50)) if lat.size else None,
            "p99_latency_s": float(np.percentile(lat, 99)) if lat.size else None,
            "batch_calls": self.batch_calls, "policy": self.policy, "evictions": self.evictions,
        }


def fcfs_baseline(jobs, step_time, out_every: int = 500) -> dict:
    """First-come-first-served single-lattice execution of the same jobs: one
    job at a time, each taking steps * step_time(job) seconds (step times of
    the plain kernel measured on the GPU) plus, when step_time measured them,
    the job's own costs -- creating and initialising its lattice once and
    copying its fields back every out_every steps and at its end -- with
    queueing simulated exactly."""
    overhead = getattr(step_time, "job_overhead", None)
    t, lat, busy = 0.0, [], 0.0
    for j in sorted(jobs, key=lambda j: j.arrival):
        start = max(t, j.arrival)
        service = j.steps * step_time(j)
        if overhead is not None:
            service += overhead(j, -(-j.steps // out_every))
        t = start + service
        busy += service
        lat.append(t - j.arrival)
    lat = np.array(lat)
    total = sum(j.steps * j.sites for j in jobs)
    return {"p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "makespan_s": t, "sustained_gsite_updates_s": total / t / 1e9 if t else 0.0}


class StepTimeTable:
    """Per-step time of single-lattice execution by (model, W, H), measured on
    the GPU, and the per-job costs around the steps.

    Grid: widths 256 .. 8192 by powers of two, and the same widths plus 64
    (8128 for the last), whose odd word counts take the one-step kernel's
    padded last pair and never the resident kernel; heights 256 .. 4096 by
    powers of two; two geometry classes, periodic and walls (pipe walls and a
    forcing column, standing for the pipe and disc jobs, whose solid plane is
    read alike).  Each point is a lattice of that shape and class run alone
    with the automatic kernel choice in calls of `steps` steps (500: the
    calls of the FCFS run between field outputs), `repeats` times, wall clock
    with launches; it records the kernel family its calls take.  A job's
    per-step time comes from the points of its model, geometry class,
    word-count parity and kernel family (the family `plan` gives for its
    shape, lgca_plan_shape by default): the time per site interpolated in
    (log W, log H) by inverse squared distance over the nearest four such
    points, or the point itself when the job's shape is on the grid.  `stat`
    "median" uses the median repeat of each point, "best" the fastest.

    Set-up (create, pipe walls painted, occupation drawn, waited for) and one
    field output (16 x 16 block sums copied to the host) are measured on the
    shapes W x max(256, W / 2) of the power-of-two widths and interpolated by
    site count."""

    WIDTHS = (256, 512, 1024, 2048, 4096, 8192)
    HEIGHTS = (256, 512, 1024, 2048, 4096)

    def __init__(self, steps: int = 500, repeats: int = 3, stat: str = "median", plan=None):
        import lgca_gb300 as gpu
        self.stat = stat
        self.plan = plan
        # model -> [(W, H, family, geometry class, [seconds per step of each repeat])]
        self.samples = {}
        self.costs = {}    # model -> [(sites, setup seconds, output seconds)]
        widths = self.WIDTHS + tuple(min(w + 64, 8128) for w in self.WIDTHS)
        for m in range(4):
            pts = []
            for geo, W, H in ((geo, W, H) for geo in ("periodic", "walls") for W in widths
                              for H in self.HEIGHTS):
                L = gpu.GpuLattice(m, W, H, seed=1)
                if geo == "walls":
                    L.apply_bc_pipe()
                    L.set_forcing_column(8, 0.01)
                L.init_random(0.25, 0.25)
                fam = L.step_plan(steps)[0]
                L.collide_and_propagate(steps)
                L.sync()
                reps = []
                for _ in range(repeats):
                    t0 = time.perf_counter()
                    L.collide_and_propagate(steps)
                    L.sync()
                    reps.append((time.perf_counter() - t0) / steps)
                pts.append((W, H, fam, geo, reps))
                L.close()
            self.samples[m] = pts
            costs = []
            for W in self.WIDTHS:
                H = max(256, W // 2)
                setup = []
                for _ in range(repeats):
                    t0 = time.perf_counter()
                    L = gpu.GpuLattice(m, W, H, seed=1)
                    L.apply_bc_pipe()
                    L.init_random(0.25, 0.25)
                    L.sync()
                    setup.append(time.perf_counter() - t0)
                    L.close()
                L = gpu.GpuLattice(m, W, H, seed=1)
                L.init_random(0.25, 0.25)
                L.block_sums(16)
                out = []
                for _ in range(repeats):
                    t0 = time.perf_counter()
                    L.block_sums(16)
                    out.append(time.perf_counter() - t0)
                L.close()
                costs.append((W * H, float(np.median(setup)), float(np.median(out))))
            self.costs[m] = costs

    def with_stat(self, stat: str) -> "StepTimeTable":
        """The same samples read with another statistic."""
        other = object.__new__(StepTimeTable)
        other.__dict__.update(self.__dict__)
        other.stat = stat
        return other

    def family(self, job: Job) -> int:
        """The kernel family of the job's calls when run alone."""
        plan = getattr(self, "plan", None)
        if plan is None:
            import lgca_gb300 as gpu
            plan = gpu.plan_shape
        key = (job.model, job.W, job.H, min(500, job.steps))
        cache = self.__dict__.setdefault("_families", {})
        if key not in cache:
            cache[key] = plan(*key)[0]
        return cache[key]

    def __call__(self, job: Job) -> float:
        f = np.min if self.stat == "best" else np.median
        odd = (job.W // 64) % 2
        geo = "periodic" if job.geometry == "periodic" else "walls"
        pts = [p for p in self.samples[job.model] if (p[0] // 64) % 2 == odd and p[3] == geo]
        same = [p for p in pts if p[2] == self.family(job)]
        pts = same or pts or self.samples[job.model]
        lw, lh = math.log(job.W), math.log(job.H)
        near = sorted(((math.log(p[0]) - lw) ** 2 + (math.log(p[1]) - lh) ** 2, i)
                      for i, p in enumerate(pts))[:4]
        near = [(d, pts[i]) for d, i in near]
        per_site = lambda p: float(f(p[4])) / (p[0] * p[1])
        if near[0][0] < 1e-12:
            return per_site(near[0][1]) * job.sites
        wts = [1.0 / d for d, _ in near]
        log_ps = sum(w * math.log(per_site(p)) for w, (_, p) in zip(wts, near)) / sum(wts)
        return math.exp(log_ps) * job.sites

    def job_overhead(self, job: Job, outputs: int) -> float:
        """Seconds a job spends outside its steps when run alone: set-up and
        `outputs` field copies (0 without measured costs)."""
        costs = getattr(self, "costs", {}).get(job.model)
        if not costs:
            return 0.0
        xs = np.log([c[0] for c in costs])
        setup = float(np.exp(np.interp(math.log(job.sites), xs, np.log([c[1] for c in costs]))))
        out = float(np.exp(np.interp(math.log(job.sites), xs, np.log([c[2] for c in costs]))))
        return setup + outputs * out


def build_alone(job: Job):
    """The job as a lone lattice, its geometry given as a host cell map (the
    other construction path from the served one, which paints on the device)."""
    import lgca_gb300 as gpu
    from lgca_gb300 import geometry as G
    L = gpu.GpuLattice(job.model, job.W, job.H, seed=job.seed)
    if job.geometry == "pipe":
        L.set_cell_types(G.pipe(job.W, job.H))
        L.set_forcing_column(8, 0.01)
    elif job.geometry == "disc":
        L.set_cell_types(G.disc(job.W, job.H, job.W // 8, job.H // 2, max(1, job.H // 16),
                                walls=False))
    L.init_random(job.p, job.p)
    return L


def mark_sample(jobs, n: int = 16, seed: int = 0, horizon: float = 0.5):
    """Choose n jobs to verify before the run (so that every field they stream
    is logged): drawn without replacement from the jobs that arrive in the
    first `horizon` of the stream, which are the ones most likely to be
    served within the run."""
    if not jobs or n <= 0:
        return []
    t_end = max(j.arrival for j in jobs)
    pool = [j for j in jobs if j.arrival <= horizon * t_end] or list(jobs)
    rng = np.random.default_rng(seed)
    pick = [pool[i] for i in rng.choice(len(pool), size=min(n, len(pool)), replace=False)]
    for j in pick:
        j.record = True
    return pick


def verify_sample(jobs, n: int = 8, block: int = 16) -> dict:
    """Rerun up to n sampled jobs (marked before the run) alone through the
    plain kernel in another code path (host cell map, one word per lane),
    stopping at every step where the served job streamed fields: each of
    those outputs, not only the last, must have the same block sums."""
    sample = [j for j in jobs if j.record and j.field_log][:n]
    fields = 0
    ok = True
    for j in sample:
        L = build_alone(j)
        L.set_kernel_variant(1)  # one word per lane: another code path than the batch's
        done = 0
        for at, want in j.field_log:
            L.collide_and_propagate(at - done)
            done = at
            ok &= fields_sha(L.block_sums(block)) == want
            fields += 1
        L.close()
    return {"jobs": len(sample), "fields": fields, "bit_exact": bool(ok and sample)}


def fcfs_measured(jobs, n: int = 200, block: int = 16, out_every: int = 500) -> dict:
    """The first n jobs of the stream run first come, first served, one at a
    time through the plain kernel on the GPU: each is created as the served
    form creates it (device-painted geometry), stepped with its block sums
    copied to the host every out_every steps and at its end, and destroyed.
    Measures the service rate of FCFS execution directly (wall clock)."""
    import lgca_gb300 as gpu
    sel = sorted(jobs, key=lambda j: j.arrival)[:n]
    t0 = time.perf_counter()
    work = 0
    for j in sel:
        L = gpu.GpuLattice(j.model, j.W, j.H, seed=j.seed)
        if j.geometry == "pipe":
            L.apply_bc_pipe()
            L.set_forcing_column(8, 0.01)
        elif j.geometry == "disc":
            L.paint_cells(gpu.SHAPE_DISC, gpu.SOLID_NO_SLIP, j.W // 8, j.H // 2, max(1, j.H // 16))
        L.init_random(j.p, j.p)
        L.set_kernel_variant(0)  # the plain kernel: one step per pass, its fastest form
        done = 0
        while done < j.steps:
            k = min(out_every - done % out_every, j.steps - done)
            L.collide_and_propagate(k)
            done += k
            L.block_sums(block)
        work += j.steps * j.sites
        L.close()
    dt = time.perf_counter() - t0
    return {"jobs": len(sel), "site_updates": work, "seconds": dt,
            "gsite_updates_s": work / dt / 1e9 if dt else 0.0}


# resident-site slots of the served runs: 2^30 sites keep a 100-step batch
# call near 30 ms on the GPU; at full load they gave 1.7 % more throughput
# than 2^29 at the same latency
SERVE_MAX_SITES = float(1 << 30)


def serve(rate: float, duration: float, budget: float = 150e9, drain_limit: float = 60.0,
          verify: int = 8, fcfs: bool = True, max_sites: float = SERVE_MAX_SITES,
          quantum: int = 100, policy: str = "fcfs", fcfs_sample: int = 0, **job_kw) -> dict:
    jobs = make_jobs(rate, duration, **job_kw)
    if verify:
        mark_sample(jobs, 2 * verify)
    backend = GpuBackend()
    srv = Server(backend, budget=budget, max_sites=max_sites, max_quantum=quantum, policy=policy)
    rep = srv.run(jobs, drain_limit=drain_limit)
    backend.close()
    rep.update(rate=rate, duration=duration, max_sites=max_sites, quantum=quantum)
    if fcfs:
        table = StepTimeTable()
        base = fcfs_baseline(jobs, table)
        rep["fcfs"] = base
        if rep["p50_latency_s"] and base["p50_latency_s"]:
            rep["p50_speedup_vs_fcfs"] = base["p50_latency_s"] / rep["p50_latency_s"]
        rep["throughput_speedup_vs_fcfs"] = (rep["sustained_gsite_updates_s"] /
                                             base["sustained_gsite_updates_s"])
        # against the fastest repeat of every step-time sample
        best = fcfs_baseline(jobs, table.with_stat("best"))
        rep["fcfs_best"] = best
        rep["throughput_speedup_vs_fcfs_best"] = (rep["sustained_gsite_updates_s"] /
                                                  best["sustained_gsite_updates_s"])
    if fcfs and fcfs_sample:
        # FCFS measured on the GPU for the first jobs, beside the table's
        # prediction for the same jobs
        meas = fcfs_measured(jobs, fcfs_sample)
        sel = sorted(jobs, key=lambda j: j.arrival)[:fcfs_sample]
        pred = sum(j.steps * table(j) + table.job_overhead(j, -(-j.steps // 500)) for j in sel)
        meas["table_predicted_seconds"] = pred
        meas["table_gsite_updates_s"] = meas["site_updates"] / pred / 1e9 if pred else 0.0
        rep["fcfs_measured"] = meas
        rep["throughput_speedup_vs_fcfs_measured"] = (rep["sustained_gsite_updates_s"] /
                                                      meas["gsite_updates_s"])
    if verify:
        v = verify_sample(jobs, verify)
        rep["sample_verified"] = v
        rep["sample_bit_exact"] = v["bit_exact"]
    return rep


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--rate", type=float, nargs="+", default=[50.0])
    ap.add_argument("--duration", type=float, default=60.0)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--drain", type=float, default=60.0)
    ap.add_argument("--verify", type=int, default=8)
    ap.add_argument("--max-sites", type=float, nargs="+", default=[SERVE_MAX_SITES],
                    help="resident site caps to try (slots)")
    ap.add_argument("--quantum", type=int, default=100)
    ap.add_argument("--no-fcfs", action="store_true")
    ap.add_argument("--fcfs-sample", type=int, default=0,
                    help="also run the first N jobs FCFS on the GPU (measured, not simulated)")
    ap.add_argument("--policy", nargs="+", default=["fcfs"], choices=["fcfs", "srpt"],
                    help="admission order (srpt: least remaining work first, with eviction)")
    a = ap.parse_args(argv)
    import lgca_gb300 as gpu
    gpu.build()
    for r in a.rate:
        for cap in a.max_sites:
            for pol in a.policy:
                print(json.dumps(serve(r, a.duration, a.budget_gb * 1e9, a.drain, a.verify,
                                       not a.no_fcfs, cap, a.quantum, pol, a.fcfs_sample)),
                      flush=True)


if __name__ == "__main__":
    main()

__all__ = ["Job", "Server", "GpuBackend", "make_jobs", "lattice_bytes", "fcfs_baseline", "serve"]
