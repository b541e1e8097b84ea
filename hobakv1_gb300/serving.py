"""Continuous-batching server for scene-timestep jobs.

A job is a scene plus a number of BACKWARD_EULER_VELOCITY steps.  The server
keeps every admitted job's state resident on the GPU until it finishes:

  1. admission: queued jobs (FIFO) are admitted while their estimated device
     footprint fits the memory budget; the jobs admitted together are packed
     into one batch (a "cohort") that joins the running set;
  2. every cohort with running jobs steps on its own CUDA stream
     (hobak_batch_step_async), so the cohorts' work overlaps on the device;
  3. a finished step is booked for the cohort's running jobs (its latency is
     the job's step latency); finished jobs are parked
     (hobak_batch_set_active(scene, 0): state kept, kernels skip them) and
     their final state is read back; a cohort whose jobs are all done is freed.

`pump()` is the event-driven loop: each cohort is polled
(hobak_batch_query) and relaunched as soon as its own step is done, so a
cohort of small fast scenes never waits for a cohort of large ones.
`tick()` is the lock-step variant (all cohorts step, all are waited for).

Within a cohort every scene keeps its own reduction tiles, so a job's result
does not depend on which other jobs shared its batch or the device.

With `async_build=True` a builder thread creates the admitted cohorts (mesh
upload, block pattern, surface extraction; the library calls release the
GIL), so admission work overlaps the running cohorts' steps instead of
stalling them; a cohort joins the running set at the first scheduling round
after it is built.  The memory budget is reserved at admission time.
"""
from __future__ import annotations

import concurrent.futures
import dataclasses
import time
from collections import deque
from typing import Deque, Dict, List, Optional

import numpy as np

from . import hobak


def footprint_bytes(scene, precision: int) -> int:
    """Conservative device bytes of one scene in a batch: the common buffers
    plus those of its precision (the library allocates only the batch's
    precision); at most 16 blocks per vertex row, padded in 32-vertex slices."""
    nv, nt = scene.nv, scene.nt
    nb = 16 * nv
    w = 4 if precision == hobak.PRECISION_MIXED else 8
    # tets, DmInv, vol, scene id, element g, contribution map, incidences, psi; element Hessians
    per_tet = 16 + 72 + 8 + 4 + 96 + 64 + 16 + 8 + 90 * w
    # cols, block row, contribution ranges, sliced column; sliced LHS values
    per_block = 4 + 4 + 4 + 4 + 9 * w
    # rest, x, v, f_ext, pin target, mass, mask, scene id, rowptr, incidences,
    # rhs, y, r64; block inverse and inner vectors
    per_vertex = 5 * 24 + 8 + 1 + 4 + 4 + 4 + 3 * 24 + 9 * w + (6 if w == 4 else 4) * 3 * w
    return int(nt * per_tet + nb * per_block + nv * per_vertex + (1 << 20))


@dataclasses.dataclass
class Job:
    id: int
    scene: object
    nsteps: int
    collisions: Optional[tuple] = None  # (eps, stiffness, beta) for vertex-face contact
    submitted: float = 0.0
    admitted: float = -1.0
    finished: float = -1.0
    done_steps: int = 0
    step_ms: List[float] = dataclasses.field(default_factory=list)
    result_x: Optional[np.ndarray] = None
    result_v: Optional[np.ndarray] = None
    cohort: Optional["Cohort"] = None
    slot: int = -1


class Cohort:
    def __init__(self, jobs: List[Job], opts, tuning: Optional[dict] = None):
        self.jobs = jobs
        self.batch = hobak.BATCH([j.scene for j in jobs], opts)
        if tuning:
            self.batch.set_tuning(**tuning)
        for k, j in enumerate(jobs):
            j.cohort, j.slot = self, k
            if j.collisions is not None:
                eps, mu, beta = j.collisions
                self.batch.set_collisions(k, True, eps, mu, beta)
        self.bytes = self.batch.device_bytes()
        self.running = len(jobs)
        self.t_launch = None  # perf_counter() of the step in flight (pump mode)

    def close(self):
        self.batch.close()


class Server:
    """Continuous batching under a device-memory budget."""

    def __init__(self, budget_bytes: int, precision: int = hobak.PRECISION_MIXED,
                 max_admit_per_tick: int = 64, keep_results: bool = True, async_build: bool = False,
                 tuning: Optional[dict] = None):
        self.budget = int(budget_bytes)
        self.opts = hobak.solver_opts(precision=precision)
        self.tuning = tuning  # launch shapes for every cohort (hobak_batch_set_tuning)
        self.max_admit = max_admit_per_tick
        self.keep_results = keep_results
        self.queue: Deque[Job] = deque()
        self.cohorts: List[Cohort] = []
        self.finished: Dict[int, Job] = {}
        self.used = 0
        self.ticks = 0
        self.tick_ms: List[float] = []
        self.rejected = 0
        self._pool = concurrent.futures.ThreadPoolExecutor(max_workers=1) if async_build else None
        self._building: List[tuple] = []  # (future, reserved bytes)

    # ---- client side ----
    def submit(self, job: Job):
        job.submitted = time.perf_counter()
        if footprint_bytes(job.scene, self.opts.precision) > self.budget:
            self.rejected += 1  # can never fit: refuse instead of blocking the queue
            raise ValueError(f"job {job.id} needs more than the whole memory budget")
        self.queue.append(job)

    def idle(self) -> bool:
        return not self.queue and not self.cohorts and not self._building

    # ---- server loop ----
    def _join(self, c: Cohort, reserved: int):
        now = time.perf_counter()
        for j in c.jobs:
            j.admitted = now
        self.used += c.bytes - reserved
        self.cohorts.append(c)

    def _collect_built(self, block: bool = False):
        keep = []
        for fut, reserved in self._building:
            if fut.done() or block:
                self._join(fut.result(), reserved)
            else:
                keep.append((fut, reserved))
        self._building = keep

    def _admit(self):
        if self._pool is not None:
            self._collect_built(block=not self.cohorts)  # nothing running: wait for the build
        take: List[Job] = []
        est = 0
        while self.queue and len(take) < self.max_admit:
            need = footprint_bytes(self.queue[0].scene, self.opts.precision)
            if self.used + est + need > self.budget:
                break
            est += need
            take.append(self.queue.popleft())
        if not take:
            return
        self.used += est  # reserved until the cohort reports its real size
        if self._pool is None:
            self._join(Cohort(take, self.opts, self.tuning), est)
        else:
            self._building.append((self._pool.submit(Cohort, take, self.opts, self.tuning), est))
            if not self.cohorts:
                self._collect_built(block=True)

    def _step_done(self, c: Cohort, ms: float, now: float) -> int:
        """Book one finished step of cohort c (latency ms) for its running jobs."""
        done = 0
        for j in c.jobs:
            if j.finished >= 0:
                continue
            j.done_steps += 1
            j.step_ms.append(ms)
            done += 1
            if j.done_steps >= j.nsteps:
                j.finished = now
                if self.keep_results:
                    j.result_x, j.result_v = c.batch.get_state(j.slot)
                c.batch.set_active(j.slot, False)
                c.running -= 1
                self.finished[j.id] = j
        return done

    def _retire(self):
        for c in [c for c in self.cohorts if c.running == 0 and c.t_launch is None]:
            self.used -= c.bytes
            c.close()
            self.cohorts.remove(c)

    def tick(self) -> int:
        """One lock-step scheduling round: every running cohort advances one
        step, all are waited for; returns the number of job-steps completed."""
        self._admit()
        live = [c for c in self.cohorts if c.running > 0 and c.t_launch is None]
        if not live:
            return 0
        t0 = time.perf_counter()
        for c in live:
            c.batch.step_async(1)
        for c in live:
            c.batch.wait()
        ms = (time.perf_counter() - t0) * 1e3
        self.tick_ms.append(ms)
        self.ticks += 1
        now = time.perf_counter()
        done = sum(self._step_done(c, ms, now) for c in live)
        self._retire()
        return done

    def pump(self) -> int:
        """One event-driven scheduling round: admit, start a step on every
        idle cohort, and book every cohort whose step has finished, starting
        its next step at once; cohorts never wait for one another.  A job's
        step latency is its cohort's launch-to-completion time.  Returns the
        number of job-steps completed (0 when nothing finished yet)."""
        self._admit()
        done = 0
        for c in list(self.cohorts):
            if c.t_launch is not None:
                if not c.batch.query():
                    continue
                c.batch.wait()
                now = time.perf_counter()
                ms = (now - c.t_launch) * 1e3
                c.t_launch = None
                self.tick_ms.append(ms)
                self.ticks += 1
                done += self._step_done(c, ms, now)
            if c.running > 0:
                c.batch.step_async(1)
                c.t_launch = time.perf_counter()
        self._retire()
        return done

    def drain(self, max_ticks: int = 1_000_000):
        while not self.idle() and max_ticks > 0:
            self.tick()
            max_ticks -= 1

    def close(self):
        if self._pool is not None:
            self._collect_built(block=True)
            self._pool.shutdown()
        for c in self.cohorts:
            c.close()
        self.cohorts.clear()
