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

Merging (on by default): once a cohort's finished jobs hold at least
`merge_fraction` of its jobs, or jobs are queued, the cohort is re-packed
into a new batch of its running jobs plus the queued arrivals that fit the
budget, built in the background while the old one keeps stepping.  At the
old cohort's next step boundary the running jobs' state (displacement,
velocity; acceleration for NEWMARK) is copied into the new batch, the old
batch is freed, and the arrivals start stepping beside the jobs already
running.  A job's trajectory carries no other state between steps, so its
result is bitwise the same as run alone, whichever cohorts it passed
through; finished jobs stop holding device memory.

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
import ctypes
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
    # (90 values padded to 92 per tet)
    per_tet = 16 + 72 + 8 + 4 + 96 + 64 + 16 + 8 + 92 * w
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
    """One batch of jobs.  Built on the builder thread; it takes ownership of
    its jobs (attach) only when it joins the running set on the server's
    thread, so a re-pack can be built while the jobs still step elsewhere."""

    def __init__(self, jobs: List[Job], opts, tuning: Optional[dict] = None):
        self.jobs = jobs
        self.batch = hobak.BATCH([j.scene for j in jobs], opts)
        if tuning:
            self.batch.set_tuning(**tuning)
        for k, j in enumerate(jobs):
            if j.collisions is not None:
                eps, mu, beta = j.collisions
                self.batch.set_collisions(k, True, eps, mu, beta)
        self.bytes = self.batch.device_bytes()
        self.running = len(jobs)
        self.t_launch = None  # perf_counter() of the step in flight (pump mode)
        self.replacement = None  # (future or Cohort, reserved bytes): its re-pack being built

    def attach(self):
        for k, j in enumerate(self.jobs):
            j.cohort, j.slot = self, k

    def close(self):
        self.batch.close()


class Server:
    """Continuous batching under a device-memory budget."""

    def __init__(self, budget_bytes: int, precision: int = hobak.PRECISION_MIXED,
                 max_admit_per_tick: int = 64, keep_results: bool = True, async_build: bool = False,
                 tuning: Optional[dict] = None, merge: bool = True, merge_fraction: float = 0.5,
                 max_cohort: int = 64):
        self.budget = int(budget_bytes)
        self.opts = hobak.solver_opts(precision=precision)
        self.merge = merge
        self.merge_fraction = merge_fraction
        self.max_cohort = max_cohort
        self.merges = 0  # re-packs swapped in
        self.merged_arrivals = 0  # queued jobs that joined through a re-pack
        self.used_history: List[tuple] = []  # (perf_counter, bytes in use) after each round
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
        c.attach()
        self.used += c.bytes - reserved
        self.cohorts.append(c)

    def _build(self, jobs: List[Job]):
        """A cohort built now, or a future of one built on the builder thread."""
        if self._pool is None:
            return Cohort(jobs, self.opts, self.tuning)
        return self._pool.submit(Cohort, jobs, self.opts, self.tuning)

    def _plan_merges(self):
        """Start re-packing cohorts whose finished jobs hold memory (or when
        arrivals wait): their running jobs plus the queued jobs that fit the
        budget, which counts the old cohort until the swap frees it."""
        if not self.merge:
            return
        for c in self.cohorts:
            if c.replacement is not None or c.running == 0:
                continue
            parked = len(c.jobs) - c.running
            if parked == 0:
                continue
            keep = [j for j in c.jobs if j.finished < 0]
            est_keep = sum(footprint_bytes(j.scene, self.opts.precision) for j in keep)
            take: List[Job] = []
            est = 0
            while self.queue and len(keep) + len(take) < self.max_cohort:
                need = footprint_bytes(self.queue[0].scene, self.opts.precision)
                if self.used + est_keep + est + need > self.budget:
                    break
                est += need
                take.append(self.queue.popleft())
            if parked < self.merge_fraction * len(c.jobs) and not take:
                continue
            if self.used + est_keep + est > self.budget:
                self.queue.extendleft(reversed(take))  # no room for both batches at once yet
                continue
            self.used += est_keep + est
            c.replacement = (self._build(keep + take), est_keep + est)

    def _swap_ready(self, c: Cohort) -> Optional[Cohort]:
        """At c's step boundary: its re-pack, if built, with the running jobs'
        state copied in; c is freed.  None while the build is still running."""
        if c.replacement is None or c.t_launch is not None:
            return None
        built, reserved = c.replacement
        if isinstance(built, concurrent.futures.Future):
            if not built.done():
                return None
            built = built.result()
        newmark = self.opts.integrator == hobak.INTEGRATOR_NEWMARK
        now = time.perf_counter()
        for k, j in enumerate(built.jobs):
            if j.cohort is c:  # carried over: continue from where it is
                x, v = c.batch.get_state(j.slot)
                built.batch.set_state(k, x, v)
                if newmark:
                    built.batch.set_acceleration(k, c.batch.get_acceleration(j.slot))
                if j.finished >= 0:  # finished while the re-pack was built
                    built.batch.set_active(k, False)
                    built.running -= 1
            else:  # a merged arrival
                j.admitted = now
                self.merged_arrivals += 1
        built.attach()
        self.used += built.bytes - reserved - c.bytes
        c.close()
        self.cohorts[self.cohorts.index(c)] = built
        self.merges += 1
        return built

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
        # arrivals join running cohorts that have finished jobs first (a
        # re-pack), the rest form a new cohort
        self._plan_merges()
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
            if c.replacement is not None:
                # every carried job finished first: keep the re-pack for its arrivals, if any
                nxt = self._finish_replacement(c)
                if nxt is not None:
                    continue
            self.used -= c.bytes
            c.close()
            self.cohorts.remove(c)
        self.used_history.append((time.perf_counter(), self.used))

    def _finish_replacement(self, c: Cohort) -> Optional[Cohort]:
        """c has no running jobs left but its re-pack is being built: wait for
        it and swap it in when it holds arrivals, else drop it."""
        built, reserved = c.replacement
        if isinstance(built, concurrent.futures.Future):
            built = built.result()
        c.replacement = (built, reserved)
        if any(j.cohort is not c for j in built.jobs):
            return self._swap_ready(c)
        built.close()
        self.used -= reserved
        c.replacement = None
        return None

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
        self._plan_merges()
        for c in list(self.cohorts):
            self._swap_ready(c)
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
            if c.running > 0 and c.replacement is not None:
                c = self._swap_ready(c) or c
            if c.running > 0:
                c.batch.step_async(1)
                c.t_launch = time.perf_counter()
        self._retire()
        self._plan_merges()
        return done

    def drain(self, max_ticks: int = 1_000_000):
        while not self.idle() and max_ticks > 0:
            self.tick()
            max_ticks -= 1

    def close(self):
        if self._pool is not None:
            self._collect_built(block=True)
        for c in self.cohorts:
            if c.replacement is not None:
                built = c.replacement[0]
                (built.result() if isinstance(built, concurrent.futures.Future) else built).close()
            c.close()
        if self._pool is not None:
            self._pool.shutdown()
        self.cohorts.clear()


class NativeServer:
    """The same server in the library (hobak_server_*: host C++ over the
    batch ABI, a builder thread for async builds), with Server's interface:
    submit Job objects, drive it with pump() or tick(), read the jobs back.
    A C or C++ host uses the hobak_server_* calls directly."""

    def __init__(self, budget_bytes: int, precision: int = hobak.PRECISION_MIXED,
                 max_admit_per_tick: int = 64, keep_results: bool = True, async_build: bool = False,
                 tuning: Optional[dict] = None, merge: bool = True, merge_fraction: float = 0.5,
                 max_cohort: int = 64, solver_opts=None):
        from . import _lib
        self._lib = _lib
        L = _lib.load()
        o = _lib.HobakServerOpts()
        L.hobak_default_server_opts(o)
        o.budget_bytes = int(budget_bytes)
        o.max_admit, o.max_cohort = int(max_admit_per_tick), int(max_cohort)
        o.merge, o.merge_fraction = int(merge), float(merge_fraction)
        o.async_build, o.keep_results = int(async_build), int(keep_results)
        if tuning:
            cur = dict(tile_vertices=128, element_threads=128, assembly_threads=64, pcg_chunk=8, cluster_pcg=0,
                       cluster_max=16, step_ms=0.0)
            cur.update(tuning)
            o.use_tuning = 1
            o.tuning = _lib.HobakTuning(*[cur[k] for k in hobak.BATCH.TUNING])
        self.opts = solver_opts if solver_opts is not None else hobak.solver_opts(precision=precision)
        self.budget = int(budget_bytes)
        self.keep_results = keep_results
        self.h = ctypes.c_void_p()
        hobak.check(L.hobak_server_create(o, self.opts, ctypes.byref(self.h)), "hobak_server_create")
        self.jobs: Dict[int, Job] = {}  # server job id -> Job
        self.open: Dict[int, Job] = {}  # not finished yet
        self.finished: Dict[int, Job] = {}
        self.used_history: List[tuple] = []
        self.tick_ms: List[float] = []
        self.rejected = 0

    def submit(self, job: Job):
        a = hobak._SceneArrays(job.scene.rest, job.scene.tets,
                               hobak.make_material(job.scene.material, job.scene.mu, job.scene.lam,
                                                   getattr(job.scene, "fiber", None)),
                               job.scene.density, job.scene.gravity, job.scene.dt, job.scene.pinned,
                               job.scene.x0, job.scene.v0)
        contact = (ctypes.c_double * 3)(*job.collisions) if job.collisions is not None else None
        jid = ctypes.c_int()
        rc = self._lib.load().hobak_server_submit(self.h, ctypes.byref(a.desc), int(job.nsteps), contact,
                                                  ctypes.byref(jid))
        if rc != 0:
            self.rejected += 1
            raise ValueError(f"job {job.id}: " + self._lib.load().hobak_last_error().decode())
        self.jobs[jid.value] = job
        self.open[jid.value] = job
        info = self._info(jid.value)
        job.submitted = info.submitted_s

    def _info(self, jid: int, step_ms=None, x=None, v=None):
        info = self._lib.HobakJobInfo()
        hobak.check(self._lib.load().hobak_server_job(self.h, jid, ctypes.byref(info), hobak.dptr(step_ms),
                                                      hobak.dptr(x), hobak.dptr(v)), "hobak_server_job")
        return info

    def _stats(self):
        if not self.h.value:  # closed: the last figures
            return self._final
        st = self._lib.HobakServerStats()
        hobak.check(self._lib.load().hobak_server_get_stats(self.h, ctypes.byref(st)), "hobak_server_get_stats")
        return st

    def _sync(self):
        for jid, job in list(self.open.items()):
            info = self._info(jid)
            job.admitted = info.admitted_s
            job.done_steps = info.done_steps
            if info.state == 3:  # HOBAK_JOB_FAILED: its cohort could not be built
                job.failed = True
                del self.open[jid]
                continue
            if info.state == 2:  # HOBAK_JOB_FINISHED
                ms = np.zeros(info.done_steps)
                x = v = None
                if self.keep_results:
                    x, v = np.zeros(3 * info.nv), np.zeros(3 * info.nv)
                self._info(jid, ms, x, v)
                job.step_ms = ms.tolist()
                job.result_x, job.result_v = x, v
                job.finished = info.finished_s
                self.finished[job.id] = job
                del self.open[jid]
        st = self._stats()
        self.used_history.append((st.now_s, st.used_bytes))
        return st

    def _round(self, fn) -> int:
        n = ctypes.c_int()
        t0 = time.perf_counter()
        hobak.check(fn(self.h, ctypes.byref(n)), "hobak_server_round")
        if n.value:
            self.tick_ms.append((time.perf_counter() - t0) * 1e3)
        self._sync()
        return n.value

    def pump(self) -> int:
        return self._round(self._lib.load().hobak_server_pump)

    def tick(self) -> int:
        return self._round(self._lib.load().hobak_server_tick)

    def idle(self) -> bool:
        return bool(self._lib.load().hobak_server_idle(self.h))

    def drain(self, max_ticks: int = 1_000_000):
        while not self.idle() and max_ticks > 0:
            self.tick()
            max_ticks -= 1

    @property
    def used(self) -> int:
        return int(self._stats().used_bytes)

    @property
    def cohorts(self) -> list:
        return [None] * self._stats().cohorts

    @property
    def merges(self) -> int:
        return int(self._stats().merges)

    @property
    def merged_arrivals(self) -> int:
        return int(self._stats().merged_arrivals)

    @property
    def ticks(self) -> int:
        return int(self._stats().ticks)

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self._final = self._stats()
            self._lib.load().hobak_server_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
