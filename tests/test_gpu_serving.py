"""Serving loop: jobs arriving while others run are admitted under the memory
budget, stepped concurrently, and each result is the same as the job run
alone."""
import numpy as np
import pytest

from hobakv1_gb300 import hobak, scenes
from hobakv1_gb300.serving import Job, NativeServer, Server, footprint_bytes

pytestmark = pytest.mark.gpu
VF = (1e-3, 1e3, 0.001)
# the Python server and the library's own (hobak_server_*), same tests
IMPLS = {"python": Server, "native": NativeServer}
impl = pytest.mark.parametrize("impl", sorted(IMPLS))


def jobs():
    mix = scenes.config4_scenes(count=4, nmin=5, nmax=8)
    out = [Job(0, mix[0], 7), Job(1, scenes.two_cubes_scene(6), 9, VF), Job(2, mix[1], 3),
           Job(3, mix[2], 11), Job(4, scenes.two_cubes_scene(5, gap=3e-4), 5, VF), Job(5, mix[3], 6)]
    return out


def alone(job, precision):
    b = hobak.BATCH([job.scene], hobak.solver_opts(precision=precision))
    if job.collisions:
        b.set_collisions(0, True, *job.collisions)
    b.step(job.nsteps)
    return b.get_state(0)


@impl
@pytest.mark.parametrize("precision", [hobak.PRECISION_FP64, hobak.PRECISION_MIXED], ids=["fp64", "mixed"])
def test_results_equal_alone_and_in_the_mix(precision, impl):
    js = jobs()
    srv = IMPLS[impl](budget_bytes=1 << 34, precision=precision)
    # staggered arrivals: two jobs, a few ticks, then the rest while those run
    srv.submit(js[0])
    srv.submit(js[1])
    srv.tick()
    srv.tick()
    for j in js[2:]:
        srv.submit(j)
        srv.tick()
    srv.drain()
    assert len(srv.finished) == len(js)
    for j in js:
        assert j.done_steps == j.nsteps
        x, v = alone(j, precision)
        # per-scene tiles and reductions: bitwise the same alone and in the mix
        assert np.array_equal(j.result_x, x) and np.array_equal(j.result_v, v), j.id


@impl
def test_admission_respects_the_memory_budget(impl):
    js = jobs()
    budget = max(footprint_bytes(j.scene, 1) for j in js) * 2  # about two jobs at a time
    srv = IMPLS[impl](budget_bytes=budget, precision=hobak.PRECISION_MIXED)
    for j in js:
        srv.submit(j)
    peak = 0
    while not srv.idle():
        srv.tick()
        assert srv.used <= budget
        peak = max(peak, len(srv.cohorts))
    assert len(srv.finished) == len(js)
    assert all(j.admitted >= j.submitted for j in js)
    with pytest.raises(ValueError):
        IMPLS[impl](budget_bytes=1024).submit(js[0])


@impl
def test_event_driven_pump_matches_alone(impl):
    """pump(): cohorts relaunch independently (async builds, small cohorts);
    results stay bitwise equal to each job run alone."""
    js = jobs()
    srv = IMPLS[impl](budget_bytes=1 << 34, precision=hobak.PRECISION_MIXED, async_build=True,
                      max_admit_per_tick=2)
    srv.submit(js[0])
    for _ in range(3):
        srv.pump()
    for j in js[1:]:
        srv.submit(j)
        srv.pump()
    while not srv.idle():
        srv.pump()
    srv.close()
    assert len(srv.finished) == len(js)
    for j in js:
        assert j.done_steps == j.nsteps and len(j.step_ms) == j.nsteps
        x, v = alone(j, hobak.PRECISION_MIXED)
        assert np.array_equal(j.result_x, x) and np.array_equal(j.result_v, v), j.id


@impl
@pytest.mark.parametrize("mode", ["tick", "pump"])
def test_arrivals_merge_into_a_running_cohort_and_results_equal_alone(mode, impl):
    """Arrivals queued while a cohort has a finished (parked) job are merged
    into it: the cohort is re-packed with its running jobs plus the arrivals
    and swapped in at a step boundary.  Every result, of the jobs carried
    across the re-pack and of the merged arrivals, is bitwise the same as the
    job run alone."""
    js = jobs()
    a, b, c, d, e = js[2], js[3], js[0], js[1], js[5]  # 3, 11, 7, 9 (contact) and 6 steps
    srv = IMPLS[impl](budget_bytes=1 << 34, precision=hobak.PRECISION_MIXED, merge_fraction=1.0,
                      async_build=(mode == "pump"))
    step = srv.tick if mode == "tick" else srv.pump
    for j in (a, b, c):
        srv.submit(j)
    while a.finished < 0:
        step()
    assert srv.merges == 0  # nothing queued: merge_fraction 1 keeps the cohort as it is
    srv.submit(d)
    srv.submit(e)
    while not srv.idle():
        step()
    srv.close()
    assert srv.merges >= 1 and srv.merged_arrivals == 2
    assert d.admitted > a.finished and e.admitted > a.finished
    for j in (a, b, c, d, e):
        assert j.done_steps == j.nsteps
        x, v = alone(j, hobak.PRECISION_MIXED)
        assert np.array_equal(j.result_x, x) and np.array_equal(j.result_v, v), j.id


@impl
def test_finished_jobs_release_their_memory(impl):
    """With no arrivals, a cohort half of whose jobs finished is re-packed
    without them: device memory in use falls, and the remaining job's result
    is unchanged (bitwise equal to running it alone)."""
    js = jobs()
    short, longer = js[2], js[3]  # 3 and 11 steps
    srv = IMPLS[impl](budget_bytes=1 << 34, precision=hobak.PRECISION_FP64, merge_fraction=0.5)
    srv.submit(short)
    srv.submit(longer)
    srv.tick()
    before = srv.used
    while short.finished < 0:
        srv.tick()
    assert srv.merges == 1
    assert srv.used < before
    srv.drain()
    x, v = alone(longer, hobak.PRECISION_FP64)
    assert np.array_equal(longer.result_x, x) and np.array_equal(longer.result_v, v)


@pytest.mark.parametrize("precision", [hobak.PRECISION_FP64, hobak.PRECISION_MIXED], ids=["fp64", "mixed"])
def test_admission_estimate_bounds_the_device_bytes(precision):
    """The footprint both servers admit by is an upper bound of what a batch
    of those scenes holds on the device (so the budget is never exceeded),
    with and without contact."""
    sc = scenes.config4_scenes(count=3, nmin=5, nmax=14) + [scenes.two_cubes_scene(6)]
    for s in sc:
        b = hobak.BATCH([s], hobak.solver_opts(precision=precision))
        assert footprint_bytes(s, precision) >= b.device_bytes(), s.name
        b.close()
    b = hobak.BATCH(sc, hobak.solver_opts(precision=precision))
    b.set_collisions(len(sc) - 1, True, *VF)
    b.step(1)
    assert sum(footprint_bytes(s, precision) for s in sc) >= b.device_bytes()
    b.close()
