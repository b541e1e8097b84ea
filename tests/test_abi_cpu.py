"""C ABI checks that need no GPU: the library builds, loads and exports every
function include/hobak_gpu.h declares; argument validation fails cleanly."""
import ctypes
import os
import re

import numpy as np
import pytest

from hobakv1_gb300 import _lib, build, scenes
from hobakv1_gb300.hobak import _SceneArrays, make_material, solver_opts

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "hobak_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hobak_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n
    # and the Python binding table covers the header exactly
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)


def test_version_and_defaults():
    L = _lib.load()
    assert b"sm_103a" in L.hobak_version()
    o = _lib.HobakSolverOpts()
    L.hobak_default_solver_opts(ctypes.byref(o))
    assert o.tol == 1e-8 and o.max_iters == 1000 and o.use_graph == 1


def _desc(scene):
    return _SceneArrays(scene.rest, scene.tets, make_material(scene.material, scene.mu, scene.lam),
                        scene.density, scene.gravity, scene.dt, scene.pinned, scene.x0, scene.v0)


@pytest.mark.parametrize("mutate,expect", [
    (lambda d: setattr(d, "nv", 0), "empty mesh"),
    (lambda d: setattr(d, "dt", -1.0), "dt and density"),
    (lambda d: setattr(d.material, "kind", 42), "unknown material"),
])
def test_invalid_scene_is_rejected_before_touching_the_device(mutate, expect):
    L = _lib.load()
    a = _desc(scenes.config1_scene(2))
    mutate(a.desc)
    h = ctypes.c_void_p()
    opts = solver_opts()
    rc = L.hobak_batch_create(ctypes.byref(a.desc), 1, ctypes.byref(opts), ctypes.byref(h))
    assert rc == -1
    assert expect in L.hobak_last_error().decode()
    assert not h.value


def test_out_of_range_tet_index_rejected():
    L = _lib.load()
    s = scenes.config1_scene(2)
    s.tets = s.tets.copy()
    s.tets[3, 2] = 10_000
    a = _desc(s)
    h = ctypes.c_void_p()
    rc = L.hobak_batch_create(ctypes.byref(a.desc), 1, None, ctypes.byref(h))
    assert rc == -1 and "out of range" in L.hobak_last_error().decode()


def test_bad_solver_options_rejected():
    L = _lib.load()
    a = _desc(scenes.config1_scene(2))
    h = ctypes.c_void_p()
    opts = solver_opts(tol=-1.0)
    assert L.hobak_batch_create(ctypes.byref(a.desc), 1, ctypes.byref(opts), ctypes.byref(h)) == -1
    opts = solver_opts(max_refinements=9)
    assert L.hobak_batch_create(ctypes.byref(a.desc), 1, ctypes.byref(opts), ctypes.byref(h)) == -1


def test_null_handles_are_errors_not_crashes():
    L = _lib.load()
    assert L.hobak_batch_step(None, 1, None) == -1
    assert L.hobak_batch_get_state(None, 0, None, None) == -1
    assert L.hobak_batch_destroy(None) == 0


def test_server_options_and_admission_checks_without_a_device():
    """hobak_server_*: defaults, refused options and jobs, and a queued job's
    state, all before any batch is built (no device needed)."""
    L = _lib.load()
    o = _lib.HobakServerOpts()
    L.hobak_default_server_opts(ctypes.byref(o))
    assert o.max_admit == 64 and o.max_cohort == 64 and o.merge == 1 and o.merge_fraction == 0.5
    assert o.keep_results == 1 and o.async_build == 0 and o.budget_bytes > 0
    h = ctypes.c_void_p()
    bad = _lib.HobakServerOpts()
    L.hobak_default_server_opts(ctypes.byref(bad))
    bad.merge_fraction = 1.5
    assert L.hobak_server_create(ctypes.byref(bad), None, ctypes.byref(h)) == -1
    assert "merge_fraction" in L.hobak_last_error().decode() and not h.value
    assert L.hobak_server_create(ctypes.byref(o), None, ctypes.byref(h)) == 0 and h.value
    a = _desc(scenes.config1_scene(2))
    jid = ctypes.c_int(-1)
    assert L.hobak_server_submit(h, ctypes.byref(a.desc), 0, None, ctypes.byref(jid)) == -1
    assert L.hobak_server_submit(h, ctypes.byref(a.desc), 5, None, ctypes.byref(jid)) == 0 and jid.value == 0
    info = _lib.HobakJobInfo()
    assert L.hobak_server_job(h, 0, ctypes.byref(info), None, None, None) == 0
    assert (info.state, info.done_steps, info.nsteps, info.nv) == (0, 0, 5, 27)
    assert info.submitted_s > 0 and info.admitted_s == -1 and info.finished_s == -1
    x = np.zeros(81)
    assert L.hobak_server_job(h, 0, None, None, x.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None) == -1
    assert L.hobak_server_job(h, 7, ctypes.byref(info), None, None, None) == -1
    assert L.hobak_server_idle(h) == 0
    st = _lib.HobakServerStats()
    assert L.hobak_server_get_stats(h, ctypes.byref(st)) == 0 and (st.queued, st.cohorts, st.used_bytes) == (1, 0, 0)
    assert L.hobak_server_destroy(h) == 0
    small = _lib.HobakServerOpts()
    L.hobak_default_server_opts(ctypes.byref(small))
    small.budget_bytes = 1024
    h2 = ctypes.c_void_p()
    assert L.hobak_server_create(ctypes.byref(small), None, ctypes.byref(h2)) == 0
    assert L.hobak_server_submit(h2, ctypes.byref(a.desc), 5, None, ctypes.byref(jid)) == -1
    assert "budget" in L.hobak_last_error().decode()
    assert L.hobak_server_destroy(h2) == 0


def test_server_reports_a_failed_build_once_and_marks_its_jobs():
    """A job whose batch cannot be built (an unknown material, refused
    before the device is touched): the round returns the error, the job is
    marked failed, its reservation is returned and the server goes idle."""
    L = _lib.load()
    o = _lib.HobakServerOpts()
    L.hobak_default_server_opts(ctypes.byref(o))
    h = ctypes.c_void_p()
    assert L.hobak_server_create(ctypes.byref(o), None, ctypes.byref(h)) == 0
    a = _desc(scenes.config1_scene(2))
    a.desc.material.kind = 42
    jid = ctypes.c_int(-1)
    assert L.hobak_server_submit(h, ctypes.byref(a.desc), 3, None, ctypes.byref(jid)) == 0
    steps = ctypes.c_int(-1)
    assert L.hobak_server_pump(h, ctypes.byref(steps)) == -1
    msg = L.hobak_last_error().decode()
    assert "building a cohort" in msg and "material" in msg, msg
    info = _lib.HobakJobInfo()
    assert L.hobak_server_job(h, jid.value, ctypes.byref(info), None, None, None) == 0 and info.state == 3
    st = _lib.HobakServerStats()
    assert L.hobak_server_get_stats(h, ctypes.byref(st)) == 0 and st.used_bytes == 0 and st.building == 0
    assert L.hobak_server_pump(h, ctypes.byref(steps)) == 0 and steps.value == 0
    assert L.hobak_server_idle(h) == 1
    assert L.hobak_server_destroy(h) == 0
