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
