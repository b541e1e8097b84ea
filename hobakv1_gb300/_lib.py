"""Loads libhobak_gpu.so (the sm_103a CUDA library) and declares its C ABI.

There is no CPU fallback: if the library is missing or cannot find a GB300,
every entry point raises.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


class HobakMaterial(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("mu", ctypes.c_double), ("lambda_", ctypes.c_double),
                ("fiber", ctypes.c_double * 3)]


class HobakSceneDesc(ctypes.Structure):
    _fields_ = [("nv", ctypes.c_int), ("nt", ctypes.c_int), ("rest", _dp), ("tets", _ip),
                ("material", HobakMaterial), ("density", ctypes.c_double),
                ("gravity", ctypes.c_double * 3), ("dt", ctypes.c_double),
                ("npinned", ctypes.c_int), ("pinned", _ip), ("x0", _dp), ("v0", _dp)]


class HobakSolverOpts(ctypes.Structure):
    _fields_ = [("tol", ctypes.c_double), ("max_iters", ctypes.c_int), ("precision", ctypes.c_int),
                ("preconditioner", ctypes.c_int), ("max_refinements", ctypes.c_int),
                ("use_graph", ctypes.c_int), ("integrator", ctypes.c_int),
                ("rayleigh_alpha", ctypes.c_double), ("rayleigh_beta", ctypes.c_double),
                ("max_newton", ctypes.c_int), ("newton_tolerance", ctypes.c_double),
                ("inner_tolerance", ctypes.c_double)]


class HobakTuning(ctypes.Structure):
    _fields_ = [("tile_vertices", ctypes.c_int), ("element_threads", ctypes.c_int),
                ("assembly_threads", ctypes.c_int), ("pcg_chunk", ctypes.c_int), ("cluster_pcg", ctypes.c_int),
                ("cluster_max", ctypes.c_int), ("step_ms", ctypes.c_double)]


class HobakServerOpts(ctypes.Structure):
    _fields_ = [("budget_bytes", ctypes.c_longlong), ("max_admit", ctypes.c_int), ("max_cohort", ctypes.c_int),
                ("merge", ctypes.c_int), ("merge_fraction", ctypes.c_double), ("async_build", ctypes.c_int),
                ("keep_results", ctypes.c_int), ("use_tuning", ctypes.c_int), ("tuning", HobakTuning)]


class HobakServerStats(ctypes.Structure):
    _fields_ = [("used_bytes", ctypes.c_longlong), ("cohorts", ctypes.c_int), ("queued", ctypes.c_int),
                ("building", ctypes.c_int), ("merges", ctypes.c_int), ("merged_arrivals", ctypes.c_int),
                ("finished", ctypes.c_int), ("ticks", ctypes.c_longlong), ("now_s", ctypes.c_double)]


class HobakJobInfo(ctypes.Structure):
    _fields_ = [("state", ctypes.c_int), ("done_steps", ctypes.c_int), ("nsteps", ctypes.c_int),
                ("nv", ctypes.c_int), ("submitted_s", ctypes.c_double), ("admitted_s", ctypes.c_double),
                ("finished_s", ctypes.c_double)]


class HobakStepStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("converged", ctypes.c_int),
                ("rel_residual", ctypes.c_double), ("refinements", ctypes.c_int)]


# name -> (restype, argtypes); mirrors include/hobak_gpu.h
SIGNATURES = {
    "hobak_default_server_opts": (None, [ctypes.POINTER(HobakServerOpts)]),
    "hobak_server_create": (ctypes.c_int, [ctypes.POINTER(HobakServerOpts), ctypes.POINTER(HobakSolverOpts),
                                           ctypes.POINTER(ctypes.c_void_p)]),
    "hobak_server_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(HobakSceneDesc), ctypes.c_int, _dp, _ip]),
    "hobak_server_pump": (ctypes.c_int, [ctypes.c_void_p, _ip]),
    "hobak_server_tick": (ctypes.c_int, [ctypes.c_void_p, _ip]),
    "hobak_server_idle": (ctypes.c_int, [ctypes.c_void_p]),
    "hobak_server_get_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(HobakServerStats)]),
    "hobak_server_job": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(HobakJobInfo), _dp, _dp, _dp]),
    "hobak_server_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "hobak_version": (ctypes.c_char_p, []),
    "hobak_last_error": (ctypes.c_char_p, []),
    "hobak_device_check": (ctypes.c_int, [_ip, _ip, _ip]),
    "hobak_default_solver_opts": (None, [ctypes.POINTER(HobakSolverOpts)]),
    "hobak_batch_create": (ctypes.c_int, [ctypes.POINTER(HobakSceneDesc), ctypes.c_int,
                                          ctypes.POINTER(HobakSolverOpts), ctypes.POINTER(ctypes.c_void_p)]),
    "hobak_batch_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "hobak_batch_num_scenes": (ctypes.c_int, [ctypes.c_void_p, _ip]),
    "hobak_batch_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(HobakStepStats)]),
    "hobak_batch_step_async": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "hobak_batch_wait": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(HobakStepStats)]),
    "hobak_batch_query": (ctypes.c_int, [ctypes.c_void_p]),
    "hobak_batch_set_state_all": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp]),
    "hobak_batch_get_state_all": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp]),
    "hobak_batch_set_external_forces_all": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "hobak_batch_set_active": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "hobak_batch_set_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp, _dp]),
    "hobak_batch_get_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp, _dp]),
    "hobak_batch_set_external_forces": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp]),
    "hobak_batch_set_solver": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(HobakSolverOpts)]),
    "hobak_batch_device_bytes": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)]),
    "hobak_batch_energy": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp]),
    "hobak_gpu_create": (ctypes.c_int, [ctypes.POINTER(HobakSceneDesc), ctypes.POINTER(HobakSolverOpts),
                                        ctypes.POINTER(ctypes.c_void_p)]),
    "hobak_gpu_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(HobakStepStats)]),
    "hobak_gpu_set_state": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp]),
    "hobak_gpu_get_state": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp]),
    "hobak_gpu_set_external_forces": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "hobak_gpu_set_collisions": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                                ctypes.c_double]),
    "hobak_gpu_set_edge_collisions": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "hobak_gpu_set_solver": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(HobakSolverOpts)]),
    "hobak_gpu_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "hobak_material_eval": (ctypes.c_int, [ctypes.POINTER(HobakMaterial), ctypes.c_int, _dp, _dp, _dp, _dp]),
    "hobak_material_hessian": (ctypes.c_int, [ctypes.POINTER(HobakMaterial), ctypes.c_int, _dp, _dp]),
    "hobak_material_eval_svd": (ctypes.c_int, [ctypes.POINTER(HobakMaterial), ctypes.c_int, _dp, _dp, _dp,
                                               _dp, _dp, _dp, _dp]),
    "hobak_material_needs_svd": (ctypes.c_int, [ctypes.c_int, _ip, _ip]),
    "hobak_element_eval": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _dp, _ip, _dp,
                                          ctypes.POINTER(HobakMaterial), _dp, _dp, _dp, _dp]),
    "hobak_batch_assemble": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _ip, _ip, _ip, _dp, _dp]),
    "hobak_batch_get_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "hobak_batch_enable_timing": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "hobak_batch_phase_times": (ctypes.c_int, [ctypes.c_void_p, _dp, ctypes.POINTER(ctypes.c_longlong)]),
    "hobak_batch_launch_count": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)]),
    "hobak_batch_time_kernels": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp]),
    "hobak_batch_kernel_bytes": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "hobak_batch_get_tuning": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(HobakTuning)]),
    "hobak_batch_pcg_path": (ctypes.c_int, [ctypes.c_void_p, _ip]),
    "hobak_batch_set_scene_cluster": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "hobak_batch_set_green_damping": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_double]),
    "hobak_batch_get_acceleration": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "hobak_batch_set_acceleration": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "hobak_batch_set_pin_targets": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "hobak_batch_set_edge_collisions": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "hobak_batch_edge_pairs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _ip, _ip, ctypes.c_int]),
    "hobak_batch_snapshot_bytes": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t)]),
    "hobak_batch_snapshot": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
    "hobak_batch_restore": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
    "hobak_batch_set_tuning": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(HobakTuning)]),
    "hobak_batch_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(HobakTuning)]),
    "hobak_batch_set_collisions": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                                  ctypes.c_double, ctypes.c_double]),
    "hobak_batch_collision_pairs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _ip, _ip,
                                                   ctypes.c_int, _ip, _ip]),
    "hobak_batch_collision_response": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _ip, _dp, _dp]),
    "hobak_element_eval_noalloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.c_void_p, ctypes.POINTER(HobakMaterial), ctypes.c_void_p,
                                                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.c_void_p]),
}

_lib = None


class HobakError(RuntimeError):
    def __init__(self, code, where, msg):
        super().__init__(f"{where} failed with status {code}: {msg}")
        self.code = code


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load the CUDA library (building it with nvcc if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing; build it with hobakv1_gb300.build.build()")
        _build.build()
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(rc: int, where: str) -> int:
    """Raise on a negative status; return warnings (positive) to the caller."""
    if rc < 0:
        raise HobakError(rc, where, load().hobak_last_error().decode())
    return rc


def dptr(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def iptr(a):
    return a.ctypes.data_as(_ip) if a is not None else None
