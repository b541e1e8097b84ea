"""ctypes wrapper of the CPU oracle (oracle/hobak_oracle.cpp).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, as the checker or the timed CPU baseline.  The
product library (hobakv1_gb300) never imports this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libhobak_oracle.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lib = None

MATERIALS = {"snh": 0, "arap": 1, "stvk": 2, "linear": 3, "neo_hookean_bw": 4, "snh_barrier": 5,
             "aniso_arap": 6, "aniso_stvk": 7, "aniso_fung": 8, "aniso_dirichlet": 9}


def build(quiet: bool = True) -> str:
    """Compile the oracle with make (portable flags; works on x86 and aarch64)."""
    subprocess.run(["make", "-C", HERE, "-s"], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.oracle_elements.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _ip, _dp, ctypes.c_int, ctypes.c_double,
                                      ctypes.c_double, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        L.oracle_set_fiber.argtypes = [ctypes.c_void_p, _dp]
        L.oracle_svd.argtypes = [ctypes.c_int, _dp, _dp, _dp, _dp]
        L.oracle_create.restype = ctypes.c_void_p
        L.oracle_create.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _ip, ctypes.c_int, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_double, _dp, ctypes.c_double]
        L.oracle_destroy.argtypes = [ctypes.c_void_p]
        L.oracle_set_state.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.oracle_get_state.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.oracle_attach_pins.argtypes = [ctypes.c_void_p, ctypes.c_int, _ip]
        L.oracle_set_pin_targets.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp]
        L.oracle_ee_pairs.argtypes = [ctypes.c_void_p, _ip, _ip]
        L.oracle_set_green_damping.argtypes = [ctypes.c_void_p, ctypes.c_double]
        L.oracle_set_solver.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_int]
        L.oracle_set_external_forces.argtypes = [ctypes.c_void_p, _dp]
        L.oracle_step.argtypes = [ctypes.c_void_p, ctypes.c_int, _ip, _dp]
        L.oracle_nblocks.argtypes = [ctypes.c_void_p]
        L.oracle_assemble.argtypes = [ctypes.c_void_p, _ip, _ip, _dp, _dp]
        L.oracle_set_collisions.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                            ctypes.c_double]
        L.oracle_vf_pairs.argtypes = [ctypes.c_void_p, _ip, ctypes.c_int, _ip]
        L.oracle_num_surface_triangles.argtypes = [ctypes.c_void_p]
        L.oracle_vf_response.argtypes = [ctypes.c_void_p, _ip, _dp, _dp]
        L.oracle_set_integrator.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.oracle_newton_iterations.argtypes = [ctypes.c_void_p]
        L.oracle_get_acceleration.argtypes = [ctypes.c_void_p, _dp]
        L.oracle_energy.argtypes = [ctypes.c_void_p]
        L.oracle_energy.restype = ctypes.c_double
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def set_threads(n: int) -> int:
    """OpenMP threads of the oracle's next calls (n <= 0: every host core)."""
    return lib().oracle_set_threads(int(n))


def _d(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def _i(a):
    return a.ctypes.data_as(_ip) if a is not None else None


def elements(rest, tets, x, material, mu, lam, fiber=None):
    """Per-tet F, svd_rv sigma, psi, PK1, clamped and unclamped 9x9 Hessians
    (H9, H9u), element forces and 12x12 element Hessians."""
    rest = np.ascontiguousarray(rest, dtype=np.float64)
    tets = np.ascontiguousarray(tets, dtype=np.int32)
    x = np.ascontiguousarray(x, dtype=np.float64)
    a = np.ascontiguousarray(fiber, dtype=np.float64) if fiber is not None else None
    nv, nt = rest.shape[0], tets.shape[0]
    out = {k: np.zeros((nt, n)) for k, n in
           [("F", 9), ("Sigma", 3), ("P", 9), ("H9", 81), ("fe", 12), ("He", 144), ("H9u", 81)]}
    out["psi"] = np.zeros(nt)
    rc = lib().oracle_elements(nv, nt, _d(rest), _i(tets), _d(x), MATERIALS[material], mu, lam, _d(a),
                               _d(out["F"]), _d(out["Sigma"]), _d(out["psi"]), _d(out["P"]),
                               _d(out["H9"]), _d(out["fe"]), _d(out["He"]), _d(out["H9u"]))
    assert rc == 0
    return out


def svd(F):
    F = np.ascontiguousarray(F, dtype=np.float64).reshape(-1, 9)
    n = F.shape[0]
    U, S, V = np.zeros((n, 9)), np.zeros((n, 3)), np.zeros((n, 9))
    lib().oracle_svd(n, _d(F), _d(U), _d(S), _d(V))
    return U, S, V


class Sim:
    """CPU oracle timestepper on one scene: BACKWARD_EULER_VELOCITY
    (integrator "velocity", optional vertex-face collisions) or
    BACKWARD_EULER_POSITION (integrator "position", Rayleigh damped with
    alpha, beta = rayleigh) or NEWMARK (integrator "newmark")."""

    def __init__(self, scene, tol=1e-8, maxit=1000, precond=0, integrator="velocity", rayleigh=(0.01, 0.01)):
        L = lib()
        self.scene = scene
        self._rest = np.ascontiguousarray(scene.rest, dtype=np.float64)
        self._tets = np.ascontiguousarray(scene.tets, dtype=np.int32)
        g = np.array(scene.gravity, dtype=np.float64)
        self.h = L.oracle_create(scene.nv, scene.nt, _d(self._rest), _i(self._tets),
                                 MATERIALS[scene.material], scene.mu, scene.lam, scene.density,
                                 _d(g), scene.dt)
        assert self.h
        x0 = np.ascontiguousarray(scene.x0.reshape(-1), dtype=np.float64)
        v0 = np.ascontiguousarray(scene.v0.reshape(-1), dtype=np.float64)
        if getattr(scene, "fiber", None) is not None:
            a = np.ascontiguousarray(scene.fiber, dtype=np.float64)
            assert L.oracle_set_fiber(self.h, _d(a)) == 0
        L.oracle_set_state(self.h, _d(x0), _d(v0))
        pins = np.ascontiguousarray(scene.pinned, dtype=np.int32)
        assert L.oracle_attach_pins(self.h, len(pins), _i(pins)) == 0
        L.oracle_set_solver(self.h, tol, maxit, precond)
        if integrator != "velocity":
            code = {"position": 1, "newmark": 2}[integrator]
            assert L.oracle_set_integrator(self.h, code, rayleigh[0], rayleigh[1]) == 0

    def set_green_damping(self, mu):
        """NEWMARK's energy-damped solve with GREEN_DAMPING(mu)."""
        assert lib().oracle_set_green_damping(self.h, float(mu)) == 0

    def set_pin_targets(self, targets):
        """Target displacements of the pinned vertices (scene.pinned order)."""
        t = np.ascontiguousarray(targets, dtype=np.float64).reshape(-1)
        assert lib().oracle_set_pin_targets(self.h, len(t) // 3, _d(t)) == 0

    def ee_pairs(self):
        """Edge-edge pairs of the last step as vertex quadruples
        (edge0[0], edge0[1], edge1[0], edge1[1])."""
        L = lib()
        ne = L.oracle_ee_pairs(self.h, None, None)
        edges = np.zeros(2 * max(ne, 1), dtype=np.int32)
        L.oracle_ee_pairs(self.h, None, _i(edges))
        pairs = np.zeros(2 * max(ne, 1), dtype=np.int32)
        n = L.oracle_ee_pairs(self.h, _i(pairs), None)
        e = edges[:2 * ne].reshape(-1, 2)
        p = pairs[:2 * n].reshape(-1, 2)
        return np.concatenate([e[p[:, 0]], e[p[:, 1]]], axis=1) if n else np.zeros((0, 4), np.int32)

    def set_collisions(self, vf=True, eps=0.01, mu=1.0, beta=0.001, ee=False):
        """Vertex-face (and with ee, edge-edge) self collisions
        (TIMESTEPPER.cpp:83-86 defaults: mu 1, beta 0.001)."""
        assert lib().oracle_set_collisions(self.h, int(bool(vf)) | (2 if ee else 0), eps, mu, beta) == 0

    def vf_pairs(self):
        """(vertex, surface triangle) pairs at the current state, and the surface triangles."""
        L = lib()
        ntri = L.oracle_num_surface_triangles(self.h)
        tris = np.zeros(3 * ntri, dtype=np.int32)
        cap = 1 << 20
        pairs = np.zeros(2 * cap, dtype=np.int32)
        n = L.oracle_vf_pairs(self.h, _i(pairs), cap, _i(tris))
        return pairs[:2 * n].reshape(-1, 2), tris.reshape(-1, 3)

    def vf_response(self):
        """Collision tets, forces and clamped Hessians of the last vf_pairs() detection."""
        pairs, _ = self.vf_pairs()
        n = len(pairs)
        tets = np.zeros(4 * max(n, 1), dtype=np.int32)
        f = np.zeros(12 * max(n, 1))
        H = np.zeros(144 * max(n, 1))
        lib().oracle_vf_response(self.h, _i(tets), _d(f), _d(H))
        return tets[:4 * n].reshape(-1, 4), f[:12 * n].reshape(-1, 12), H[:144 * n].reshape(-1, 144)

    def step(self, n=1):
        iters = np.zeros(n, dtype=np.int32)
        errs = np.zeros(n)
        assert lib().oracle_step(self.h, n, _i(iters), _d(errs)) == 0
        return iters, errs

    def acceleration(self):
        a = np.zeros(3 * self.scene.nv)
        lib().oracle_get_acceleration(self.h, _d(a))
        return a

    def newton_iterations(self) -> int:
        """Newton iterations of the last NEWMARK step."""
        return lib().oracle_newton_iterations(self.h)

    def state(self):
        x = np.zeros(3 * self.scene.nv)
        v = np.zeros(3 * self.scene.nv)
        lib().oracle_get_state(self.h, _d(x), _d(v))
        return x, v

    def assemble(self):
        nb = lib().oracle_nblocks(self.h)
        rowptr = np.zeros(self.scene.nv + 1, dtype=np.int32)
        cols = np.zeros(nb, dtype=np.int32)
        K = np.zeros(9 * nb)
        R = np.zeros(3 * self.scene.nv)
        lib().oracle_assemble(self.h, _i(rowptr), _i(cols), _d(K), _d(R))
        return rowptr, cols, K.reshape(nb, 9), R

    def energy(self):
        return lib().oracle_energy(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_destroy(self.h)
            self.h = None


def bsr_to_dense(rowptr, cols, blocks, nv):
    """Dense 3V x 3V matrix from BSR (blocks column major)."""
    A = np.zeros((3 * nv, 3 * nv))
    for u in range(nv):
        for k in range(rowptr[u], rowptr[u + 1]):
            w = cols[k]
            A[3 * u:3 * u + 3, 3 * w:3 * w + 3] = blocks[k].reshape(3, 3, order="F")
    return A


def csc_to_dense(colptr, rowidx, values, n):
    A = np.zeros((n, n))
    for c in range(n):
        for k in range(colptr[c], colptr[c + 1]):
            A[rowidx[k], c] = values[k]
    return A
