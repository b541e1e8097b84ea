"""Python mirror of HOBAK's hot-path interfaces over the GB300 C ABI.

Class and method names follow the reference so code written against it reads
the same:

  * VOLUME::HYPERELASTIC and its energies (Hyperelastic/Volume/HYPERELASTIC.h:31-64):
    SNH, ARAP, STVK, LINEAR, NEO_HOOKEAN_BW, SNH_WITH_BARRIER and the
    anisotropic ANISOTROPIC_ARAP, ANISOTROPIC_STVK, ANISOTROPIC_FUNG,
    ANISOTROPIC_DIRICHLET with psi / PK1 / hessian / clampedHessian (from F or
    from (U, Sigma, V)), energyNeedsSVD / PK1NeedsSVD, evaluated on the GPU
    in batches.
  * TET_MESH (Geometry/TET_MESH.h): rest vertices, tets, displacement.
  * TIMESTEPPER::BACKWARD_EULER_VELOCITY (Timestepper/BACKWARD_EULER_VELOCITY.h:35-58):
    position() / velocity() / externalForces() host state, setDt, addGravity,
    attachKinematicConstraints, scaleMass, solve(verbose).
  * BATCH: many scenes stepped together (hobak_batch_*).

Matrices use numpy's [i, j] indexing; the C ABI's column-major flatten order
(util/MATRIX_UTIL.cpp:33-43) is applied at the boundary.
"""
from __future__ import annotations

import ctypes
from typing import Iterable, Optional, Sequence

import numpy as np

from . import _lib
from ._lib import HobakMaterial, HobakSceneDesc, HobakSolverOpts, HobakStepStats, check, dptr, iptr

PRECISION_FP64 = 0
PRECISION_MIXED = 1
PRECOND_JACOBI = 0
PRECOND_BLOCK_JACOBI = 1
INTEGRATOR_VELOCITY = 0   # BACKWARD_EULER_VELOCITY::solve
INTEGRATOR_POSITION = 1   # BACKWARD_EULER_POSITION::solveRayleighDamped
INTEGRATOR_NEWMARK = 2    # NEWMARK::solveRayleighDamped (Newton loop)


def _colmajor(F: np.ndarray) -> np.ndarray:
    F = np.asarray(F, dtype=np.float64)
    single = F.ndim == 2
    F = F.reshape(-1, 3, 3)
    return np.ascontiguousarray(F.transpose(0, 2, 1).reshape(-1, 9)), single


class HYPERELASTIC:
    """Base of the volume energies; (mu, lambda) are the reference constructor
    arguments (the SNH reparameterisation happens in the library)."""
    KIND = -1
    NAME = "HYPERELASTIC"
    fiber = None

    def __init__(self, mu: float, lam: float):
        self.mu = float(mu)
        self.lam = float(lam)

    def name(self) -> str:
        return self.NAME

    def _c(self) -> HobakMaterial:
        a = self.fiber if self.fiber is not None else (0.0, 0.0, 0.0)
        return HobakMaterial(self.KIND, self.mu, self.lam, (ctypes.c_double * 3)(*a))

    def energyNeedsSVD(self) -> bool:
        """HYPERELASTIC::energyNeedsSVD (HYPERELASTIC.h:56)."""
        e, p = ctypes.c_int(), ctypes.c_int()
        check(_lib.load().hobak_material_needs_svd(self.KIND, ctypes.byref(e), ctypes.byref(p)),
              "hobak_material_needs_svd")
        return bool(e.value)

    def PK1NeedsSVD(self) -> bool:
        """HYPERELASTIC::PK1NeedsSVD (HYPERELASTIC.h:59)."""
        e, p = ctypes.c_int(), ctypes.c_int()
        check(_lib.load().hobak_material_needs_svd(self.KIND, ctypes.byref(e), ctypes.byref(p)),
              "hobak_material_needs_svd")
        return bool(p.value)

    @staticmethod
    def computeMu(E: float, nu: float) -> float:
        """HYPERELASTIC::computeMu (HYPERELASTIC.cpp:111-115)."""
        return E / (2.0 * (1.0 + nu))

    @staticmethod
    def computeLambda(E: float, nu: float) -> float:
        """HYPERELASTIC::computeLambda (HYPERELASTIC.cpp:117-122)."""
        return (E * nu) / ((1.0 + nu) * (1.0 - 2.0 * nu))

    def _eval(self, F, want_psi=False, want_P=False, want_H=False):
        Fc, single = _colmajor(F)
        n = Fc.shape[0]
        psi = np.zeros(n) if want_psi else None
        P = np.zeros((n, 9)) if want_P else None
        H = np.zeros((n, 81)) if want_H else None
        mat = self._c()
        check(_lib.load().hobak_material_eval(ctypes.byref(mat), n, dptr(Fc), dptr(psi), dptr(P), dptr(H)),
              "hobak_material_eval")
        return psi, P, H, single

    def psi(self, F):
        """Strain energy density psi(F)."""
        psi, _, _, single = self._eval(F, want_psi=True)
        return float(psi[0]) if single else psi

    def PK1(self, F):
        """First Piola-Kirchhoff stress, [..., 3, 3]."""
        _, P, _, single = self._eval(F, want_P=True)
        P = P.reshape(-1, 3, 3).transpose(0, 2, 1)
        return P[0] if single else P

    def clampedHessian(self, F, Sigma=None, V=None):
        """d2psi/dF2 projected to PSD, 9x9 in flatten() order, [..., 9, 9];
        clampedHessian(U, Sigma, V) with three arguments."""
        if Sigma is not None:
            return self._eval_svd(F, Sigma, V)[3]
        _, _, H, single = self._eval(F, want_H=True)
        H = H.reshape(-1, 9, 9).transpose(0, 2, 1)
        return H[0] if single else H

    def hessian(self, F, Sigma=None, V=None):
        """The unclamped d2psi/dF2 (HYPERELASTIC.h:44-45), 9x9 in flatten()
        order; hessian(U, Sigma, V) with three arguments."""
        if Sigma is not None:
            return self._eval_svd(F, Sigma, V)[2]
        Fc, single = _colmajor(F)
        n = Fc.shape[0]
        H = np.zeros((n, 81))
        mat = self._c()
        check(_lib.load().hobak_material_hessian(ctypes.byref(mat), n, dptr(Fc), dptr(H)), "hobak_material_hessian")
        H = H.reshape(-1, 9, 9).transpose(0, 2, 1)
        return H[0] if single else H

    def _eval_svd(self, U, Sigma, V):
        """psi, PK1, hessian, clampedHessian of the (U, Sigma, V) overloads."""
        Uc, single = _colmajor(U)
        Vc, _ = _colmajor(V)
        S = np.ascontiguousarray(np.asarray(Sigma, dtype=np.float64).reshape(-1, 3))
        n = Uc.shape[0]
        psi, P, H, Hc = np.zeros(n), np.zeros((n, 9)), np.zeros((n, 81)), np.zeros((n, 81))
        mat = self._c()
        check(_lib.load().hobak_material_eval_svd(ctypes.byref(mat), n, dptr(Uc), dptr(S), dptr(Vc), dptr(psi),
                                                  dptr(P), dptr(H), dptr(Hc)), "hobak_material_eval_svd")
        P = P.reshape(-1, 3, 3).transpose(0, 2, 1)
        H = H.reshape(-1, 9, 9).transpose(0, 2, 1)
        Hc = Hc.reshape(-1, 9, 9).transpose(0, 2, 1)
        if single:
            return float(psi[0]), P[0], H[0], Hc[0]
        return psi, P, H, Hc

    def psi_svd(self, U, Sigma, V):
        """psi(U, Sigma, V) (HYPERELASTIC.h:37)."""
        return self._eval_svd(U, Sigma, V)[0]

    def PK1_svd(self, U, Sigma, V):
        """PK1(U, Sigma, V) (HYPERELASTIC.h:41)."""
        return self._eval_svd(U, Sigma, V)[1]


class SNH(HYPERELASTIC):
    KIND, NAME = 0, "SNH"


class ARAP(HYPERELASTIC):
    KIND, NAME = 1, "ARAP"


class STVK(HYPERELASTIC):
    KIND, NAME = 2, "STVK"


class LINEAR(HYPERELASTIC):
    KIND, NAME = 3, "LINEAR"


class NEO_HOOKEAN_BW(HYPERELASTIC):
    KIND, NAME = 4, "NEO_HOOKEAN_BW"


class SNH_WITH_BARRIER(HYPERELASTIC):
    KIND, NAME = 5, "SNH_WITH_BARRIER"


class ANISOTROPIC(HYPERELASTIC):
    """Base of the anisotropic energies: constructed as (mu, a) like
    ANISOTROPIC_ARAP(mu, a) (ANISOTROPIC_ARAP.h:28); the library normalises a."""

    def __init__(self, mu: float, a):
        super().__init__(mu, 0.0)
        self.fiber = tuple(float(c) for c in np.asarray(a, dtype=np.float64).reshape(3))


class ANISOTROPIC_ARAP(ANISOTROPIC):
    KIND, NAME = 6, "ANISOTROPIC_ARAP"


class ANISOTROPIC_STVK(ANISOTROPIC):
    KIND, NAME = 7, "ANISOTROPIC_STVK"


class ANISOTROPIC_FUNG(ANISOTROPIC):
    KIND, NAME = 8, "ANISOTROPIC_FUNG"


class ANISOTROPIC_DIRICHLET(ANISOTROPIC):
    KIND, NAME = 9, "ANISOTROPIC_DIRICHLET"


MATERIAL_CLASSES = {"snh": SNH, "arap": ARAP, "stvk": STVK, "linear": LINEAR,
                    "neo_hookean_bw": NEO_HOOKEAN_BW, "snh_barrier": SNH_WITH_BARRIER,
                    "aniso_arap": ANISOTROPIC_ARAP, "aniso_stvk": ANISOTROPIC_STVK,
                    "aniso_fung": ANISOTROPIC_FUNG, "aniso_dirichlet": ANISOTROPIC_DIRICHLET}


def make_material(name: str, mu: float, lam: float, fiber=None) -> HYPERELASTIC:
    """The material class of a scene: (mu, lambda) for the isotropic energies,
    (mu, fiber) for the anisotropic ones."""
    cls = MATERIAL_CLASSES[name]
    if issubclass(cls, ANISOTROPIC):
        return cls(mu, fiber if fiber is not None else (1.0, 0.0, 0.0))
    return cls(mu, lam)


class TET_MESH:
    """Rest mesh plus current displacement (Geometry/TET_MESH.h)."""

    def __init__(self, restVertices: np.ndarray, tets: np.ndarray):
        self._rest = np.ascontiguousarray(restVertices, dtype=np.float64).reshape(-1, 3)
        self._tets = np.ascontiguousarray(tets, dtype=np.int32).reshape(-1, 4)
        self._disp = np.zeros_like(self._rest)
        d1 = self._rest[self._tets[:, 1]] - self._rest[self._tets[:, 0]]
        d2 = self._rest[self._tets[:, 2]] - self._rest[self._tets[:, 0]]
        d3 = self._rest[self._tets[:, 3]] - self._rest[self._tets[:, 0]]
        self._restVolumes = np.einsum("ij,ij->i", d3, np.cross(d1, d2)) / 6.0
        if (self._restVolumes <= 0).any():
            raise ValueError("TET_MESH: tets must have positive rest volume")
        self._oneRing = np.zeros(len(self._rest))
        np.add.at(self._oneRing, self._tets.reshape(-1), np.repeat(0.25 * self._restVolumes, 4))

    def restVertices(self):
        return self._rest

    def tets(self):
        return self._tets

    def vertices(self):
        return self._rest + self._disp

    def totalVertices(self) -> int:
        return len(self._rest)

    def surfaceVertices(self):
        """Vertices of the boundary triangles (tet faces that belong to one
        tet only), ascending like TET_MESH::computeSurfaceVertices
        (TET_MESH.cpp:567-590)."""
        t = self._tets
        faces = np.concatenate([t[:, [0, 1, 2]], t[:, [0, 1, 3]], t[:, [0, 2, 3]], t[:, [1, 2, 3]]])
        uniq, count = np.unique(np.sort(faces, axis=1), axis=0, return_counts=True)
        return np.unique(uniq[count == 1]).astype(np.int64)

    def DOFs(self) -> int:
        return 3 * len(self._rest)

    def restOneRingVolumes(self):
        return self._oneRing

    def setDisplacement(self, delta):
        self._disp = np.asarray(delta, dtype=np.float64).reshape(-1, 3).copy()

    def getDisplacement(self):
        return self._disp.reshape(-1).copy()

    def computeElements(self, material: HYPERELASTIC):
        """Per-tet F, Sigma, element force (12) and element Hessian (12x12) on
        the GPU at the current displacement."""
        nt, nv = len(self._tets), len(self._rest)
        F, S = np.zeros((nt, 9)), np.zeros((nt, 3))
        f, H = np.zeros((nt, 12)), np.zeros((nt, 144))
        x = np.ascontiguousarray(self._disp.reshape(-1))
        mat = material._c()
        check(_lib.load().hobak_element_eval(nv, nt, dptr(self._rest), iptr(self._tets), dptr(x),
                                             ctypes.byref(mat), dptr(F), dptr(S), dptr(f), dptr(H)),
              "hobak_element_eval")
        return {"F": F, "Sigma": S, "force": f, "hessian": H}


def solver_opts(tol=1e-8, max_iters=1000, precision=PRECISION_FP64, preconditioner=PRECOND_BLOCK_JACOBI,
                max_refinements=3, use_graph=True, integrator=INTEGRATOR_VELOCITY,
                rayleigh=(0.01, 0.01), max_newton=10, newton_tolerance=1e-7, inner_tolerance=1e-5) -> HobakSolverOpts:
    """Solver options; integrator INTEGRATOR_VELOCITY (BACKWARD_EULER_VELOCITY),
    INTEGRATOR_POSITION (BACKWARD_EULER_POSITION, Rayleigh damped with
    alpha, beta = rayleigh) or INTEGRATOR_NEWMARK (NEWMARK, at most
    max_newton Newton iterations until |rhs|^2 <= newton_tolerance)."""
    o = HobakSolverOpts()
    o.tol, o.max_iters, o.precision = tol, max_iters, precision
    o.preconditioner, o.max_refinements, o.use_graph = preconditioner, max_refinements, int(use_graph)
    o.integrator = integrator
    o.rayleigh_alpha, o.rayleigh_beta = rayleigh
    o.max_newton, o.newton_tolerance = max_newton, newton_tolerance
    o.inner_tolerance = inner_tolerance
    return o


class _SceneArrays:
    """Keeps the numpy buffers a HobakSceneDesc points into alive."""

    def __init__(self, rest, tets, material, density, gravity, dt, pinned, x0, v0):
        self.rest = np.ascontiguousarray(rest, dtype=np.float64).reshape(-1)
        self.tets = np.ascontiguousarray(tets, dtype=np.int32).reshape(-1)
        self.pinned = np.ascontiguousarray(pinned if pinned is not None else [], dtype=np.int32)
        self.x0 = np.ascontiguousarray(x0, dtype=np.float64).reshape(-1) if x0 is not None else None
        self.v0 = np.ascontiguousarray(v0, dtype=np.float64).reshape(-1) if v0 is not None else None
        d = HobakSceneDesc()
        d.nv, d.nt = len(self.rest) // 3, len(self.tets) // 4
        d.rest, d.tets = dptr(self.rest), iptr(self.tets)
        d.material = material._c()
        d.density = float(density)
        d.gravity = (ctypes.c_double * 3)(*[float(g) for g in gravity])
        d.dt = float(dt)
        d.npinned = len(self.pinned)
        d.pinned = iptr(self.pinned) if len(self.pinned) else None
        d.x0, d.v0 = dptr(self.x0), dptr(self.v0)
        self.desc = d


class BATCH:
    """Many scenes packed into one device-resident batch (hobak_batch_*)."""

    def __init__(self, scenes: Sequence, opts: Optional[HobakSolverOpts] = None):
        L = _lib.load()
        self._arrays = [_SceneArrays(s.rest, s.tets,
                                     make_material(s.material, s.mu, s.lam, getattr(s, "fiber", None)), s.density,
                                     s.gravity, s.dt, s.pinned, s.x0, s.v0) for s in scenes]
        descs = (HobakSceneDesc * len(self._arrays))(*[a.desc for a in self._arrays])
        self.nv = [len(a.rest) // 3 for a in self._arrays]
        self.opts = opts if opts is not None else solver_opts()
        h = ctypes.c_void_p()
        check(L.hobak_batch_create(descs, len(self._arrays), ctypes.byref(self.opts), ctypes.byref(h)),
              "hobak_batch_create")
        self.h = h
        self.last_stats = None
        self.last_status = 0

    def __len__(self):
        return len(self._arrays)

    @property
    def total_vertices(self) -> int:
        return int(sum(self.nv))

    def offsets(self):
        """First index of every scene in the whole-batch (3 * total vertices) vectors."""
        return np.concatenate([[0], np.cumsum([3 * n for n in self.nv])])

    def step(self, nsteps: int = 1):
        stats = (HobakStepStats * len(self))()
        self.last_status = check(_lib.load().hobak_batch_step(self.h, nsteps, stats), "hobak_batch_step")
        self.last_stats = [(s.iterations, s.converged, s.rel_residual, s.refinements) for s in stats]
        return self.last_stats

    def step_async(self, nsteps: int = 1):
        check(_lib.load().hobak_batch_step_async(self.h, nsteps), "hobak_batch_step_async")

    def wait(self):
        stats = (HobakStepStats * len(self))()
        self.last_status = check(_lib.load().hobak_batch_wait(self.h, stats), "hobak_batch_wait")
        self.last_stats = [(s.iterations, s.converged, s.rel_residual, s.refinements) for s in stats]
        return self.last_stats

    # ---- whole batch at once (scene order, 3 * total vertices) ----
    def set_state_all(self, x: np.ndarray, v: np.ndarray):
        """Enqueue the upload of every scene's displacement and velocity; the
        arrays must stay unchanged until the next step/wait/get returns."""
        self._pending_in = (x, v)  # keep the buffers alive until then
        check(_lib.load().hobak_batch_set_state_all(self.h, dptr(x), dptr(v)), "hobak_batch_set_state_all")

    def set_external_forces_all(self, f: np.ndarray):
        self._pending_f = f
        check(_lib.load().hobak_batch_set_external_forces_all(self.h, dptr(f)), "hobak_batch_set_external_forces_all")

    def get_state_all(self, x: Optional[np.ndarray] = None, v: Optional[np.ndarray] = None):
        n = 3 * self.total_vertices
        x = np.empty(n) if x is None else x
        v = np.empty(n) if v is None else v
        check(_lib.load().hobak_batch_get_state_all(self.h, dptr(x), dptr(v)), "hobak_batch_get_state_all")
        return x, v

    def get_acceleration(self, scene: int) -> np.ndarray:
        """NEWMARK's acceleration state of one scene (3*nv)."""
        a = np.empty(3 * self.nv[scene])
        check(_lib.load().hobak_batch_get_acceleration(self.h, scene, dptr(a)), "hobak_batch_get_acceleration")
        return a

    def set_acceleration(self, scene: int, a: np.ndarray):
        a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
        check(_lib.load().hobak_batch_set_acceleration(self.h, scene, dptr(a)), "hobak_batch_set_acceleration")

    def set_pin_targets(self, scene: int, targets):
        """Target displacements (world - rest) of one scene's pinned vertices,
        3 per pin in the scene's pinned order, from the next step on."""
        t = np.ascontiguousarray(targets, dtype=np.float64).reshape(-1)
        check(_lib.load().hobak_batch_set_pin_targets(self.h, scene, dptr(t)), "hobak_batch_set_pin_targets")

    def snapshot_bytes(self) -> int:
        n = ctypes.c_size_t(0)
        check(_lib.load().hobak_batch_snapshot_bytes(self.h, ctypes.byref(n)), "hobak_batch_snapshot_bytes")
        return int(n.value)

    def snapshot(self, dst_ptr: Optional[int] = None) -> Optional[np.ndarray]:
        """The batch's dynamic state as bytes on the host, or written to the
        device (or host) address dst_ptr of snapshot_bytes() bytes."""
        n = self.snapshot_bytes()
        if dst_ptr is not None:
            check(_lib.load().hobak_batch_snapshot(self.h, ctypes.c_void_p(dst_ptr), n), "hobak_batch_snapshot")
            return None
        buf = np.empty(n, dtype=np.uint8)
        check(_lib.load().hobak_batch_snapshot(self.h, buf.ctypes.data_as(ctypes.c_void_p), n),
              "hobak_batch_snapshot")
        return buf

    def restore(self, snap=None, src_ptr: Optional[int] = None, nbytes: Optional[int] = None):
        """Restore from snapshot() bytes, or from a host/device address."""
        if src_ptr is not None:
            n = nbytes if nbytes is not None else self.snapshot_bytes()
            check(_lib.load().hobak_batch_restore(self.h, ctypes.c_void_p(src_ptr), n), "hobak_batch_restore")
            return
        buf = np.ascontiguousarray(snap, dtype=np.uint8)
        check(_lib.load().hobak_batch_restore(self.h, buf.ctypes.data_as(ctypes.c_void_p), buf.size),
              "hobak_batch_restore")

    def query(self) -> bool:
        """True when the batch's enqueued steps have finished (non-blocking)."""
        return check(_lib.load().hobak_batch_query(self.h), "hobak_batch_query") == 1

    def set_active(self, scene: int, active: bool = True):
        """Park (False) or resume one scene; parked scenes keep their state."""
        check(_lib.load().hobak_batch_set_active(self.h, scene, int(active)), "hobak_batch_set_active")

    def get_state(self, scene: int):
        n = 3 * self.nv[scene]
        x, v = np.zeros(n), np.zeros(n)
        check(_lib.load().hobak_batch_get_state(self.h, scene, dptr(x), dptr(v)), "hobak_batch_get_state")
        return x, v

    def set_state(self, scene: int, x=None, v=None):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1) if x is not None else None
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(-1) if v is not None else None
        check(_lib.load().hobak_batch_set_state(self.h, scene, dptr(x), dptr(v)), "hobak_batch_set_state")

    def set_external_forces(self, scene: int, f):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        check(_lib.load().hobak_batch_set_external_forces(self.h, scene, dptr(f)), "hobak_batch_set_external_forces")

    def set_solver(self, opts: HobakSolverOpts):
        self.opts = opts
        check(_lib.load().hobak_batch_set_solver(self.h, ctypes.byref(opts)), "hobak_batch_set_solver")

    def device_bytes(self) -> int:
        b = ctypes.c_longlong()
        check(_lib.load().hobak_batch_device_bytes(self.h, ctypes.byref(b)), "hobak_batch_device_bytes")
        return b.value

    def energy(self, scene: int) -> float:
        e = ctypes.c_double()
        check(_lib.load().hobak_batch_energy(self.h, scene, ctypes.byref(e)), "hobak_batch_energy")
        return e.value

    def assemble(self, scene: int):
        """BSR pattern, K blocks (column major) and R at the current state."""
        L = _lib.load()
        nb = ctypes.c_int()
        check(L.hobak_batch_assemble(self.h, scene, ctypes.byref(nb), None, None, None, None), "hobak_batch_assemble")
        rowptr = np.zeros(self.nv[scene] + 1, dtype=np.int32)
        cols = np.zeros(nb.value, dtype=np.int32)
        K = np.zeros(9 * nb.value)
        R = np.zeros(3 * self.nv[scene])
        check(L.hobak_batch_assemble(self.h, scene, None, iptr(rowptr), iptr(cols), dptr(K), dptr(R)),
              "hobak_batch_assemble")
        return rowptr, cols, K.reshape(-1, 9), R

    def set_collisions(self, scene: int, vf: bool = True, eps: float = 0.01, stiffness: float = 1.0,
                       damping_beta: float = 0.001):
        """Vertex-face self collisions of one scene (TIMESTEPPER.h:62-69 flags,
        TET_MESH::setCollisionEps)."""
        check(_lib.load().hobak_batch_set_collisions(self.h, scene, int(vf), eps, stiffness, damping_beta),
              "hobak_batch_set_collisions")

    def collision_pairs(self, scene: int, detect_now: bool = False):
        """(vertex, surface triangle) pairs (scene-local ids, sorted) and the
        scene's surface triangles."""
        L = _lib.load()
        n, nt = ctypes.c_int(), ctypes.c_int()
        check(L.hobak_batch_collision_pairs(self.h, scene, int(detect_now), ctypes.byref(n), None, 0,
                                            ctypes.byref(nt), None), "hobak_batch_collision_pairs")
        pairs = np.zeros(2 * max(n.value, 1), dtype=np.int32)
        tris = np.zeros(3 * max(nt.value, 1), dtype=np.int32)
        check(L.hobak_batch_collision_pairs(self.h, scene, 0, ctypes.byref(n), iptr(pairs), n.value,
                                            ctypes.byref(nt), iptr(tris)), "hobak_batch_collision_pairs")
        return pairs[:2 * n.value].reshape(-1, 2), tris[:3 * nt.value].reshape(-1, 3)

    def set_edge_collisions(self, scene: int, on: bool = True):
        """Edge-edge self collisions (edgeEdgeSelfCollisionsOn) with the
        scene's collision distance, stiffness and damping."""
        check(_lib.load().hobak_batch_set_edge_collisions(self.h, scene, int(on)), "hobak_batch_set_edge_collisions")

    def edge_pairs(self, scene: int) -> np.ndarray:
        """Edge-edge pairs of the last detection, [n, 4] scene-local vertex ids."""
        L = _lib.load()
        n = ctypes.c_int(0)
        check(L.hobak_batch_edge_pairs(self.h, scene, ctypes.byref(n), None, 0), "hobak_batch_edge_pairs")
        q = np.zeros(4 * max(n.value, 1), dtype=np.int32)
        check(L.hobak_batch_edge_pairs(self.h, scene, ctypes.byref(n), iptr(q), n.value), "hobak_batch_edge_pairs")
        return q[:4 * n.value].reshape(-1, 4)

    def collision_response(self, scene: int):
        """Collision tets, forces (-w grad psi) and clamped Hessians of the last detection."""
        pairs, _ = self.collision_pairs(scene)
        n = len(pairs)
        tets = np.zeros(4 * max(n, 1), dtype=np.int32)
        f = np.zeros(12 * max(n, 1))
        H = np.zeros(144 * max(n, 1))
        check(_lib.load().hobak_batch_collision_response(self.h, scene, n, iptr(tets), dptr(f), dptr(H)),
              "hobak_batch_collision_response")
        return tets[:4 * n].reshape(-1, 4), f[:12 * n].reshape(-1, 12), H[:144 * n].reshape(-1, 144)

    # ---- measurement ----
    KERNELS = ("element", "assemble", "spmv", "pcg_update")
    PHASES = ("element", "assembly", "pcg_init", "pcg_iterations", "update")

    def stream_handle(self) -> int:
        p = ctypes.c_void_p()
        check(_lib.load().hobak_batch_get_stream(self.h, ctypes.byref(p)), "hobak_batch_get_stream")
        return p.value or 0

    def enable_timing(self, on: bool = True):
        check(_lib.load().hobak_batch_enable_timing(self.h, int(on)), "hobak_batch_enable_timing")

    def phase_times(self):
        ms = np.zeros(5)
        n = (ctypes.c_longlong * 5)()
        check(_lib.load().hobak_batch_phase_times(self.h, dptr(ms), n), "hobak_batch_phase_times")
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(self.PHASES)}

    def launch_count(self) -> int:
        n = ctypes.c_longlong()
        check(_lib.load().hobak_batch_launch_count(self.h, ctypes.byref(n)), "hobak_batch_launch_count")
        return n.value

    def time_kernels(self, reps: int = 20):
        ms = np.zeros(4)
        check(_lib.load().hobak_batch_time_kernels(self.h, reps, dptr(ms)), "hobak_batch_time_kernels")
        return dict(zip(self.KERNELS, ms.tolist()))

    def kernel_bytes(self):
        b = np.zeros(4)
        check(_lib.load().hobak_batch_kernel_bytes(self.h, dptr(b)), "hobak_batch_kernel_bytes")
        return dict(zip(self.KERNELS, b.tolist()))

    TUNING = ("tile_vertices", "element_threads", "assembly_threads", "pcg_chunk", "cluster_pcg", "cluster_max",
              "step_ms")

    def get_tuning(self) -> dict:
        """Launch shapes: tile size, element / assembly CTA sizes, PCG chunk."""
        t = _lib.HobakTuning()
        check(_lib.load().hobak_batch_get_tuning(self.h, ctypes.byref(t)), "hobak_batch_get_tuning")
        return {k: getattr(t, k) for k in self.TUNING}

    def set_green_damping(self, scene: int, mu: float):
        """NEWMARK's energy-damped solve with GREEN_DAMPING(mu) for one scene
        (NEWMARK batches only; mu = 0 turns it off)."""
        check(_lib.load().hobak_batch_set_green_damping(self.h, scene, float(mu)), "hobak_batch_set_green_damping")

    def pcg_path(self) -> np.ndarray:
        """Per scene: CTAs of the cluster that solves its inner PCG (0: the tile path)."""
        out = np.zeros(len(self), dtype=np.int32)
        check(_lib.load().hobak_batch_pcg_path(self.h, iptr(out)), "hobak_batch_pcg_path")
        return out

    def set_scene_cluster(self, scene: int, ctas: int):
        """Per-scene PCG path: a cluster of ctas CTAs (1..16), -1 the tile
        path, 0 by the batch's tuning."""
        check(_lib.load().hobak_batch_set_scene_cluster(self.h, scene, int(ctas)), "hobak_batch_set_scene_cluster")

    def blocks(self, scene: int) -> int:
        """3x3 blocks of one scene's system matrix (its BSR pattern)."""
        n = ctypes.c_int()
        check(_lib.load().hobak_batch_assemble(self.h, scene, ctypes.byref(n), None, None, None, None),
              "hobak_batch_assemble")
        return n.value

    def set_tuning(self, **kw):
        cur = self.get_tuning()
        cur.update(kw)
        t = _lib.HobakTuning(*[cur[k] for k in self.TUNING])
        check(_lib.load().hobak_batch_set_tuning(self.h, ctypes.byref(t)), "hobak_batch_set_tuning")

    def autotune(self, reps: int = 3) -> dict:
        """Time candidate launch shapes on this batch and keep the fastest
        (state restored afterwards; the trajectory is unchanged)."""
        t = _lib.HobakTuning()
        check(_lib.load().hobak_batch_autotune(self.h, reps, ctypes.byref(t)), "hobak_batch_autotune")
        return {k: getattr(t, k) for k in self.TUNING}

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            _lib.load().hobak_batch_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BACKWARD_EULER_VELOCITY:
    """GPU drop-in for TIMESTEPPER::BACKWARD_EULER_VELOCITY.

    Host-side position() (displacement), velocity() and externalForces() stay
    the source of truth like the reference's mutable references
    (TIMESTEPPER.h:44-58): solve() uploads them, takes one step on the GPU and
    downloads the new state.  Settings (dt, pins, mass scale) are frozen at the
    first solve()."""

    def __init__(self, tetMesh: TET_MESH, hyperelastic: HYPERELASTIC, opts: Optional[HobakSolverOpts] = None):
        self._mesh = tetMesh
        self._material = hyperelastic
        self._opts = opts if opts is not None else solver_opts()
        n = tetMesh.DOFs()
        self._position = tetMesh.getDisplacement()
        self._velocity = np.zeros(n)
        self._externalForces = np.zeros(n)
        self._dt = 1.0 / 60.0  # BACKWARD_EULER_VELOCITY.cpp:37
        self._massScale = 1.0
        self._pinned: list = []
        self._shapePins: dict = {}  # vertex -> (shape, local position) for pins that follow a shape
        self._pinnedAt = None       # displacement of each pin when the GPU state was built
        self._batch: Optional[BATCH] = None
        self._currentTimestep = 0
        self._lastStats = None
        # contact flags (TIMESTEPPER.cpp:83-86 defaults)
        self._vertexFaceSelfCollisionsOn = False
        self._edgeEdgeSelfCollisionsOn = False
        self._collisionStiffness = 1.0
        self._collisionDampingBeta = 0.001
        self._collisionEps = 0.01  # TET_MESH's default collision distance

    # ---- reference accessors ----
    def vertexFaceSelfCollisionsOn(self) -> bool:
        return self._vertexFaceSelfCollisionsOn

    def setVertexFaceSelfCollisionsOn(self, on: bool):
        self._vertexFaceSelfCollisionsOn = bool(on)
        self._push_collisions()

    def edgeEdgeSelfCollisionsOn(self) -> bool:
        return self._edgeEdgeSelfCollisionsOn

    def setEdgeEdgeSelfCollisionsOn(self, on: bool):
        self._edgeEdgeSelfCollisionsOn = bool(on)
        self._push_collisions()

    def collisionStiffness(self) -> float:
        return self._collisionStiffness

    def setCollisionStiffness(self, mu: float):
        self._collisionStiffness = float(mu)
        self._push_collisions()

    def collisionDampingBeta(self) -> float:
        return self._collisionDampingBeta

    def setCollisionDampingBeta(self, beta: float):
        self._collisionDampingBeta = float(beta)
        self._push_collisions()

    def setCollisionEps(self, eps: float):
        """TET_MESH::setCollisionEps (TET_MESH.cpp:2160-2165)."""
        self._collisionEps = float(eps)
        self._push_collisions()

    def _push_collisions(self):
        if self._batch is None:
            return
        check(_lib.load().hobak_gpu_set_collisions(self._batch.h, int(self._vertexFaceSelfCollisionsOn),
                                                   self._collisionEps, self._collisionStiffness,
                                                   self._collisionDampingBeta), "hobak_gpu_set_collisions")
        check(_lib.load().hobak_gpu_set_edge_collisions(self._batch.h, int(self._edgeEdgeSelfCollisionsOn)),
              "hobak_gpu_set_edge_collisions")

    def position(self):
        return self._position

    def velocity(self):
        return self._velocity

    def externalForces(self):
        return self._externalForces

    def dt(self):
        return self._dt

    def setDt(self, dt: float):
        self._require_unbuilt("setDt")
        self._dt = float(dt)

    def scaleMass(self, scalar: float):
        """M *= scalar (TIMESTEPPER.h:100)."""
        self._require_unbuilt("scaleMass")
        self._massScale *= float(scalar)

    def addGravity(self, bodyForce):
        """f_ext += oneRingVolume * bodyForce (TIMESTEPPER.cpp:334-345)."""
        g = np.asarray(bodyForce, dtype=np.float64).reshape(1, 3)
        self._externalForces += (self._mesh.restOneRingVolumes()[:, None] * g).reshape(-1)

    def attachKinematicConstraints(self, vertices: Iterable[int]):
        """Pin vertices at their current positions (TIMESTEPPER.cpp:380-403).
        Takes vertex ids, or a kinematic shape (inside(point); with
        worldVertexToLocal/localVertexToWorld, like KINEMATIC_SHAPE, the pins
        follow the shape when it moves between solves)."""
        self._require_unbuilt("attachKinematicConstraints")
        if hasattr(vertices, "inside"):
            self._attach_shape(vertices, range(self._mesh.totalVertices()))
        else:
            ids = [int(i) for i in vertices]
            self._pinned.extend(ids)

    def attachKinematicSurfaceConstraints(self, shape):
        """Pin the surface vertices inside a kinematic shape to it
        (TIMESTEPPER.cpp:350-375)."""
        self._require_unbuilt("attachKinematicSurfaceConstraints")
        self._attach_shape(shape, self._mesh.surfaceVertices())

    def _attach_shape(self, shape, candidates):
        verts = self._mesh.restVertices() + self._position.reshape(-1, 3)
        movable = hasattr(shape, "worldVertexToLocal") and hasattr(shape, "localVertexToWorld")
        for i in candidates:
            p = verts[int(i)]
            if not shape.inside(p):
                continue
            self._pinned.append(int(i))
            if movable:  # later constraints on a vertex override earlier ones (TIMESTEPPER.cpp:105-122)
                self._shapePins[int(i)] = (shape, np.asarray(shape.worldVertexToLocal(p), dtype=np.float64))

    def constrainedNodes(self):
        return sorted(set(self._pinned))

    def _push_pin_targets(self):
        """applyKinematicConstraints: each shape-held pin's target is
        localVertexToWorld(local) - rest for the shape's current transform."""
        if not self._shapePins:
            return
        pins = self.constrainedNodes()
        rest = self._mesh.restVertices()
        t = np.empty((len(pins), 3))
        for k, u in enumerate(pins):
            if u in self._shapePins:
                shape, local = self._shapePins[u]
                t[k] = np.asarray(shape.localVertexToWorld(local), dtype=np.float64) - rest[u]
            else:
                t[k] = self._pinnedAt[k]
        self._batch.set_pin_targets(0, t)

    def _require_unbuilt(self, what):
        if self._batch is not None:
            raise RuntimeError(f"{what}: the GPU state is built at the first solve(); call it before")

    def _build(self):
        class _S:  # scene record for BATCH
            pass
        s = _S()
        s.rest, s.tets = self._mesh.restVertices(), self._mesh.tets()
        s.material = [k for k, c in MATERIAL_CLASSES.items() if c is type(self._material)][0]
        s.mu, s.lam = self._material.mu, self._material.lam
        s.fiber = self._material.fiber
        s.density, s.gravity, s.dt = self._massScale, (0.0, 0.0, 0.0), self._dt
        s.pinned = np.array(sorted(set(self._pinned)), dtype=np.int32)
        s.x0, s.v0 = self._position, self._velocity
        self._pinnedAt = self._position.reshape(-1, 3)[s.pinned].copy()
        self._batch = BATCH([s], self._opts)
        if self._vertexFaceSelfCollisionsOn or self._edgeEdgeSelfCollisionsOn:
            self._push_collisions()

    def solve(self, verbose: bool = False) -> bool:
        if self._batch is None:
            self._build()
        b = self._batch
        b.set_state(0, self._position, self._velocity)
        self._push_pin_targets()
        check(_lib.load().hobak_gpu_set_external_forces(b.h, dptr(np.ascontiguousarray(self._externalForces))),
              "hobak_gpu_set_external_forces")
        stats = b.step(1)
        x, v = b.get_state(0)
        self._position[:] = x
        self._velocity[:] = v
        self._currentTimestep += 1
        self._lastStats = stats[0]
        if verbose:
            print(f"  PCG iters: {stats[0][0]:3d} err: {stats[0][2]:6.4e}")
        return True

    def lastSolveStats(self):
        return self._lastStats


class BACKWARD_EULER_POSITION(BACKWARD_EULER_VELOCITY):
    """GPU drop-in for TIMESTEPPER::BACKWARD_EULER_POSITION with Rayleigh
    damping (BACKWARD_EULER_POSITION.cpp:138-330): the same host-state
    semantics; the solve's unknown is the position update and
    C = alpha M + beta K(rest).  Vertex-face contact works as for
    BACKWARD_EULER_VELOCITY (forces in b, beta H_coll / dt + H_coll in A)."""

    def __init__(self, tetMesh: TET_MESH, hyperelastic: HYPERELASTIC, opts: Optional[HobakSolverOpts] = None):
        super().__init__(tetMesh, hyperelastic, None if opts is None else HobakSolverOpts.from_buffer_copy(opts))
        self._opts.integrator = INTEGRATOR_POSITION
        if opts is None:
            self._opts.rayleigh_alpha, self._opts.rayleigh_beta = 0.01, 0.01  # BACKWARD_EULER_POSITION.cpp:53-54

    def rayleighAlpha(self) -> float:
        return self._opts.rayleigh_alpha

    def rayleighBeta(self) -> float:
        return self._opts.rayleigh_beta

    def setRayleigh(self, alpha: float, beta: float):
        self._require_unbuilt("setRayleigh")
        self._opts.rayleigh_alpha, self._opts.rayleigh_beta = float(alpha), float(beta)



class GREEN_DAMPING:
    """VOLUME::GREEN_DAMPING(mu) (Damping/Volume/GREEN_DAMPING.h): the damping
    of NEWMARK's energy-damped solve; psi = mu |sym(Fdot^T F)|^2,
    PK1 = mu F (F^T Fdot + Fdot^T F) (GREEN_DAMPING.cpp:36-50)."""

    def __init__(self, mu: float):
        self.mu = float(mu)

    def name(self) -> str:
        return "GREEN_DAMPING"


class NEWMARK(BACKWARD_EULER_VELOCITY):
    """GPU drop-in for TIMESTEPPER::NEWMARK (Rayleigh-damped solve,
    NEWMARK.cpp:183-340: a Newton loop of at most maxNewtonIterations() solves,
    beta = 1/4, gamma = 1/2).  position(), velocity() and acceleration() are
    host state that solve() uploads and downloads.  Vertex-face and edge-edge
    contact run inside the Newton loop (NEWMARK.cpp:226-242), as in the
    reference."""

    def __init__(self, tetMesh: TET_MESH, hyperelastic: HYPERELASTIC, damping=None,
                 opts: Optional[HobakSolverOpts] = None):
        if isinstance(damping, HobakSolverOpts):  # NEWMARK(mesh, material, opts)
            damping, opts = None, damping
        super().__init__(tetMesh, hyperelastic, None if opts is None else HobakSolverOpts.from_buffer_copy(opts))
        self._opts.integrator = INTEGRATOR_NEWMARK
        self._acceleration = np.zeros(tetMesh.DOFs())
        # NEWMARK(mesh, material, damping): the energy-damped solve (NEWMARK.cpp:344-420)
        self._damping = damping

    def acceleration(self):
        return self._acceleration

    def maxNewtonIterations(self) -> int:
        return self._opts.max_newton

    def setMaxNewtonIterations(self, n: int):
        self._require_unbuilt("setMaxNewtonIterations")
        self._opts.max_newton = int(n)

    def solve(self, verbose: bool = False) -> bool:
        if self._batch is None:
            self._build()
            if self._damping is not None:
                self._batch.set_green_damping(0, self._damping.mu)
        self._batch.set_acceleration(0, self._acceleration)
        ok = super().solve(verbose)
        self._acceleration[:] = self._batch.get_acceleration(0)
        return ok
