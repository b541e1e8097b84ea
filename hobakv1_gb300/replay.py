"""Scene record/replay in the reference's JSON scene format, and the
reference's scene-regression driver, on top of the GPU timesteppers.

The format is HOBAK's (FILE_IO.cpp:393-540, JSON_SCENE.h): a "scene" object
with the frame-independent settings (camera, gravity, mesh file name, initial
transform, dt, collision flags and constants, material name, kinematic
shapes) and a "frames" array with, per simulated frame, "frameNumber",
"position" (displacement from rest), "positionOld", "velocity",
"externalForces" (3*nv each) and the collision pairs flattened as
[first, second, ...].  Files ending in ".gz" are gzip-compressed.  3x3
matrices are written flattened in Eigen's column-major order.

`scene_regression` follows regressionTests.cpp:45-102: step a scene frame by
frame and compare its displacement against the recorded frames with a
relative L2 tolerance (1e-8 there).
"""
from __future__ import annotations

import gzip
import json
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import hobak


# ---------------------------------------------------------------- mesh files

def read_tobj(path: str):
    """TET_MESH::readTobjFile (TET_MESH.cpp:1177-1230): "v x y z" vertex
    lines, then "t a b c d" tet lines (0-based ids)."""
    verts, tets = [], []
    with open(path) as f:
        for line in f:
            p = line.split()
            if not p:
                continue
            if p[0] == "v":
                verts.append([float(c) for c in p[1:4]])
            elif p[0] == "t":
                tets.append([int(c) for c in p[1:5]])
    return np.array(verts, dtype=np.float64), np.array(tets, dtype=np.int32)


# ---------------------------------------------------------- kinematic shapes

class KINEMATIC_SHAPE:
    """A rigid kinematic shape: world = rotation * scale * local + translation
    (KINEMATIC_SHAPE.h:55-69).  Subclasses define inside(local test)."""

    name = "KINEMATIC_SHAPE"

    def __init__(self, translation, scale: float = 1.0):
        self._translation = np.array(translation, dtype=np.float64)
        self._scale = np.eye(3) * float(scale)
        self._rotation = np.eye(3)
        self._scaleInverse = np.linalg.inv(self._scale)

    def translation(self) -> np.ndarray:
        """Mutable like the reference's translation() reference."""
        return self._translation

    def rotation(self) -> np.ndarray:
        return self._rotation

    def scale(self) -> np.ndarray:
        return self._scale

    def localVertexToWorld(self, local) -> np.ndarray:
        return self._rotation @ self._scale @ np.asarray(local, dtype=np.float64) + self._translation

    def worldVertexToLocal(self, world) -> np.ndarray:
        return self._scaleInverse @ self._rotation.T @ (np.asarray(world, dtype=np.float64) - self._translation)

    def localNormalToWorld(self, normal) -> np.ndarray:
        return self._rotation @ np.asarray(normal, dtype=np.float64)

    def to_json(self) -> dict:
        flat = lambda m: [float(v) for v in np.asarray(m).reshape(-1, order="F")]
        return {"name": self.name, "translation": [float(v) for v in self._translation],
                "scale": flat(self._scale), "scaleInverse": flat(self._scaleInverse),
                "rotation": flat(self._rotation)}

    @staticmethod
    def from_json(d: dict) -> "KINEMATIC_SHAPE":
        kinds = {"CUBE": CUBE}
        if d["name"] not in kinds:
            raise ValueError(f"kinematic shape {d['name']!r} is not supported")
        s = kinds[d["name"]]((0.0, 0.0, 0.0), 1.0)
        m = lambda k: np.asarray(d[k], dtype=np.float64).reshape(3, 3, order="F")
        s._translation = np.asarray(d["translation"], dtype=np.float64)
        s._scale, s._scaleInverse, s._rotation = m("scale"), m("scaleInverse"), m("rotation")
        return s


class CUBE(KINEMATIC_SHAPE):
    """Unit cube [-0.5, 0.5]^3 in local coordinates (CUBE.cpp:27-55)."""

    name = "CUBE"

    def inside(self, point) -> bool:
        p = self.worldVertexToLocal(point)
        return bool(np.all(p <= 0.5) and np.all(p >= -0.5))


# ------------------------------------------------------------- JSON records

@dataclass
class SceneRecord:
    """A scene JSON file in memory: settings plus per-frame state arrays."""
    scene: dict
    frameNumber: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    position: np.ndarray = field(default_factory=lambda: np.zeros((0, 0)))
    positionOld: np.ndarray = field(default_factory=lambda: np.zeros((0, 0)))
    velocity: np.ndarray = field(default_factory=lambda: np.zeros((0, 0)))
    externalForces: np.ndarray = field(default_factory=lambda: np.zeros((0, 0)))
    vertexFaceCollisions: list = field(default_factory=list)  # per frame: [(vertex, face), ...]
    edgeEdgeCollisions: list = field(default_factory=list)    # per frame: [(edge, edge), ...]
    frameIndex: Optional[np.ndarray] = None  # which frames the rows hold (None: all, in order)
    recordedFrames: Optional[int] = None     # frames in the original record (None: the rows)

    def totalFrames(self) -> int:
        return int(self.recordedFrames if self.recordedFrames is not None else len(self.frameNumber))

    def row(self, frame: int) -> Optional[int]:
        """Row holding frame `frame` (0-based), or None when not kept."""
        if self.frameIndex is None:
            return frame if frame < len(self.frameNumber) else None
        hit = np.nonzero(self.frameIndex == frame)[0]
        return int(hit[0]) if len(hit) else None

    def kinematicShapes(self):
        return [KINEMATIC_SHAPE.from_json(d) for d in self.scene.get("kinematicShapes", [])]


def _pairs(flat):
    a = np.asarray(flat, dtype=np.int64).reshape(-1, 2)
    return [(int(p), int(q)) for p, q in a]


def read_scene_json(path: str) -> SceneRecord:
    """readSceneJSON (FILE_IO.cpp:480-620); ".gz" files are read through gzip
    directly instead of the reference's copy-and-gunzip."""
    opener = gzip.open if path.endswith(".gz") else open
    with opener(path, "rt") as f:
        doc = json.load(f)
    if "scene" not in doc:
        raise ValueError(f"{path}: no 'scene' object")
    frames = doc.get("frames", [])
    rec = SceneRecord(scene=doc["scene"])
    if frames:
        arr = lambda k: np.array([fr[k] for fr in frames], dtype=np.float64)
        rec.frameNumber = np.array([fr["frameNumber"] for fr in frames], dtype=np.int64)
        rec.position, rec.positionOld = arr("position"), arr("positionOld")
        rec.velocity, rec.externalForces = arr("velocity"), arr("externalForces")
        rec.vertexFaceCollisions = [_pairs(fr.get("vertexFaceCollisions", [])) for fr in frames]
        rec.edgeEdgeCollisions = [_pairs(fr.get("edgeEdgeCollisions", [])) for fr in frames]
    return rec


class SceneRecorder:
    """initializeSceneJSON / recordFrameToJSON / writeSceneJSON
    (FILE_IO.cpp:393-470) for a SIMULATION_SCENE below."""

    def __init__(self, scene: "SIMULATION_SCENE"):
        s, solver = scene, scene.solver()
        v3 = lambda v: [float(c) for c in np.asarray(v, dtype=np.float64).reshape(3)]
        self.scene = {
            "eye": v3(s.eye), "lookAt": v3(s.lookAt), "up": v3(s.up), "worldCenter": v3(s.worldCenter),
            "gravity": v3(s.gravity), "pauseFrame": int(s.pauseFrame), "arrowCounter": int(s.arrowCounter),
            "drawFeature": bool(s.drawFeature), "tetMeshFilename": s.tetMeshFilename,
            "normalizedVertices": bool(s.normalizedVertices),
            "initialA": [float(c) for c in np.asarray(s.initialA).reshape(-1, order="F")],
            "initialTranslation": v3(s.initialTranslation),
            "dt": float(solver.dt()),
            "vertexFaceSelfCollisionsOn": bool(solver.vertexFaceSelfCollisionsOn()),
            "edgeEdgeSelfCollisionsOn": bool(s.edgeEdgeSelfCollisionsOn),
            "collisionStiffness": float(solver.collisionStiffness()),
            "collisionDampingBeta": float(solver.collisionDampingBeta()),
            "materialName": s.materialName,
            "kinematicShapes": [k.to_json() for k in s.kinematicShapes],
        }
        self.frames: list = []

    def record_frame(self, scene: "SIMULATION_SCENE"):
        solver = scene.solver()
        lst = lambda a: [float(c) for c in np.asarray(a, dtype=np.float64).reshape(-1)]
        flat = lambda pairs: [int(c) for pq in pairs for c in pq]
        self.frames.append({
            "frameNumber": int(scene.frameNumber),
            "position": lst(solver.position()), "positionOld": lst(scene.positionOld),
            "velocity": lst(solver.velocity()), "externalForces": lst(solver.externalForces()),
            "vertexFaceCollisions": flat(scene.vertexFaceCollisions()),
            "edgeEdgeCollisions": [],
        })

    def write(self, path: str):
        opener = gzip.open if path.endswith(".gz") else open
        with opener(path, "wt") as f:
            json.dump({"scene": self.scene, "frames": self.frames}, f)


# ------------------------------------------------------------------- scenes

class SIMULATION_SCENE:
    """The parts of SIMULATION_SCENE (SIMULATION_SCENE.h:40-200) that a
    headless run needs: build, step, and the fields the JSON record keeps."""

    def __init__(self, opts: Optional[hobak.HobakSolverOpts] = None):
        self.opts = opts
        self.sceneName = ""
        self.tetMeshFilename = ""
        self.eye = np.zeros(3)
        self.lookAt = np.zeros(3)
        self.up = np.array([0.0, 1.0, 0.0])
        self.worldCenter = np.zeros(3)
        self.gravity = np.zeros(3)  # SIMULATION_SCENE.h:60
        self.pauseFrame = -2
        self.arrowCounter = -1
        self.drawFeature = False
        self.frameNumber = 0
        self.normalizedVertices = False
        self.initialA = np.eye(3)
        self.initialTranslation = np.zeros(3)
        self.edgeEdgeSelfCollisionsOn = False
        self.materialName = ""
        self.kinematicShapes: list = []
        self.tetMesh: Optional[hobak.TET_MESH] = None
        self._solver = None
        self.positionOld = None

    def solver(self):
        return self._solver

    def vertexFaceCollisions(self):
        return []

    def buildScene(self) -> bool:
        raise NotImplementedError

    def stepSimulation(self, verbose: bool = False):
        """The default step (SIMULATION_SCENE.h:118-125): f_ext = M g, solve."""
        self._solve(verbose)
        self.frameNumber += 1

    def _solve(self, verbose):
        s = self._solver
        self.positionOld = s.position().copy()
        s.externalForces()[:] = 0.0
        s.addGravity(self.gravity)
        s.solve(verbose)


class NEWMARK_STRETCH(SIMULATION_SCENE):
    """NEWMARK_STRETCH.h: a 10x10x10-cell cube (cube_10.tobj), SNH(1, 10),
    NEWMARK, the surface vertices inside two unit CUBEs pinned to them; the
    first cube moves 0.01 along -z on frames 2..24, stretching the block.
    The mesh comes in as arrays (the reference reads ../data/cube_10.tobj).
    The reference leaves its self-collision flags on; the block never
    touches itself (no pairs in any recorded frame), so the GPU NEWMARK,
    which has no contact, takes the same steps."""

    def __init__(self, rest: np.ndarray, tets: np.ndarray, opts: Optional[hobak.HobakSolverOpts] = None):
        super().__init__(opts)
        self._rest, self._tets = rest, tets

    def buildScene(self) -> bool:
        self.sceneName = "newmark_stretch"
        self.tetMeshFilename = "../data/cube_10.tobj"
        self.tetMesh = hobak.TET_MESH(self._rest, self._tets)
        self.materialName = "SNH"
        self._solver = hobak.NEWMARK(self.tetMesh, hobak.SNH(1.0, 10.0), self.opts)
        self.kinematicShapes = [CUBE((0.56, 0.48, -0.24), 1.0), CUBE((0.56, 0.48, 1.23), 1.0)]
        self._solver.attachKinematicSurfaceConstraints(self.kinematicShapes[0])
        self._solver.attachKinematicSurfaceConstraints(self.kinematicShapes[1])
        self.eye = np.array([-1.73357, 0.953765, 0.471698])
        self.lookAt = np.array([-0.749345, 0.790722, 0.402909])
        self.up = np.array([0.160779, 0.986286, -0.0372856])
        self.pauseFrame = 75
        self.edgeEdgeSelfCollisionsOn = True  # the reference's default; this scene never collides
        return True

    def stepSimulation(self, verbose: bool = False):
        if 1 < self.frameNumber < 25:  # cubeMotion
            self.kinematicShapes[0].translation()[2] -= 0.01
        self._solve(verbose)
        self.frameNumber += 1


def compute_mu(E: float, nu: float) -> float:
    """HYPERELASTIC::computeMu (HYPERELASTIC.cpp:111-114)."""
    return E / (2.0 * (1.0 + nu))


def compute_lambda(E: float, nu: float) -> float:
    """HYPERELASTIC::computeLambda (HYPERELASTIC.cpp:119-122)."""
    return (E * nu) / ((1.0 + nu) * (1.0 - 2.0 * nu))


class _TWO_TET_VF(SIMULATION_SCENE):
    """The two-tet contact scenes: BACKWARD_EULER_POSITION at dt = 1/30, the
    surface vertices inside the kinematic cubes pinned, vertex-face or
    edge-edge self collisions on.  The reference also registers the
    lower cube as a collision object (addKinematicCollisionObject, plane
    constraints); in these scenes no free vertex ever enters it, so that part
    never acts and is not built."""

    mesh_file = ""
    material = None        # hobak material class
    E = nu = 0.0
    gravity_y = 0.0
    shapes = ()            # ((center), scale) of each pinning cube
    collision_eps = 0.01   # TET_MESH default (TET_MESH.cpp:70)
    rayleigh = None        # (alpha, beta), None: the integrator's default
    pause = 0
    vf, ee = True, False   # which self collisions

    def __init__(self, rest: np.ndarray, tets: np.ndarray, opts: Optional[hobak.HobakSolverOpts] = None):
        super().__init__(opts)
        self._rest, self._tets = rest, tets

    def collision_mu(self, mu: float) -> float:
        raise NotImplementedError

    def buildScene(self) -> bool:
        self.tetMeshFilename = self.mesh_file
        self.gravity = np.array([0.0, self.gravity_y, 0.0])
        mu, lam = compute_mu(self.E, self.nu), compute_lambda(self.E, self.nu)
        self.tetMesh = hobak.TET_MESH(self._rest, self._tets)
        self.materialName = self.material.NAME
        solver = hobak.BACKWARD_EULER_POSITION(self.tetMesh, self.material(mu, lam), self.opts)
        self._solver = solver
        solver.setDt(1.0 / 30.0)
        solver.setCollisionEps(self.collision_eps)
        self.kinematicShapes = [CUBE(c, sc) for c, sc in self.shapes]
        for shape in self.kinematicShapes:
            solver.attachKinematicSurfaceConstraints(shape)
        if self.rayleigh is not None:
            solver.setRayleigh(*self.rayleigh)
        solver.setCollisionStiffness(self.collision_mu(mu))
        solver.setCollisionDampingBeta(0.01)
        solver.setVertexFaceSelfCollisionsOn(self.vf)
        solver.setEdgeEdgeSelfCollisionsOn(self.ee)
        self.edgeEdgeSelfCollisionsOn = self.ee
        self.eye = np.array([-2.13557, 0.947023, 2.39579])
        self.lookAt = np.array([-1.35707, 0.964614, 1.76839])
        self.up = np.array([-0.00368317, 0.999718, 0.0234604])
        self.pauseFrame = self.pause
        return True

    def vertexFaceCollisions(self):
        b = self._solver._batch
        return [] if b is None or not self.vf else [tuple(p) for p in b.collision_pairs(0)[0]]

    def edgeEdgeQuads(self):
        """The last step's edge-edge pairs as vertex quadruples."""
        b = self._solver._batch
        return np.zeros((0, 4), np.int32) if b is None or not self.ee else b.edge_pairs(0)


class TWO_TET_DROP_VF(_TWO_TET_VF):
    """TWO_TET_DROP_VF.h: a tet dropped (gravity 0.3) onto a pinned one,
    SNH(E = 3, nu = 0.45), collision stiffness 10."""
    mesh_file = "../data/two_tets_vertex_face.tobj"
    material = hobak.SNH
    E, nu, gravity_y = 3.0, 0.45, -0.3
    shapes = (((0.0, -4.90, 0.0), 10.0),)
    pause = 200

    def collision_mu(self, mu):
        return 10.0

    def buildScene(self) -> bool:
        self.sceneName = "two_tet_drop_vf"
        return super().buildScene()


class TWO_TET_KISS_VF(_TWO_TET_VF):
    """TWO_TET_KISS_VF.h: two pinned tets barely touching at a vertex and a
    face, ARAP(E = 10, nu = 0.45), collision distance 0.03, stiffness 10 mu,
    no Rayleigh damping."""
    mesh_file = "../data/two_tets_vertex_face_kiss.tobj"
    material = hobak.ARAP
    E, nu, gravity_y = 10.0, 0.45, 0.0
    shapes = (((0.0, -4.90, 0.0), 10.0), ((0.0, 6.9, 0.0), 10.0))
    collision_eps = 0.03
    rayleigh = (0.0, 0.0)
    pause = 100

    def collision_mu(self, mu):
        return mu * 10.0

    def buildScene(self) -> bool:
        self.sceneName = "two_tet_kiss_vf"
        return super().buildScene()


class TWO_TET_DROP_EE(_TWO_TET_VF):
    """TWO_TET_DROP_EE.h: a tet dropped edge-first (gravity 0.3) onto a
    pinned one, SNH(E = 1, nu = 0.45), edge-edge collisions, stiffness 10."""
    mesh_file = "../data/two_tets_edge_edge.tobj"
    material = hobak.SNH
    E, nu, gravity_y = 1.0, 0.45, -0.3
    shapes = (((0.0, -4.90, 0.0), 10.0),)
    pause = 200
    vf, ee = False, True

    def collision_mu(self, mu):
        return 10.0

    def buildScene(self) -> bool:
        self.sceneName = "two_tet_drop_ee"
        return super().buildScene()


class TWO_TET_KISS_EE(_TWO_TET_VF):
    """TWO_TET_KISS_EE.h: two pinned tets whose edges barely touch,
    ARAP(E = 1, nu = 0.45), collision distance 0.03, stiffness 1000, no
    Rayleigh damping."""
    mesh_file = "../data/two_tets_edge_edge_kiss.tobj"
    material = hobak.ARAP
    E, nu, gravity_y = 1.0, 0.45, 0.0
    shapes = (((0.0, -4.90, 0.0), 10.0), ((0.0, 6.9, 0.0), 10.0))
    collision_eps = 0.03
    rayleigh = (0.0, 0.0)
    pause = 30
    vf, ee = False, True

    def collision_mu(self, mu):
        return 1000.0

    def buildScene(self) -> bool:
        self.sceneName = "two_tet_kiss_ee"
        return super().buildScene()


# --------------------------------------------------------------- regression

def scene_regression(scene: SIMULATION_SCENE, truth: SceneRecord, tol: float = 1e-8,
                     frames: Optional[int] = None, noise_floor: float = 1e-12):
    """sceneRegression (regressionTests.cpp:45-102): build the scene, step it
    once per recorded frame and compare the displacement against the frame
    with relative L2 error <= tol.  A frame whose recorded displacement is
    below noise_floor in norm (the rounding residue of an unforced step) is
    compared absolutely against noise_floor instead.  Returns (ok, errors)."""
    scene.buildScene()
    n = truth.totalFrames() if frames is None else min(frames, truth.totalFrames())
    errors = []
    ok = True
    for k in range(n):
        scene.stepSimulation(False)
        r = truth.row(k)
        if r is None:
            continue
        x = scene.solver().position()
        g = truth.position[r]
        gn, dn = float(np.linalg.norm(g)), float(np.linalg.norm(x - g))
        err = dn / gn if gn > noise_floor else dn
        bound = tol if gn > noise_floor else noise_floor
        errors.append(err)
        ok = ok and err <= bound
    return ok, np.array(errors)
