"""Seeded synthetic scenes for the implicit tet-FEM timestep.

Every mesh, initial state and pin set used by the tests, the benchmark and the
oracle fixtures comes from this module, so the GPU path and the CPU oracle see
byte-identical inputs.

Meshes are Kuhn-split cubes: an N x N x N grid of hex cells over [0, 1]^3, each
cell cut into six tets around its main diagonal (corner 000 -> corner 111).  The
reference builds its test meshes by hand (projects/unitTests, data/*.tobj); the
workloads here are the synthetic Kuhn cubes the hot-path configurations name.

Conventions shared with the reference (HOBAK):
  * vertex ids: idx = i + (N+1) * (j + (N+1) * k), x = i h, y = j h, z = k h;
    y is up (gravity is -y), so the "top face" is the layer j = N.
  * tets are (v0, v1, v2, v3) with positive rest volume
    diff3 . (diff1 x diff2) / 6 > 0  (Geometry/TET_MESH.cpp:145-151).
  * state is the displacement from rest, interleaved xyz, like
    TIMESTEPPER::_position (Timestepper/TIMESTEPPER.cpp:105-122).
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional

import numpy as np

BASE_SEED = 20261203

# material kinds; the integer codes are the C ABI's HOBAK_MATERIAL_* values
MATERIALS = {"snh": 0, "arap": 1, "stvk": 2, "linear": 3, "neo_hookean_bw": 4, "snh_barrier": 5,
             "aniso_arap": 6, "aniso_stvk": 7, "aniso_fung": 8, "aniso_dirichlet": 9}
ANISOTROPIC = ("aniso_arap", "aniso_stvk", "aniso_fung", "aniso_dirichlet")
# fibre direction of the anisotropic test scenes (normalised by the material)
FIBER = (0.3, 0.8, -0.52)


def lame(E: float, nu: float):
    """Young's modulus / Poisson ratio -> (mu, lambda).

    Same formulas as HYPERELASTIC::computeMu / computeLambda
    (Hyperelastic/Volume/HYPERELASTIC.cpp:111-122)."""
    mu = E / (2.0 * (1.0 + nu))
    lam = (E * nu) / ((1.0 + nu) * (1.0 - 2.0 * nu))
    return mu, lam


def kuhn_cube(N: int, jitter: float = 0.01, seed: Optional[int] = BASE_SEED):
    """Kuhn-split unit cube with N cells per side.

    Returns (rest [V,3] float64, tets [T,4] int32).  `jitter` perturbs every
    rest vertex by U(-jitter*h, jitter*h) per axis (seeded)."""
    n1 = N + 1
    h = 1.0 / N
    i, j, k = np.meshgrid(np.arange(n1), np.arange(n1), np.arange(n1), indexing="ij")
    # idx = i + n1*(j + n1*k): build in (k, j, i) order
    ii = i.transpose(2, 1, 0).reshape(-1)
    jj = j.transpose(2, 1, 0).reshape(-1)
    kk = k.transpose(2, 1, 0).reshape(-1)
    rest = np.stack([ii * h, jj * h, kk * h], axis=1).astype(np.float64)
    if jitter and seed is not None:
        rng = np.random.default_rng(seed)
        rest = rest + rng.uniform(-jitter * h, jitter * h, size=rest.shape)

    # six tets per cell, one per axis permutation (a, b, c):
    #   000 -> e_a -> e_a + e_b -> 111, odd permutations get v1/v2 swapped
    perms = [((0, 1, 2), +1), ((1, 2, 0), +1), ((2, 0, 1), +1),
             ((0, 2, 1), -1), ((2, 1, 0), -1), ((1, 0, 2), -1)]
    local = []
    for (a, b, c), sign in perms:
        e = np.zeros((4, 3), dtype=np.int64)
        e[1, a] = 1
        e[2, a] = 1
        e[2, b] = 1
        e[3, :] = 1
        if sign < 0:
            e[[1, 2]] = e[[2, 1]]
        local.append(e)
    local = np.stack(local)  # [6, 4, 3] corner offsets

    ci, cj, ck = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    ci = ci.transpose(2, 1, 0).reshape(-1)
    cj = cj.transpose(2, 1, 0).reshape(-1)
    ck = ck.transpose(2, 1, 0).reshape(-1)
    cells = np.stack([ci, cj, ck], axis=1)  # [C, 3] in (k, j, i) order
    corners = cells[:, None, None, :] + local[None, :, :, :]  # [C, 6, 4, 3]
    idx = corners[..., 0] + n1 * (corners[..., 1] + n1 * corners[..., 2])
    tets = idx.reshape(-1, 4).astype(np.int32)
    return rest, tets


def tet_volumes(x: np.ndarray, tets: np.ndarray) -> np.ndarray:
    d1 = x[tets[:, 1]] - x[tets[:, 0]]
    d2 = x[tets[:, 2]] - x[tets[:, 0]]
    d3 = x[tets[:, 3]] - x[tets[:, 0]]
    return np.einsum("ij,ij->i", d3, np.cross(d1, d2)) / 6.0


def top_layer(N: int) -> np.ndarray:
    """Vertex ids of the j = N layer (the pinned top face)."""
    n1 = N + 1
    k, i = np.meshgrid(np.arange(n1), np.arange(n1), indexing="ij")
    return (i.reshape(-1) + n1 * (N + n1 * k.reshape(-1))).astype(np.int32)


def compress_and_twist(rest: np.ndarray, N: int, squash: float = 0.6,
                       max_deg: float = 15.0, seed: int = BASE_SEED + 1):
    """Deformed start: y <- squash*y, then each j-layer is rotated about the
    vertical axis through the cube centre by a seeded U(-max_deg, max_deg)."""
    n1 = N + 1
    rng = np.random.default_rng(seed)
    theta = np.deg2rad(rng.uniform(-max_deg, max_deg, size=n1))
    x = rest.copy()
    x[:, 1] *= squash
    layer = (np.arange(rest.shape[0]) // n1) % n1
    c, s = np.cos(theta[layer]), np.sin(theta[layer])
    dx = x[:, 0] - 0.5
    dz = x[:, 2] - 0.5
    x[:, 0] = 0.5 + c * dx + s * dz
    x[:, 2] = 0.5 - s * dx + c * dz
    return x


def random_rotation(rng) -> np.ndarray:
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, a, b, c = q
    return np.array([[1 - 2 * (b * b + c * c), 2 * (a * b - c * w), 2 * (a * c + b * w)],
                     [2 * (a * b + c * w), 1 - 2 * (a * a + c * c), 2 * (b * c - a * w)],
                     [2 * (a * c - b * w), 2 * (b * c + a * w), 1 - 2 * (a * a + b * b)]])


@dataclasses.dataclass
class Scene:
    """One timestep job: mesh, material, pins, initial displacement/velocity."""
    name: str
    rest: np.ndarray          # [V, 3] float64 rest positions
    tets: np.ndarray          # [T, 4] int32
    material: str             # key of MATERIALS
    mu: float
    lam: float
    pinned: np.ndarray        # [P] int32 vertex ids
    x0: np.ndarray            # [V, 3] initial displacement from rest
    v0: np.ndarray            # [V, 3] initial velocity
    density: float = 1000.0
    gravity: tuple = (0.0, -9.8, 0.0)
    dt: float = 1.0 / 60.0
    N: int = 0
    fiber: Optional[tuple] = None  # anisotropic energies: fibre direction a

    @property
    def nv(self) -> int:
        return int(self.rest.shape[0])

    @property
    def nt(self) -> int:
        return int(self.tets.shape[0])


def config1_scene(N: int = 10, material: str = "snh") -> Scene:
    """Plain FP64 CPU-runnable case: 10^3 Kuhn cube, SNH E=1e3 nu=0.45, top pinned."""
    rest, tets = kuhn_cube(N)
    mu, lam = lame(1e3, 0.45)
    zeros = np.zeros_like(rest)
    return Scene(f"kuhn{N}_{material}", rest, tets, material, mu, lam, top_layer(N),
                 zeros.copy(), zeros.copy(), N=N)


def config2_scene(N: int = 40, material: str = "snh") -> Scene:
    """FP64-at-scale case: 40^3 Kuhn cube, E=1e4 nu=0.45, compressed 0.6 in y and
    twisted +-15 deg per layer; pins attached in that deformed state."""
    rest, tets = kuhn_cube(N)
    mu, lam = lame(1e4, 0.45)
    x = compress_and_twist(rest, N)
    return Scene(f"kuhn{N}_{material}_twist", rest, tets, material, mu, lam, top_layer(N),
                 x - rest, np.zeros_like(rest), N=N)


def aniso_scene(N: int = 6, material: str = "aniso_arap", fiber=FIBER) -> Scene:
    """An anisotropic energy (ANISOTROPIC_ARAP / STVK / FUNG / DIRICHLET, with
    mu from E = 1e4, nu = 0.45 and fibre direction `fiber`) on the compressed
    and twisted Kuhn cube of config2_scene, top layer pinned, no gravity: the
    cube springs back along the fibre."""
    s = config2_scene(N, "snh")
    s.name = f"kuhn{N}_{material}_twist"
    s.material = material
    s.fiber = tuple(float(c) for c in fiber)
    s.gravity = (0.0, 0.0, 0.0)
    return s


def config4_scenes(count: int = 256, nmin: int = 6, nmax: int = 24,
                   seed: int = BASE_SEED + 4) -> List[Scene]:
    """Batched mix: N ~ U{nmin..nmax}, random rotation, SNH/ARAP 50/50,
    mu ~ logU[1e2, 1e5], nu ~ U[0.3, 0.48], top face (in the cube frame) pinned."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(count):
        N = int(rng.integers(nmin, nmax + 1))
        rest, tets = kuhn_cube(N, seed=seed + 1000 + s)
        R = random_rotation(rng)
        rest = (rest - 0.5) @ R.T + 0.5
        material = "snh" if rng.random() < 0.5 else "arap"
        mu = float(math.exp(rng.uniform(math.log(1e2), math.log(1e5))))
        nu = float(rng.uniform(0.3, 0.48))
        lam = 2.0 * mu * nu / (1.0 - 2.0 * nu)
        zeros = np.zeros_like(rest)
        out.append(Scene(f"mix{s}_n{N}_{material}", rest, tets, material, mu, lam,
                         top_layer(N), zeros.copy(), zeros.copy(), N=N))
    return out


def two_cubes_scene(N: int = 8, gap: float = 5e-4, offset: float = 0.1, material: str = "snh",
                    E: float = 1e4, nu: float = 0.45, jitter: float = 0.002, seed: int = BASE_SEED + 5) -> Scene:
    """Two Kuhn cubes in one mesh, the upper one resting `gap` above the lower
    one and shifted by `offset` in x and z, so their faces start inside the
    vertex-face collision distance.  The lower cube's bottom face (j = 0) is
    pinned; contact between the cubes is vertex-face self collision."""
    rest_a, tets_a = kuhn_cube(N, jitter=jitter, seed=seed)
    rest_b, tets_b = kuhn_cube(N, jitter=jitter, seed=seed + 1)
    rest_b = rest_b + np.array([offset, 1.0 + gap, offset])
    rest = np.concatenate([rest_a, rest_b])
    tets = np.concatenate([tets_a, tets_b + len(rest_a)]).astype(np.int32)
    n1 = N + 1
    k, i = np.meshgrid(np.arange(n1), np.arange(n1), indexing="ij")
    bottom = (i.reshape(-1) + n1 * (0 + n1 * k.reshape(-1))).astype(np.int32)
    mu, lam = lame(E, nu)
    zeros = np.zeros_like(rest)
    return Scene(f"two_cubes{N}_{material}", rest, tets, material, mu, lam, bottom, zeros.copy(), zeros.copy(), N=N)


# vertex-face contact of the serving mix: collision distance, spring stiffness,
# damping beta (TIMESTEPPER.cpp:86 default)
SERVE_CONTACT = (1e-3, 1e3, 0.001)


def config5_jobs(count: int = 64, nmin: int = 8, nmax: int = 32, smin: int = 10, smax: int = 200,
                 seed: int = BASE_SEED + 6):
    """Serving mix: jobs of N ~ U{nmin..nmax} cells per side running
    U{smin..smax} steps.  Even jobs are two SNH cubes in one mesh (lower bottom
    face pinned, upper cube 0.1 offset, resting 5e-4 above it, so contact is on
    from the first step) with vertex-face contact SERVE_CONTACT; odd jobs are
    single cubes drawn like the batched mix (random rotation, SNH/ARAP,
    log-uniform mu).  Returns [(scene, nsteps, contact or None)]."""
    rng = np.random.default_rng(seed)
    out = []
    for j in range(count):
        N = int(rng.integers(nmin, nmax + 1))
        steps = int(rng.integers(smin, smax + 1))
        if j % 2 == 0:
            sc = two_cubes_scene(N, seed=seed + 1000 + 2 * j)
            sc.name = f"serve{j}_two_cubes{N}"
            out.append((sc, steps, SERVE_CONTACT))
        else:
            sc = config4_scenes(1, N, N, seed=seed + 1000 + 2 * j)[0]
            sc.name = f"serve{j}_n{N}_{sc.material}"
            out.append((sc, steps, None))
    return out
