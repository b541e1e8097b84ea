"""GPU parity: the sm_103a kernels, called through the C ABI, against the
reference's golden vectors (tests/golden/) and the CPU oracle."""
import glob
import os

import numpy as np
import pytest

from hobakv1_gb300 import hobak, scenes
from oracle import oracle

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
ELEMENT_FILES = sorted(glob.glob(os.path.join(GOLDEN, "elements_*.npz")))


def relmax(a, b, floor=1e-300):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), floor))


def floors(g):
    mu = float(g["mu"])
    area = float(np.mean(g["restVolume"])) ** (2.0 / 3.0)
    return {"psi": mu, "P": mu, "fe": mu * area, "R": mu * area}


def _mat(path):
    return os.path.basename(path)[len("elements_"):].rsplit("_", 1)[0]


def _material(path, g):
    """The golden file's material (anisotropic ones with their fibre)."""
    return hobak.make_material(_mat(path), float(g["mu"]), float(g["lam"]),
                               g["fiber"] if "fiber" in g.files else None)


@pytest.mark.parametrize("path", ELEMENT_FILES, ids=[os.path.basename(p)[9:-4] for p in ELEMENT_FILES])
def test_element_terms_match_reference(path):
    """Per-element F, sigma, force and 12x12 Hessian within 1e-10 (FP64)."""
    g = np.load(path)
    mesh = hobak.TET_MESH(g["rest"], g["tets"])
    mesh.setDisplacement(g["x"])
    mat = _material(path, g)
    e = mesh.computeElements(mat)
    fl = floors(g)
    assert relmax(e["F"], g["F"]) < 1e-10
    assert relmax(e["Sigma"], g["Sigma"]) < 1e-10
    assert relmax(e["force"], g["fe"], fl["fe"]) < 1e-10
    assert relmax(e["hessian"], g["He"]) < 1e-10


@pytest.mark.parametrize("path", ELEMENT_FILES, ids=[os.path.basename(p)[9:-4] for p in ELEMENT_FILES])
def test_material_interface_matches_reference(path):
    """psi / PK1 / clampedHessian / hessian of the HYPERELASTIC boundary
    within 1e-10, from F (HYPERELASTIC.h:36-48) and from the reference's own
    (U, Sigma, V) (HYPERELASTIC.h:37-49)."""
    g = np.load(path)
    mat = _material(path, g)
    sq = lambda a: a.reshape(-1, 3, 3).transpose(0, 2, 1)  # column-major flatten -> [i, j]
    flat = lambda a, n: a.transpose(0, 2, 1).reshape(-1, n)
    F = sq(g["F"])
    fl = floors(g)
    assert relmax(mat.psi(F), g["psi"], fl["psi"]) < 1e-10
    assert relmax(flat(mat.PK1(F), 9), g["P"], fl["P"]) < 1e-10
    assert relmax(flat(mat.clampedHessian(F), 81), g["H9"]) < 1e-10
    assert relmax(flat(mat.hessian(F), 81), g["H9u"], fl["P"]) < 1e-10
    psi, P, H, Hc = mat._eval_svd(sq(g["U"]), g["Sigma"], sq(g["V"]))
    assert relmax(psi, g["psi"], fl["psi"]) < 1e-10
    assert relmax(flat(P, 9), g["P"], fl["P"]) < 1e-10
    assert relmax(flat(Hc, 81), g["H9"]) < 1e-10
    assert relmax(flat(H, 81), g["H9u"], fl["P"]) < 1e-10


def test_material_needs_svd_flags():
    """energyNeedsSVD / PK1NeedsSVD as each reference class answers them."""
    expect = {"snh": False, "arap": True, "stvk": False, "linear": False, "neo_hookean_bw": False,
              "snh_barrier": False, "aniso_arap": True, "aniso_stvk": True, "aniso_fung": True,
              "aniso_dirichlet": False}
    for name, flag in expect.items():
        m = hobak.make_material(name, 1.0, 1.0)
        assert m.energyNeedsSVD() == flag and m.PK1NeedsSVD() == flag, name


@pytest.mark.parametrize("path", [p for p in ELEMENT_FILES if "_snh_" in p or "_arap_" in p],
                         ids=lambda p: os.path.basename(p))
def test_assembled_stiffness_matches_reference_csc(path):
    """Block pattern bit-exact against the reference CSC; K and R within 1e-10."""
    g = np.load(path)
    s = scenes.Scene("g", g["rest"], g["tets"], _mat(path), float(g["mu"]), float(g["lam"]),
                     np.zeros(0, np.int32), g["x"].reshape(-1, 3), np.zeros_like(g["x"]).reshape(-1, 3),
                     fiber=tuple(g["fiber"]) if "fiber" in g.files else None)
    b = hobak.BATCH([s])
    rowptr, cols, K, R = b.assemble(0)
    nv = s.nv
    pattern = np.zeros((3 * nv, 3 * nv), bool)
    for u in range(nv):
        for k in range(rowptr[u], rowptr[u + 1]):
            pattern[3 * u:3 * u + 3, 3 * cols[k]:3 * cols[k] + 3] = True
    ref = np.zeros_like(pattern)
    cp, ri = g["K_colptr"], g["K_rowidx"]
    for c in range(3 * nv):
        ref[ri[cp[c]:cp[c + 1]], c] = True
    assert np.array_equal(pattern, ref)
    A = oracle.bsr_to_dense(rowptr, cols, K, nv)
    Kref = oracle.csc_to_dense(cp, ri, g["K_values"], 3 * nv)
    assert relmax(A, Kref) < 1e-10
    assert relmax(R, g["R"], floors(g)["R"]) < 1e-10


TRAJ = [("kuhn10_snh", lambda: scenes.config1_scene(10)),
        ("kuhn6_snh_twist", lambda: scenes.config2_scene(6, "snh")),
        ("kuhn6_arap_twist", lambda: scenes.config2_scene(6, "arap"))]
# the anisotropic energies against the reference's trajectories with the
# reference's own (Jacobi) preconditioner; with block Jacobi the 1e-8
# residual test stops elsewhere on these weakly coupled meshes (1.0-1.2e-8
# from the Jacobi trajectories after 40 steps), so block Jacobi is checked
# against the oracle run with the same preconditioner
# (test_anisotropic_and_isotropic_scenes_batched, test_anisotropic_block_jacobi_matches_oracle)
TRAJ_ANISO = [(f"kuhn6_{m}_twist", (lambda m=m: scenes.aniso_scene(6, m))) for m in scenes.ANISOTROPIC]
CASES = [(n, f, p) for n, f in TRAJ for p in (hobak.PRECOND_JACOBI, hobak.PRECOND_BLOCK_JACOBI)] + \
        [(n, f, hobak.PRECOND_JACOBI) for n, f in TRAJ_ANISO]


@pytest.mark.parametrize("name,fn,precond", CASES,
                         ids=[f"{n}-{'jacobi' if p == hobak.PRECOND_JACOBI else 'block'}" for n, _, p in CASES])
def test_trajectory_matches_reference(name, fn, precond):
    """Positions after every 25 of 100 BEV steps within 1e-8 relative (FP64)."""
    g = np.load(os.path.join(GOLDEN, f"traj_{name}.npz"))
    s = fn()
    b = hobak.BATCH([s], hobak.solver_opts(preconditioner=precond))
    stride = int(g["stride"])
    for k in range(1, g["x"].shape[0]):
        b.step(stride)
        x, v = b.get_state(0)
        err = np.linalg.norm(x - g["x"][k]) / np.linalg.norm(g["x"][k])
        assert err < 1e-8, (k, err)
    if precond == hobak.PRECOND_JACOBI:
        # same preconditioner as the reference: iteration counts agree closely
        # (stats count SpMV products; Eigen's iterations() counts one fewer)
        assert abs(b.last_stats[0][0] - (int(g["iters"][-1]) + 1)) <= 2


def test_python_mirror_solve_matches_oracle():
    """BACKWARD_EULER_VELOCITY.solve() with host state, like the reference API."""
    s = scenes.config2_scene(5, "snh")
    mesh = hobak.TET_MESH(s.rest, s.tets)
    mesh.setDisplacement(s.x0)
    bev = hobak.BACKWARD_EULER_VELOCITY(mesh, hobak.SNH(s.mu, s.lam))
    bev.position()[:] = s.x0.reshape(-1)
    bev.scaleMass(s.density)
    bev.attachKinematicConstraints(s.pinned)
    sim = oracle.Sim(s, precond=hobak.PRECOND_BLOCK_JACOBI)  # the GPU default
    for _ in range(5):
        bev.externalForces()[:] = 0.0
        bev.addGravity(np.array(s.gravity) * s.density)
        bev.solve(False)
    sim.step(5)
    x, _ = sim.state()
    assert np.linalg.norm(bev.position() - x) / np.linalg.norm(x) < 1e-9


def test_larger_mesh_matches_oracle_few_steps():
    """16^3 compressed/twisted SNH against the oracle, 5 steps."""
    s = scenes.config2_scene(16, "snh")
    b = hobak.BATCH([s])
    sim = oracle.Sim(s, precond=1)
    b.step(5)
    sim.step(5)
    x, _ = b.get_state(0)
    xo, _ = sim.state()
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-8


@pytest.mark.parametrize("precision,bound", [(hobak.PRECISION_FP64, 1e-8), (hobak.PRECISION_MIXED, 1e-6)],
                         ids=["fp64", "mixed"])
def test_anisotropic_and_isotropic_scenes_batched(precision, bound):
    """Anisotropic energies (k_element_aniso) beside isotropic ones
    (k_element) in one batch: each scene against the oracle, and the
    anisotropic scene's result the same alone and in the batch."""
    mix = [scenes.aniso_scene(6, "aniso_arap"), scenes.config2_scene(5, "snh"), scenes.aniso_scene(5, "aniso_fung")]
    b = hobak.BATCH(mix, hobak.solver_opts(precision=precision))
    b.step(10)
    for i, s in enumerate(mix):
        sim = oracle.Sim(s, precond=hobak.PRECOND_BLOCK_JACOBI)
        sim.step(10)
        x, _ = b.get_state(i)
        xo, _ = sim.state()
        assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < bound, (i, s.name)
    alone = hobak.BATCH([mix[0]], hobak.solver_opts(precision=precision))
    alone.step(10)
    assert np.array_equal(alone.get_state(0)[0], b.get_state(0)[0])


@pytest.mark.parametrize("name,fn", TRAJ_ANISO, ids=[t[0] for t in TRAJ_ANISO])
def test_anisotropic_block_jacobi_matches_oracle(name, fn):
    """Block Jacobi (the GPU default) on the anisotropic scenes against the
    oracle with the same preconditioner, 40 steps, within 1e-10."""
    s = fn()
    b = hobak.BATCH([s])
    sim = oracle.Sim(s, precond=hobak.PRECOND_BLOCK_JACOBI)
    b.step(40)
    sim.step(40)
    x, _ = b.get_state(0)
    xo, _ = sim.state()
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-10
