"""Pins the CPU oracle against golden vectors produced by the reference build
(tests/golden/make_golden.py).  CPU only."""
import glob
import os

import numpy as np
import pytest

from oracle import oracle
from hobakv1_gb300 import scenes

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def relmax(a, b, floor=1e-300):
    """max |a - b| over max(max |b|, floor): relative error with an absolute
    floor for quantities that vanish (stress and energy at rest)."""
    return float(np.abs(a - b).max() / max(np.abs(b).max(), floor))


def natural_floors(g):
    """Scales below which a stress/energy/force is roundoff: mu for psi and P,
    mu * (tet size)^2 for element forces."""
    mu = float(g["mu"])
    area = float(np.mean(g["restVolume"])) ** (2.0 / 3.0)
    return {"psi": mu, "P": mu, "fe": mu * area, "R": mu * area}


ELEMENT_FILES = sorted(glob.glob(os.path.join(GOLDEN, "elements_*.npz")))


@pytest.mark.parametrize("path", ELEMENT_FILES, ids=[os.path.basename(p)[9:-4] for p in ELEMENT_FILES])
def test_oracle_elements_match_reference(path):
    g = np.load(path)
    mat = os.path.basename(path)[len("elements_"):].rsplit("_", 1)[0]
    fiber = g["fiber"] if "fiber" in g.files else None
    o = oracle.elements(g["rest"], g["tets"], g["x"], mat, float(g["mu"]), float(g["lam"]), fiber=fiber)
    # per-element forces and Hessians within 1e-10 relative (FP64); H9u is
    # the unclamped hessian(F) (HYPERELASTIC.h:44)
    floors = natural_floors(g)
    for k in ["F", "psi", "P", "H9", "H9u", "fe", "He"]:
        err = relmax(o[k], g[k], floors.get(k, 1e-300))
        assert err < 1e-10, (k, err)
    # singular values with the svd_rv sign convention
    assert relmax(o["Sigma"], g["Sigma"]) < 1e-10


ASSEMBLY_FILES = [p for p in ELEMENT_FILES if os.path.basename(p).startswith(("elements_arap", "elements_aniso_arap"))]


@pytest.mark.parametrize("path", ASSEMBLY_FILES, ids=lambda p: os.path.basename(p))
def test_oracle_assembly_matches_reference_csc(path):
    g = np.load(path)
    mat = os.path.basename(path)[len("elements_"):].rsplit("_", 1)[0]
    s = scenes.Scene("g", g["rest"], g["tets"], mat, float(g["mu"]), float(g["lam"]),
                     np.zeros(0, np.int32), g["x"].reshape(-1, 3), np.zeros_like(g["x"]).reshape(-1, 3),
                     fiber=tuple(g["fiber"]) if "fiber" in g.files else None)
    sim = oracle.Sim(s)
    rowptr, cols, K, R = sim.assemble()
    nv = s.nv
    # sparsity: the scalar CSC pattern implied by the 3x3 blocks is bit-exact
    A = oracle.bsr_to_dense(rowptr, cols, K, nv)
    pattern = np.zeros((3 * nv, 3 * nv), bool)
    for u in range(nv):
        for k in range(rowptr[u], rowptr[u + 1]):
            w = cols[k]
            pattern[3 * u:3 * u + 3, 3 * w:3 * w + 3] = True
    ref_pattern = np.zeros_like(pattern)
    cp, ri = g["K_colptr"], g["K_rowidx"]
    for c in range(3 * nv):
        ref_pattern[ri[cp[c]:cp[c + 1]], c] = True
    assert np.array_equal(pattern, ref_pattern)
    Kref = oracle.csc_to_dense(cp, ri, g["K_values"], 3 * nv)
    assert relmax(A, Kref) < 1e-10
    assert relmax(R, g["R"], natural_floors(g)["R"]) < 1e-10


@pytest.mark.parametrize("name,scene_fn", [
    ("kuhn10_snh", lambda: scenes.config1_scene(10)),
    ("kuhn6_snh_twist", lambda: scenes.config2_scene(6, "snh")),
    ("kuhn6_arap_twist", lambda: scenes.config2_scene(6, "arap")),
] + [(f"kuhn6_{m}_twist", (lambda m=m: scenes.aniso_scene(6, m))) for m in scenes.ANISOTROPIC])
def test_oracle_trajectory_matches_reference(name, scene_fn):
    g = np.load(os.path.join(GOLDEN, f"traj_{name}.npz"))
    s = scene_fn()
    sim = oracle.Sim(s)
    stride = int(g["stride"])
    for k in range(1, g["x"].shape[0]):
        sim.step(stride)
        x, v = sim.state()
        err = np.linalg.norm(x - g["x"][k]) / np.linalg.norm(g["x"][k])
        assert err < 1e-8, (k, err)


@pytest.mark.parametrize("name,scene_fn", [
    ("kuhn6_snh_twist", lambda: scenes.config2_scene(6, "snh")),
    ("kuhn6_arap_twist", lambda: scenes.config2_scene(6, "arap")),
    ("kuhn8_snh", lambda: scenes.config1_scene(8)),
])
def test_oracle_position_integrator_matches_reference(name, scene_fn):
    """BACKWARD_EULER_POSITION (Rayleigh damped, alpha = beta = 0.01): the
    restatement against the reference's own trajectory, positions and
    velocities, and the iteration count of every step."""
    g = np.load(os.path.join(GOLDEN, f"traj_{name}_position.npz"))
    s = scene_fn()
    a, b = (float(c) for c in g["rayleigh"])
    sim = oracle.Sim(s, integrator="position", rayleigh=(a, b))
    stride = int(g["stride"])
    iters = []
    for k in range(1, g["x"].shape[0]):
        it, _ = sim.step(stride)
        iters.extend(it.tolist())
        x, v = sim.state()
        assert np.linalg.norm(x - g["x"][k]) / np.linalg.norm(g["x"][k]) < 1e-10, k
        assert np.linalg.norm(v - g["v"][k]) / np.linalg.norm(g["v"][k]) < 1e-9, k
    assert np.abs(np.array(iters) - g["iters"]).max() <= 1


@pytest.mark.parametrize("name,scene_fn", [
    ("kuhn6_snh_twist", lambda: scenes.config2_scene(6, "snh")),
    ("kuhn6_arap_twist", lambda: scenes.config2_scene(6, "arap")),
])
def test_oracle_newmark_matches_reference(name, scene_fn):
    """NEWMARK (Newton loop of Rayleigh-damped solves whose C the reference
    zeroes): the restatement against the reference's own trajectory, and the
    last Newton iteration's CG count of every step."""
    g = np.load(os.path.join(GOLDEN, f"traj_{name}_newmark.npz"))
    sim = oracle.Sim(scene_fn(), integrator="newmark")
    stride = int(g["stride"])
    iters = []
    for k in range(1, g["x"].shape[0]):
        it, _ = sim.step(stride)
        iters.extend(it.tolist())
        x, v = sim.state()
        assert np.linalg.norm(x - g["x"][k]) / np.linalg.norm(g["x"][k]) < 1e-10, k
        assert np.linalg.norm(v - g["v"][k]) / np.linalg.norm(g["v"][k]) < 1e-9, k
    assert np.abs(np.array(iters) - g["iters"]).max() <= 1


def test_oracle_vertex_face_collisions_match_reference():
    """Surface triangles bit-exact; vertex-face pair sets bit-exact at every
    recorded state; the 40-step trajectory with collisions within 1e-8."""
    g = np.load(os.path.join(GOLDEN, "traj_two_cubes6_snh_vf.npz"))
    s = scenes.two_cubes_scene(6)
    sim = oracle.Sim(s)
    sim.set_collisions(True, 1e-3, 1e3, 0.001)
    pairs, tris = sim.vf_pairs()
    assert np.array_equal(tris, g["surface_triangles"])
    stride = int(g["stride"])
    for k in range(g["x"].shape[0]):
        if k > 0:
            sim.step(stride)
            x, _ = sim.state()
            assert np.linalg.norm(x - g["x"][k]) / np.linalg.norm(g["x"][k]) < 1e-8
        pairs, _ = sim.vf_pairs()
        ref = g[f"pairs_{k}"]
        assert sorted(map(tuple, pairs.tolist())) == sorted(map(tuple, ref.tolist())), k


def test_oracle_green_damped_newmark_matches_the_reference_fixture():
    """NEWMARK's energy-damped solve with GREEN_DAMPING(mu) (NEWMARK.cpp:
    344-420, GREEN_DAMPING.cpp:46-74): the restatement against the committed
    trajectories of the reference built from its sources
    (traj_kuhn5_snh_newmark_green.npz, tests/golden/make_golden.py green),
    six steps at mu = 0.05 and 1.0."""
    g = np.load(os.path.join(GOLDEN, "traj_kuhn5_snh_newmark_green.npz"))
    s = scenes.config1_scene(5)
    undamped = oracle.Sim(s, precond=0, integrator="newmark")
    undamped.step(int(g["steps"]))
    xu, _ = undamped.state()
    for mu in g["mus"]:
        tag = f"mu{mu:g}".replace(".", "p")
        xr = g[f"x_{tag}"]
        sim = oracle.Sim(s, precond=0, integrator="newmark")
        sim.set_green_damping(mu)
        for k in range(int(g["steps"])):
            sim.step(1)
            x, _ = sim.state()
            assert np.linalg.norm(x - xr[k + 1]) / np.linalg.norm(xr[k + 1]) < 1e-12, (mu, k)
        # the damping term matters at this size: far above the bound
        assert np.linalg.norm(xu - xr[-1]) / np.linalg.norm(xr[-1]) > 1e-7, mu


def test_oracle_green_damping_refused_outside_newmark():
    """Only NEWMARK's energy-damped solve is defined (the reference's damped
    BACKWARD_EULER_VELOCITY reads a never-computed Fdot)."""
    sim = oracle.Sim(scenes.config1_scene(3), precond=0)
    assert oracle.lib().oracle_set_green_damping(sim.h, 0.1) == -1


def test_oracle_green_damped_newmark_matches_the_reference_when_built():
    """The same against a live run of the reference build, when that build
    exists in this checkout."""
    from oracle import refrun
    if not os.path.exists(refrun.REF_BIN):
        pytest.skip("reference build not present")
    s = scenes.config1_scene(5)
    for mu in (0.05, 1.0):
        r = refrun.run(s, 6, integrator="newmark", green_damping=mu)
        sim = oracle.Sim(s, precond=0, integrator="newmark")
        sim.set_green_damping(mu)
        for k in range(6):
            sim.step(1)
            x, _ = sim.state()
            assert np.linalg.norm(x - r["x"][k + 1]) / np.linalg.norm(r["x"][k + 1]) < 1e-12, (mu, k)


def test_oracle_newmark_contact_matches_reference():
    """NEWMARK with vertex-face contact inside the Newton loop (NEWMARK.cpp:
    226-242): the restatement against the reference build's trajectory of two
    6^3 cubes (traj_two_cubes6_snh_newmark_vf.npz)."""
    g = np.load(os.path.join(GOLDEN, "traj_two_cubes6_snh_newmark_vf.npz"))
    s = scenes.two_cubes_scene(6)
    sim = oracle.Sim(s, precond=0, integrator="newmark")
    sim.set_collisions(True, 1e-3, 1e3, 0.001)
    for k in range(1, g["x"].shape[0]):
        sim.step(int(g["stride"]))
        x, _ = sim.state()
        assert np.linalg.norm(x - g["x"][k]) / np.linalg.norm(g["x"][k]) < 1e-12, k
