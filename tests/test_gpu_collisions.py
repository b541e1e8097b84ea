"""GPU vertex-face collisions against the reference's golden pairs and
trajectory (tests/golden/traj_two_cubes6_snh_vf.npz) and the CPU oracle."""
import os

import numpy as np
import pytest

from hobakv1_gb300 import hobak, scenes
from oracle import oracle

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
EPS, MU, BETA = 1e-3, 1e3, 0.001


def as_set(p):
    return sorted(map(tuple, np.asarray(p).tolist()))


def test_pairs_and_trajectory_match_reference():
    g = np.load(os.path.join(GOLDEN, "traj_two_cubes6_snh_vf.npz"))
    s = scenes.two_cubes_scene(6)
    b = hobak.BATCH([s])
    b.set_collisions(0, True, EPS, MU, BETA)
    pairs, tris = b.collision_pairs(0, detect_now=True)
    assert np.array_equal(tris, g["surface_triangles"])  # surface extraction bit-exact
    assert as_set(pairs) == as_set(g["pairs_0"])          # pair set bit-exact
    stride = int(g["stride"])
    for k in range(1, g["x"].shape[0]):
        b.step(stride)
        x, _ = b.get_state(0)
        err = np.linalg.norm(x - g["x"][k]) / np.linalg.norm(g["x"][k])
        assert err < 1e-8, (k, err)
        pairs, _ = b.collision_pairs(0, detect_now=True)
        assert as_set(pairs) == as_set(g[f"pairs_{k}"]), k


@pytest.mark.parametrize("N", [8, 12])
def test_collision_pairs_match_oracle_along_a_trajectory(N):
    s = scenes.two_cubes_scene(N, gap=2e-4)
    b = hobak.BATCH([s])
    b.set_collisions(0, True, EPS, MU, BETA)
    sim = oracle.Sim(s, precond=1)
    sim.set_collisions(True, EPS, MU, BETA)
    for k in range(4):
        gp, _ = b.collision_pairs(0, detect_now=True)
        op, _ = sim.vf_pairs()
        assert as_set(gp) == as_set(op), k
        b.step(5)
        sim.step(5)
        x, _ = b.get_state(0)
        xo, _ = sim.state()
        assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-8


def test_collision_scene_alone_and_in_a_mix():
    mix = [scenes.two_cubes_scene(6), scenes.config1_scene(5), scenes.two_cubes_scene(7, gap=3e-4)]
    batch = hobak.BATCH(mix)
    for i in (0, 2):
        batch.set_collisions(i, True, EPS, MU, BETA)
    batch.step(6)
    for i in (0, 2):
        alone = hobak.BATCH([mix[i]])
        alone.set_collisions(0, True, EPS, MU, BETA)
        alone.step(6)
        xa, _ = alone.get_state(0)
        xm, _ = batch.get_state(i)
        assert np.array_equal(xa, xm), i


@pytest.mark.parametrize("N", [6, 10])
def test_per_pair_force_and_hessian_match_oracle(N):
    """Collision tets bit-exact; -w grad psi and -w clamped Hessian per pair
    within 1e-10 of the oracle (whose clamp is a numeric 12x12 eigensolve)."""
    s = scenes.two_cubes_scene(N, gap=2e-4)
    b = hobak.BATCH([s])
    b.set_collisions(0, True, EPS, MU, BETA)
    b.collision_pairs(0, detect_now=True)
    gt, gf, gH = b.collision_response(0)
    sim = oracle.Sim(s)
    sim.set_collisions(True, EPS, MU, BETA)
    ot, of, oH = sim.vf_response()
    assert len(gt) > 0 and np.array_equal(gt, ot)
    assert np.abs(gf - of).max() <= 1e-10 * np.abs(of).max()
    assert np.abs(gH - oH).max() <= 1e-10 * np.abs(oH).max()


def test_timestepper_mirror_contact_flags_match_oracle():
    """BACKWARD_EULER_VELOCITY mirror with vertexFaceSelfCollisionsOn, the
    stiffness, damping beta and collision eps set like the reference's
    TIMESTEPPER / TET_MESH accessors (hobak_gpu_set_collisions underneath)."""
    s = scenes.two_cubes_scene(5)
    mesh = hobak.TET_MESH(s.rest, s.tets)
    bev = hobak.BACKWARD_EULER_VELOCITY(mesh, hobak.SNH(s.mu, s.lam))
    bev.scaleMass(s.density)
    bev.attachKinematicConstraints(s.pinned)
    bev.setVertexFaceSelfCollisionsOn(True)
    bev.setCollisionStiffness(MU)
    bev.setCollisionDampingBeta(BETA)
    bev.setCollisionEps(EPS)
    sim = oracle.Sim(s, precond=hobak.PRECOND_BLOCK_JACOBI)
    sim.set_collisions(True, EPS, MU, BETA)
    for _ in range(6):
        bev.externalForces()[:] = 0.0
        bev.addGravity(np.array(s.gravity) * s.density)
        bev.solve(False)
    sim.step(6)
    x, _ = sim.state()
    assert np.linalg.norm(bev.position() - x) / np.linalg.norm(x) < 1e-8
