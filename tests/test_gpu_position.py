"""BACKWARD_EULER_POSITION (Rayleigh damped) on the GPU: the same kernels as
the velocity integrator with the position integrator's rhs, LHS and update,
against the reference's own trajectories (golden), the oracle, both
precisions, batching and the drop-in mirror."""
import os

import numpy as np
import pytest

from hobakv1_gb300 import _lib, hobak, scenes
from oracle import oracle

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
POS = hobak.INTEGRATOR_POSITION


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


TRAJ = [("kuhn6_snh_twist", lambda: scenes.config2_scene(6, "snh")),
        ("kuhn6_arap_twist", lambda: scenes.config2_scene(6, "arap")),
        ("kuhn8_snh", lambda: scenes.config1_scene(8))]


@pytest.mark.parametrize("name,fn", TRAJ, ids=[t[0] for t in TRAJ])
def test_position_trajectory_matches_reference(name, fn):
    """With the reference's Jacobi preconditioner: positions and velocities
    at every recorded step of the reference's own run within 1e-8 / 1e-7
    relative (FP64) and the iteration counts of every step. The 3x3
    block-Jacobi path (the GPU default) stops each solve at a different point
    inside the same residual tolerance; it is pinned against the oracle run
    with block Jacobi (below), the oracle itself against the reference."""
    g = np.load(os.path.join(GOLDEN, f"traj_{name}_position.npz"))
    a, bb = (float(c) for c in g["rayleigh"])
    s = fn()
    b = hobak.BATCH([s], hobak.solver_opts(preconditioner=hobak.PRECOND_JACOBI, integrator=POS, rayleigh=(a, bb)))
    stride = int(g["stride"])
    iters = []
    for k in range(1, g["x"].shape[0]):
        for _ in range(stride):
            iters.append(b.step(1)[0][0])
        x, v = b.get_state(0)
        assert rel(x, g["x"][k]) < 1e-8, (k, rel(x, g["x"][k]))
        assert rel(v, g["v"][k]) < 1e-7, (k, rel(v, g["v"][k]))
    # stats count SpMV products; Eigen's iterations() counts one fewer
    assert np.abs(np.array(iters) - (g["iters"] + 1)).max() <= 2


@pytest.mark.parametrize("name,fn", TRAJ, ids=[t[0] for t in TRAJ])
def test_position_block_jacobi_matches_oracle(name, fn):
    s = fn()
    b = hobak.BATCH([s], hobak.solver_opts(integrator=POS))
    sim = oracle.Sim(s, precond=hobak.PRECOND_BLOCK_JACOBI, integrator="position")
    for _ in range(3):
        st = b.step(10)
        it, _ = sim.step(10)
        x, v = b.get_state(0)
        xo, vo = sim.state()
        assert rel(x, xo) < 1e-10 and rel(v, vo) < 1e-9, (rel(x, xo), rel(v, vo))
    assert abs(st[0][0] - (int(it[-1]) + 1)) <= 1


@pytest.mark.parametrize("material", ["snh", "arap"])
def test_mixed_position_tracks_fp64_oracle(material):
    s = scenes.config2_scene(10, material)
    b = hobak.BATCH([s], hobak.solver_opts(precision=hobak.PRECISION_MIXED, integrator=POS))
    sim = oracle.Sim(s, precond=1, integrator="position")
    for _ in range(4):
        st = b.step(10)
        assert st[0][1] == 1, st
        sim.step(10)
        x, _ = b.get_state(0)
        xo, _ = sim.state()
        assert rel(x, xo) < 1e-6, rel(x, xo)


@pytest.mark.parametrize("precision", [hobak.PRECISION_FP64, hobak.PRECISION_MIXED], ids=["fp64", "mixed"])
def test_position_scene_is_the_same_alone_and_in_a_mix(precision):
    mix = scenes.config4_scenes(count=5, nmin=4, nmax=9)
    opts = hobak.solver_opts(precision=precision, integrator=POS, rayleigh=(0.02, 0.005))
    batch = hobak.BATCH(mix, opts)
    batch.step(4)
    for i in (0, 2, 4):
        alone = hobak.BATCH([mix[i]], opts)
        alone.step(4)
        xa, va = alone.get_state(0)
        xm, vm = batch.get_state(i)
        assert np.array_equal(xa, xm) and np.array_equal(va, vm), i


@pytest.mark.parametrize("precision", [hobak.PRECISION_FP64, hobak.PRECISION_MIXED], ids=["fp64", "mixed"])
def test_cluster_path_matches_tile_path_for_position(precision):
    mix = scenes.config4_scenes(count=6, nmin=5, nmax=14)
    out = []
    for cluster in (1, 0):
        b = hobak.BATCH(mix, hobak.solver_opts(precision=precision, integrator=POS))
        b.set_tuning(cluster_pcg=cluster)
        b.step(5)
        out.append([b.get_state(i)[0] + mix[i].rest.reshape(-1) for i in range(len(mix))])
    bound = 1e-8 if precision == hobak.PRECISION_FP64 else 1e-6
    for k in range(len(mix)):
        assert rel(out[0][k], out[1][k]) < bound, k


def test_switching_integrator_matches_a_new_batch():
    mix = scenes.config4_scenes(count=3, nmin=4, nmax=7)
    b = hobak.BATCH(mix, hobak.solver_opts())
    b.step(3)
    x, v = b.get_state_all()
    b.set_solver(hobak.solver_opts(integrator=POS))
    b.step(3)
    c = hobak.BATCH(mix, hobak.solver_opts(integrator=POS))
    c.set_state_all(x, v)
    c.step(3)
    xb, vb = b.get_state_all()
    xc, vc = c.get_state_all()
    assert np.array_equal(xb, xc) and np.array_equal(vb, vc)


def test_contact_switches_between_integrators():
    """Contact is available with every integrator: a contact batch can switch
    from the position integrator to NEWMARK and keep stepping."""
    two = scenes.two_cubes_scene(4)
    b = hobak.BATCH([two], hobak.solver_opts(integrator=hobak.INTEGRATOR_NEWMARK))
    b.set_collisions(0, True, 1e-3, 1e3, 0.001)
    b.step(2)
    c = hobak.BATCH([two], hobak.solver_opts(integrator=POS))
    c.set_collisions(0, True, 1e-3, 1e3, 0.001)
    c.step(1)
    c.set_solver(hobak.solver_opts(integrator=hobak.INTEGRATOR_NEWMARK))
    st = c.step(2)
    assert st[0][1] == 1


@pytest.mark.parametrize("precision,bound", [(hobak.PRECISION_FP64, 1e-8), (hobak.PRECISION_MIXED, 1e-6)],
                         ids=["fp64", "mixed"])
def test_position_integrator_with_contact_matches_oracle(precision, bound):
    """Two cubes pressed together (vertex-face pairs every step): forces in
    b, -(beta/dt + 1) H_coll in A (BACKWARD_EULER_POSITION.cpp:187-208)."""
    two = scenes.two_cubes_scene(5)
    b = hobak.BATCH([two], hobak.solver_opts(integrator=POS, precision=precision))
    b.set_collisions(0, True, 1e-3, 1e3, 0.001)
    sim = oracle.Sim(two, precond=1, integrator="position")
    sim.set_collisions(True, 1e-3, 1e3, 0.001)
    for _ in range(4):
        b.step(2)
        sim.step(2)
        assert len(b.collision_pairs(0)[0]) > 0
        x, _ = b.get_state(0)
        xo, _ = sim.state()
        assert rel(x + two.rest.reshape(-1), xo + two.rest.reshape(-1)) < bound


def test_python_mirror_position_solve_matches_oracle():
    """BACKWARD_EULER_POSITION.solve() with host state, like the reference API."""
    s = scenes.config2_scene(5, "snh")
    mesh = hobak.TET_MESH(s.rest, s.tets)
    mesh.setDisplacement(s.x0)
    bep = hobak.BACKWARD_EULER_POSITION(mesh, hobak.SNH(s.mu, s.lam))
    assert bep.rayleighAlpha() == 0.01 and bep.rayleighBeta() == 0.01
    bep.position()[:] = s.x0.reshape(-1)
    bep.scaleMass(s.density)
    bep.attachKinematicConstraints(s.pinned)
    sim = oracle.Sim(s, precond=hobak.PRECOND_BLOCK_JACOBI, integrator="position")
    for _ in range(5):
        bep.externalForces()[:] = 0.0
        bep.addGravity(np.array(s.gravity) * s.density)
        bep.solve(False)
    sim.step(5)
    x, v = sim.state()
    assert rel(bep.position(), x) < 1e-9
    assert rel(bep.velocity(), v) < 1e-8
