"""NEWMARK (Rayleigh-damped solve: a Newton loop of linear solves, its C
zeroed by the reference before use) on the GPU: a device-side Newton loop
around the shared kernels, against the reference's own trajectories
(golden), the oracle, both precisions, batching, graph vs eager and the
drop-in mirror."""
import os

import numpy as np
import pytest

from hobakv1_gb300 import _lib, hobak, scenes
from oracle import oracle

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
NM = hobak.INTEGRATOR_NEWMARK


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


TRAJ = [("kuhn6_snh_twist", lambda: scenes.config2_scene(6, "snh")),
        ("kuhn6_arap_twist", lambda: scenes.config2_scene(6, "arap"))]


@pytest.mark.parametrize("name,fn", TRAJ, ids=[t[0] for t in TRAJ])
def test_newmark_trajectory_matches_reference(name, fn):
    """With the reference's Jacobi preconditioner: positions and velocities at
    every recorded step within 1e-8 / 1e-7 relative (FP64), and the last
    Newton iteration's CG count of every step within 2."""
    g = np.load(os.path.join(GOLDEN, f"traj_{name}_newmark.npz"))
    s = fn()
    b = hobak.BATCH([s], hobak.solver_opts(preconditioner=hobak.PRECOND_JACOBI, integrator=NM))
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
def test_newmark_block_jacobi_matches_oracle(name, fn):
    s = fn()
    b = hobak.BATCH([s], hobak.solver_opts(integrator=NM))
    sim = oracle.Sim(s, precond=hobak.PRECOND_BLOCK_JACOBI, integrator="newmark")
    for _ in range(3):
        b.step(5)
        sim.step(5)
        x, v = b.get_state(0)
        xo, vo = sim.state()
        assert rel(x, xo) < 1e-10 and rel(v, vo) < 1e-9, (rel(x, xo), rel(v, vo))
        assert rel(b.get_acceleration(0), sim.acceleration()) < 1e-8


@pytest.mark.parametrize("material", ["snh", "arap"])
def test_mixed_newmark_tracks_fp64_oracle(material):
    s = scenes.config2_scene(8, material)
    b = hobak.BATCH([s], hobak.solver_opts(precision=hobak.PRECISION_MIXED, integrator=NM))
    sim = oracle.Sim(s, precond=1, integrator="newmark")
    for _ in range(3):
        st = b.step(5)
        assert st[0][1] == 1, st
        sim.step(5)
        x, _ = b.get_state(0)
        xo, _ = sim.state()
        assert rel(x, xo) < 1e-6, rel(x, xo)


@pytest.mark.parametrize("precision", [hobak.PRECISION_FP64, hobak.PRECISION_MIXED], ids=["fp64", "mixed"])
def test_newmark_scene_is_the_same_alone_and_in_a_mix_and_eager(precision):
    """Scenes of a batch run their own Newton loops (different iteration
    counts); each result equals the scene alone, and the eager loop equals
    the graph's."""
    mix = scenes.config4_scenes(count=5, nmin=4, nmax=9)
    batch = hobak.BATCH(mix, hobak.solver_opts(precision=precision, integrator=NM))
    batch.step(3)
    for i in (0, 2, 4):
        alone = hobak.BATCH([mix[i]], hobak.solver_opts(precision=precision, integrator=NM, use_graph=False))
        alone.step(3)
        xa, va = alone.get_state(0)
        xm, vm = batch.get_state(i)
        assert np.array_equal(xa, xm) and np.array_equal(va, vm), i
        assert np.array_equal(alone.get_acceleration(0), batch.get_acceleration(i)), i


def test_newmark_cluster_path_matches_tile_path():
    mix = scenes.config4_scenes(count=4, nmin=5, nmax=12)
    out = []
    for cluster in (1, 0):
        b = hobak.BATCH(mix, hobak.solver_opts(precision=hobak.PRECISION_MIXED, integrator=NM))
        b.set_tuning(cluster_pcg=cluster)
        b.step(3)
        out.append([b.get_state(i)[0] + mix[i].rest.reshape(-1) for i in range(len(mix))])
    for k in range(len(mix)):
        assert rel(out[0][k], out[1][k]) < 1e-6, k


def test_newmark_contact_matches_reference():
    """NEWMARK with vertex-face contact detected and answered at every Newton
    iterate (NEWMARK.cpp:226-242; C = beta H_coll, TIMESTEPPER.cpp:645-720):
    two 6^3 cubes in contact, 40 steps, positions every 10 steps within 1e-8
    of the reference build's trajectory (Jacobi, the reference's
    preconditioner), and within 1e-10 of the oracle with block Jacobi."""
    g = np.load(os.path.join(GOLDEN, "traj_two_cubes6_snh_newmark_vf.npz"))
    s = scenes.two_cubes_scene(6)
    b = hobak.BATCH([s], hobak.solver_opts(preconditioner=hobak.PRECOND_JACOBI, integrator=NM))
    b.set_collisions(0, True, 1e-3, 1e3, 0.001)
    for k in range(1, g["x"].shape[0]):
        b.step(int(g["stride"]))
        x, _ = b.get_state(0)
        assert rel(x, g["x"][k]) < 1e-8, (k, rel(x, g["x"][k]))
    bb = hobak.BATCH([s], hobak.solver_opts(integrator=NM))
    bb.set_collisions(0, True, 1e-3, 1e3, 0.001)
    sim = oracle.Sim(s, precond=hobak.PRECOND_BLOCK_JACOBI, integrator="newmark")
    sim.set_collisions(True, 1e-3, 1e3, 0.001)
    for _ in range(4):
        bb.step(5)
        sim.step(5)
        x, _ = bb.get_state(0)
        xo, _ = sim.state()
        assert rel(x, xo) < 1e-10, rel(x, xo)
        pairs, _ = bb.collision_pairs(0)
        po, _ = sim.vf_pairs()
        assert sorted(map(tuple, pairs.tolist())) == sorted(map(tuple, po.tolist()))


def test_newmark_contact_graph_equals_eager():
    """The detection inside the Newton loop's conditional graph body gives
    bitwise the same trajectory as eager launches."""
    s = scenes.two_cubes_scene(5)
    runs = []
    for graph in (True, False):
        b = hobak.BATCH([s], hobak.solver_opts(integrator=NM, use_graph=graph))
        b.set_collisions(0, True, 1e-3, 1e3, 0.001)
        b.set_edge_collisions(0, True)
        b.step(6)
        runs.append(b.get_state(0))
    assert np.array_equal(runs[0][0], runs[1][0]) and np.array_equal(runs[0][1], runs[1][1])


def test_python_mirror_newmark_matches_oracle():
    s = scenes.config2_scene(5, "arap")
    mesh = hobak.TET_MESH(s.rest, s.tets)
    mesh.setDisplacement(s.x0)
    nm = hobak.NEWMARK(mesh, hobak.ARAP(s.mu, s.lam))
    assert nm.maxNewtonIterations() == 10
    nm.position()[:] = s.x0.reshape(-1)
    nm.scaleMass(s.density)
    nm.attachKinematicConstraints(s.pinned)
    sim = oracle.Sim(s, precond=hobak.PRECOND_BLOCK_JACOBI, integrator="newmark")
    for _ in range(5):
        nm.externalForces()[:] = 0.0
        nm.addGravity(np.array(s.gravity) * s.density)
        nm.solve(False)
    sim.step(5)
    x, v = sim.state()
    assert rel(nm.position(), x) < 1e-9
    assert rel(nm.velocity(), v) < 1e-8
    assert rel(nm.acceleration(), sim.acceleration()) < 1e-7


def test_green_damped_newmark_matches_reference_fixture():
    """NEWMARK's energy-damped solve with GREEN_DAMPING(mu) (NEWMARK.cpp:
    344-420): with the reference's Jacobi preconditioner, positions after
    each of six steps within 1e-8 of the reference build's trajectories
    (traj_kuhn5_snh_newmark_green.npz), at mu = 0.05 and 1.0."""
    g = np.load(os.path.join(GOLDEN, "traj_kuhn5_snh_newmark_green.npz"))
    s = scenes.config1_scene(5)
    for mu in g["mus"]:
        xr = g[f"x_mu{mu:g}".replace(".", "p")]
        b = hobak.BATCH([s], hobak.solver_opts(preconditioner=hobak.PRECOND_JACOBI, integrator=NM))
        b.set_green_damping(0, mu)
        for k in range(int(g["steps"])):
            b.step(1)
            x, _ = b.get_state(0)
            assert rel(x, xr[k + 1]) < 1e-8, (mu, k, rel(x, xr[k + 1]))
        b.close()


@pytest.mark.parametrize("precision,bound", [(hobak.PRECISION_FP64, 1e-10), (hobak.PRECISION_MIXED, 1e-6)],
                         ids=["fp64", "mixed"])
def test_green_damped_newmark_matches_oracle_and_batches(precision, bound):
    """Block Jacobi against the oracle's energy-damped NEWMARK; a damped and
    an undamped scene in one batch each match their own oracle run, and the
    damped scene is the same alone and in the batch."""
    mix = [scenes.config2_scene(6, "snh"), scenes.config1_scene(6)]
    b = hobak.BATCH(mix, hobak.solver_opts(precision=precision, integrator=NM))
    b.set_green_damping(0, 0.5)
    b.step(8)
    for i, s in enumerate(mix):
        sim = oracle.Sim(s, precond=hobak.PRECOND_BLOCK_JACOBI, integrator="newmark")
        if i == 0:
            sim.set_green_damping(0.5)
        sim.step(8)
        x, _ = b.get_state(i)
        xo, _ = sim.state()
        assert rel(x, xo) < bound, (i, rel(x, xo))
    alone = hobak.BATCH([mix[0]], hobak.solver_opts(precision=precision, integrator=NM))
    alone.set_green_damping(0, 0.5)
    alone.step(8)
    assert np.array_equal(alone.get_state(0)[0], b.get_state(0)[0])


def test_green_damping_refused_outside_newmark():
    b = hobak.BATCH([scenes.config1_scene(3)])
    with pytest.raises(_lib.HobakError):
        b.set_green_damping(0, 0.1)


def test_python_mirror_newmark_with_green_damping():
    """NEWMARK(mesh, material, GREEN_DAMPING(mu)), as the reference constructs
    the energy-damped integrator, against the oracle."""
    s = scenes.config1_scene(5)
    mesh = hobak.TET_MESH(s.rest, s.tets)
    nm = hobak.NEWMARK(mesh, hobak.SNH(s.mu, s.lam), hobak.GREEN_DAMPING(1.0))
    nm.scaleMass(s.density)
    nm.attachKinematicConstraints(s.pinned)
    sim = oracle.Sim(s, precond=hobak.PRECOND_BLOCK_JACOBI, integrator="newmark")
    sim.set_green_damping(1.0)
    for _ in range(4):
        nm.externalForces()[:] = 0.0
        nm.addGravity(np.array(s.gravity) * s.density)
        nm.solve(False)
    sim.step(4)
    x, _ = sim.state()
    assert rel(nm.position(), x) < 1e-9
