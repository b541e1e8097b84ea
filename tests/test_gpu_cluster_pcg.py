"""Cluster-resident PCG (one thread-block cluster per small scene, vectors in
distributed shared memory, running beside the tile path) against the tile
path and the oracle."""
import numpy as np
import pytest

from hobakv1_gb300 import hobak, scenes
from oracle import oracle

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def run(scene_list, precision, steps, cluster, precond=hobak.PRECOND_BLOCK_JACOBI):
    b = hobak.BATCH(scene_list, hobak.solver_opts(precision=precision, preconditioner=precond))
    b.set_tuning(cluster_pcg=int(cluster))
    st = b.step(steps)
    out = [b.get_state(i)[0] + s.rest.reshape(-1) for i, s in enumerate(scene_list)]
    b.close()
    return out, st


@pytest.mark.parametrize("precision", [hobak.PRECISION_FP64, hobak.PRECISION_MIXED], ids=["fp64", "mixed"])
def test_cluster_path_matches_tile_path(precision):
    # scene sizes that land in clusters of 1, 2, 4, 8 and 16 CTAs
    mix = scenes.config4_scenes(count=10, nmin=5, nmax=24)
    xc, stc = run(mix, precision, 6, True)
    xt, stt = run(mix, precision, 6, False)
    bound = 1e-8 if precision == hobak.PRECISION_FP64 else 1e-6
    for k in range(len(mix)):
        assert rel(xc[k], xt[k]) < bound, (k, mix[k].nv, rel(xc[k], xt[k]))
        assert stc[k][1] == 1 and abs(stc[k][0] - stt[k][0]) <= 2, (stc[k], stt[k])
        # mixed: the cluster runs the refinement sweeps itself (residual
        # updated with compensated FP32 products) and ends on the same FP64
        # test, after as many sweeps as the tile path's FP64 residual needs
        assert stc[k][2] < 1e-8 and abs(stc[k][3] - stt[k][3]) <= 1, (stc[k], stt[k])


def test_cluster_path_matches_oracle_with_jacobi_iterations():
    s = scenes.config1_scene(10)  # 1,331 vertices: a two-CTA cluster
    b = hobak.BATCH([s], hobak.solver_opts(preconditioner=hobak.PRECOND_JACOBI))
    b.set_tuning(cluster_pcg=1)
    sim = oracle.Sim(s, precond=0)
    for _ in range(5):
        st = b.step(1)
        it, _ = sim.step(1)
        assert abs(st[0][0] - int(it[0])) <= 1, (st[0], it)
    x, _ = b.get_state(0)
    xo, _ = sim.state()
    assert rel(x + s.rest.reshape(-1), xo + s.rest.reshape(-1)) < 1e-10


@pytest.mark.parametrize("precision", [hobak.PRECISION_FP64, hobak.PRECISION_MIXED], ids=["fp64", "mixed"])
def test_large_and_small_scenes_share_a_batch(precision):
    """A scene too large for a cluster takes the tile path while the small
    ones solve in clusters beside it; each result equals the scene alone."""
    big = scenes.config2_scene(40, "snh")  # 68,921 vertices: more than 16 CTAs' shared memory holds
    small = scenes.config4_scenes(count=3, nmin=6, nmax=12)
    together, _ = run([big] + small, precision, 4, True)
    b = hobak.BATCH([big] + small, hobak.solver_opts(precision=precision))
    b.set_tuning(cluster_pcg=1)
    paths = b.pcg_path()
    b.close()
    assert paths[0] == 0 and (paths[1:] > 0).all(), paths
    for k, sc in enumerate([big] + small):
        alone, _ = run([sc], precision, 4, True)
        assert np.array_equal(together[k], alone[0]), k


def test_mid_size_scene_in_a_16_cta_cluster_matches_the_tile_path():
    """Mixed precision: a scene of 29,791 vertices (more than one per thread
    of 16 CTAs) solves in one 16-CTA cluster whose threads take two vertices
    each, and agrees with the tile path to rounding (FP64 vectors would not
    fit: the FP64 batch keeps it on the tile path)."""
    s = scenes.config2_scene(30, "snh")
    b = hobak.BATCH([s], hobak.solver_opts(precision=hobak.PRECISION_MIXED))
    b.set_tuning(cluster_pcg=1)
    assert b.pcg_path()[0] == 16
    b.close()
    b = hobak.BATCH([s], hobak.solver_opts(precision=hobak.PRECISION_FP64))
    b.set_tuning(cluster_pcg=1)
    assert b.pcg_path()[0] == 0
    b.close()
    xc, stc = run([s], hobak.PRECISION_MIXED, 6, True)
    xt, stt = run([s], hobak.PRECISION_MIXED, 6, False)
    assert rel(xc[0], xt[0]) < 1e-6 and stc[0][1] == 1 and stc[0][2] < 1e-8, (rel(xc[0], xt[0]), stc, stt)


EPS, MU, BETA = 1e-3, 1e3, 0.001


def as_set(p):
    return sorted(map(tuple, np.asarray(p).tolist()))


@pytest.mark.parametrize("ee", [False, True], ids=["vf", "vf+ee"])
@pytest.mark.parametrize("precision,bound", [(hobak.PRECISION_FP64, 1e-8), (hobak.PRECISION_MIXED, 1e-6)],
                         ids=["fp64", "mixed"])
def test_contact_scene_in_a_cluster_matches_oracle_and_alone(precision, bound, ee):
    """Self contact on the cluster path (a cluster adds its rows' contact
    terms to the SpMV and to its residual update, as the tile path does):
    two 8^3 cubes (1,458 vertices, a 2-CTA cluster) with vertex-face (and
    edge-edge) contact beside clustered small scenes: positions within
    `bound` of the FP64 oracle, the vertex-face pair sets equal the oracle's
    (FP64), and the contact scene bitwise equal to itself alone.  FP64 runs
    20 steps; mixed precision the first 10, the contact phase (the pairs
    release by step 13): once the cubes separate with edge-edge springs
    still engaged the trajectory becomes sensitive enough that mixed
    precision departs from FP64 on the tile path as well (5e-6 by step 20,
    from 1e-8 at step 13)."""
    s = scenes.two_cubes_scene(8, gap=2e-4)
    small = scenes.config4_scenes(count=2, nmin=5, nmax=8)

    def batch(scene_list):
        b = hobak.BATCH(scene_list, hobak.solver_opts(precision=precision))
        b.set_tuning(cluster_pcg=1)
        b.set_collisions(0, True, EPS, MU, BETA)
        if ee:
            b.set_edge_collisions(0, True)
        return b

    b = batch([s] + small)
    sim = oracle.Sim(s, precond=hobak.PRECOND_BLOCK_JACOBI)
    sim.set_collisions(True, EPS, MU, BETA, ee=ee)
    chunks = 4 if precision == hobak.PRECISION_FP64 else 2
    for k in range(chunks):
        if precision == hobak.PRECISION_FP64:
            gp, _ = b.collision_pairs(0, detect_now=True)
            op, _ = sim.vf_pairs()
            assert as_set(gp) == as_set(op), k
        b.step(5)
        sim.step(5)
        assert b.pcg_path()[0] > 0  # the contact scene solves in a cluster
        x, _ = b.get_state(0)
        xo, _ = sim.state()
        err = rel(x + s.rest.reshape(-1), xo + s.rest.reshape(-1))
        assert err < bound, (k, err)
    a = batch([s])
    a.step(5 * chunks)
    assert np.array_equal(b.get_state(0)[0], a.get_state(0)[0])
    b.close()
    a.close()


@pytest.mark.parametrize("precision", [hobak.PRECISION_FP64, hobak.PRECISION_MIXED], ids=["fp64", "mixed"])
@pytest.mark.parametrize("cap", [2, 4])
def test_capped_clusters_match_the_tile_path_and_the_scene_alone(precision, cap):
    """Clusters of at most `cap` CTAs: a scene of more than cap x 1024
    vertices solves in a capped cluster with several vertices per thread
    (mixed precision: its FP32 vectors fit in shared memory) or on the tile
    path (FP64 at cap 2: they do not); either way it agrees with the tile path
    to rounding and equals itself alone bitwise, beside clustered small ones."""
    big = scenes.config4_scenes(count=1, nmin=18, nmax=18)[0]  # 5,832 vertices: an 8-CTA cluster uncapped
    small = scenes.config4_scenes(count=2, nmin=6, nmax=9)
    mix = [big] + small
    b = hobak.BATCH(mix, hobak.solver_opts(precision=precision))
    b.set_tuning(cluster_pcg=1, cluster_max=cap)
    b.step(4)
    alone = hobak.BATCH([big], hobak.solver_opts(precision=precision))
    alone.set_tuning(cluster_pcg=1, cluster_max=cap)
    alone.step(4)
    assert np.array_equal(b.get_state(0)[0], alone.get_state(0)[0])
    tile, _ = run([big], precision, 4, False)
    bound = 1e-8 if precision == hobak.PRECISION_FP64 else 1e-6
    assert rel(b.get_state(0)[0] + big.rest.reshape(-1), tile[0]) < bound
    for k, sc in enumerate(small, start=1):
        c = hobak.BATCH([sc], hobak.solver_opts(precision=precision))
        c.set_tuning(cluster_pcg=1)
        c.step(4)
        assert np.array_equal(b.get_state(k)[0], c.get_state(0)[0]), k


@pytest.mark.parametrize("integrator", [hobak.INTEGRATOR_POSITION, hobak.INTEGRATOR_NEWMARK],
                         ids=["position", "newmark"])
def test_contact_in_a_cluster_with_the_other_integrators(integrator):
    """The contact rows' scale follows the integrator (collision_lhs_scale:
    BACKWARD_EULER_POSITION's -(beta/dt + 1), NEWMARK's -(a3 beta + 1)):
    two 7^3 cubes in vertex-face contact, FP64, 10 steps, the cluster path
    within 1e-9 of the tile path."""
    s = scenes.two_cubes_scene(7, gap=2e-4)

    def run_path(cluster):
        b = hobak.BATCH([s], hobak.solver_opts(integrator=integrator))
        b.set_tuning(cluster_pcg=int(cluster))
        b.set_collisions(0, True, EPS, MU, BETA)
        b.step(10)
        assert (b.pcg_path()[0] > 0) == cluster
        x = b.get_state(0)[0] + s.rest.reshape(-1)
        b.close()
        return x

    xc, xt = run_path(True), run_path(False)
    assert rel(xc, xt) < 1e-9, rel(xc, xt)
