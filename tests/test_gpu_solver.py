"""GPU solver modes: graph vs eager launch, mixed precision with FP64
refinement, and batching (each scene's result the same alone and in a mix)."""
import numpy as np
import pytest

from hobakv1_gb300 import hobak, scenes
from oracle import oracle

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_graph_and_eager_launch_are_bitwise_identical():
    s = scenes.config2_scene(8, "snh")
    g = hobak.BATCH([s], hobak.solver_opts(use_graph=True))
    e = hobak.BATCH([s], hobak.solver_opts(use_graph=False))
    g.step(5)
    e.step(5)
    xg, vg = g.get_state(0)
    xe, ve = e.get_state(0)
    assert np.array_equal(xg, xe) and np.array_equal(vg, ve)
    assert g.last_stats == e.last_stats


@pytest.mark.parametrize("material", ["snh", "arap"])
def test_mixed_precision_tracks_fp64_oracle(material):
    """FP32 Hessian/SpMV/inner PCG + FP64 refinement to the same 1e-8
    tolerance: positions stay within 1e-6 relative of the FP64 oracle."""
    s = scenes.config2_scene(10, material)
    b = hobak.BATCH([s], hobak.solver_opts(precision=hobak.PRECISION_MIXED))
    sim = oracle.Sim(s, precond=1)
    for _ in range(4):
        st = b.step(10)
        assert st[0][1] == 1, st  # converged to the FP64 tolerance
        sim.step(10)
        x, _ = b.get_state(0)
        xo, _ = sim.state()
        assert rel(x, xo) < 1e-6, rel(x, xo)


def test_mixed_precision_refines_to_fp64_residual():
    s = scenes.config2_scene(12, "snh")
    b = hobak.BATCH([s], hobak.solver_opts(precision=hobak.PRECISION_MIXED))
    st = b.step(1)[0]
    iters, converged, relres, refinements = st
    assert converged == 1 and relres < 1e-8 and refinements >= 1


@pytest.mark.parametrize("precision", [hobak.PRECISION_FP64, hobak.PRECISION_MIXED], ids=["fp64", "mixed"])
def test_scene_result_is_the_same_alone_and_in_a_mix(precision):
    mix = scenes.config4_scenes(count=6, nmin=4, nmax=9)
    batch = hobak.BATCH(mix, hobak.solver_opts(precision=precision))
    batch.step(5)
    for i in (0, 3, 5):
        alone = hobak.BATCH([mix[i]], hobak.solver_opts(precision=precision))
        alone.step(5)
        xa, va = alone.get_state(0)
        xm, vm = batch.get_state(i)
        # per-scene reductions and tiles do not depend on the batch: bitwise
        assert np.array_equal(xa, xm) and np.array_equal(va, vm), i


def test_batched_mix_matches_oracle_per_scene():
    mix = scenes.config4_scenes(count=5, nmin=4, nmax=8)
    batch = hobak.BATCH(mix)
    batch.step(3)
    for i, s in enumerate(mix):
        sim = oracle.Sim(s, precond=1)
        sim.step(3)
        x, _ = batch.get_state(i)
        xo, _ = sim.state()
        assert rel(x, xo) < 1e-8, (i, rel(x, xo))


def test_zero_rhs_scene_stays_at_rest():
    """rhs == 0 ends the solve with y = 0 (ConjugateGradient.h:49-55): an
    undeformed unit tet (DmInv = I, F = I exactly) under ARAP has P = 0."""
    rest = np.array([[0.0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]])
    tets = np.array([[0, 1, 2, 3]], dtype=np.int32)
    z = np.zeros_like(rest)
    s = scenes.Scene("unit_tet", rest, tets, "arap", 100.0, 1000.0, np.zeros(0, np.int32), z, z.copy(),
                     gravity=(0.0, 0.0, 0.0))
    b = hobak.BATCH([s])
    st = b.step(2)
    x, v = b.get_state(0)
    assert np.abs(x).max() == 0.0 and np.abs(v).max() == 0.0
    assert st[0][1] == 1 and st[0][0] == 0


def test_whole_batch_state_calls_match_per_scene_calls():
    mix = scenes.config4_scenes(count=5, nmin=4, nmax=7)
    b = hobak.BATCH(mix, hobak.solver_opts(precision=hobak.PRECISION_MIXED))
    b.step(2)
    x, v = b.get_state_all()
    off = b.offsets()
    for i in range(len(mix)):
        xi, vi = b.get_state(i)
        assert np.array_equal(x[off[i]:off[i + 1]], xi) and np.array_equal(v[off[i]:off[i + 1]], vi)
    # a round trip through the whole-batch setters changes nothing
    c = hobak.BATCH(mix, hobak.solver_opts(precision=hobak.PRECISION_MIXED))
    c.set_state_all(x, v)
    # f_ext = 0 everywhere through the whole-batch setter, on both batches
    zero = np.zeros(3 * b.total_vertices)
    b.set_external_forces_all(zero)
    c.set_external_forces_all(zero)
    b.step(3)
    c.step(3)
    xb, vb = b.get_state_all()
    xc, vc = c.get_state_all()
    assert np.array_equal(xb, xc) and np.array_equal(vb, vc)


def test_precision_switch_reallocates_and_matches_a_new_batch():
    """Only the batch's precision has buffers; switching precision between
    steps replaces them, and the steps after the switch equal those of a
    batch created with that precision from the same state."""
    mix = scenes.config4_scenes(count=3, nmin=4, nmax=7)
    b = hobak.BATCH(mix, hobak.solver_opts(precision=hobak.PRECISION_FP64))
    fp64_bytes = b.device_bytes()
    b.step(2)
    x, v = b.get_state_all()
    b.set_solver(hobak.solver_opts(precision=hobak.PRECISION_MIXED))
    assert b.device_bytes() < fp64_bytes
    b.step(3)
    c = hobak.BATCH(mix, hobak.solver_opts(precision=hobak.PRECISION_MIXED))
    c.set_state_all(x, v)
    c.step(3)
    xb, vb = b.get_state_all()
    xc, vc = c.get_state_all()
    assert np.array_equal(xb, xc) and np.array_equal(vb, vc)
    b.set_solver(hobak.solver_opts(precision=hobak.PRECISION_FP64))
    assert b.device_bytes() == fp64_bytes
    b.step(1)


@pytest.mark.parametrize("precision", [hobak.PRECISION_FP64, hobak.PRECISION_MIXED], ids=["fp64", "mixed"])
def test_serving_footprint_estimate_covers_the_allocation(precision):
    from hobakv1_gb300.serving import footprint_bytes
    for s in (scenes.config2_scene(6, "snh"), scenes.config4_scenes(count=1, nmin=14, nmax=14)[0]):
        b = hobak.BATCH([s], hobak.solver_opts(precision=precision))
        assert footprint_bytes(s, precision) >= b.device_bytes()
        b.close()


@pytest.mark.parametrize("integrator", [hobak.INTEGRATOR_VELOCITY, hobak.INTEGRATOR_NEWMARK], ids=["bev", "newmark"])
def test_mixed_precision_handles_a_tiny_right_hand_side(integrator):
    """An unloaded mesh at rest: the right-hand side is only the rounding
    residue of the rest-state forces (~1e-16).  The FP32 inner solve runs on
    the residual scaled by a power of two, so its dot products do not
    underflow to 0/0; the result stays at the FP64 solve's noise level."""
    import dataclasses
    s = dataclasses.replace(scenes.config1_scene(6), gravity=(0.0, 0.0, 0.0))
    out = {}
    for prec in (hobak.PRECISION_FP64, hobak.PRECISION_MIXED):
        b = hobak.BATCH([s], hobak.solver_opts(precision=prec, integrator=integrator))
        b.step(3)
        out[prec] = b.get_state(0)[0]
        b.close()
    x64, x32 = out[hobak.PRECISION_FP64], out[hobak.PRECISION_MIXED]
    assert np.isfinite(x32).all() and np.linalg.norm(x64) < 1e-12
    assert np.linalg.norm(x32 - x64) < 1e-12
