"""The reference's scene regression (regressionTests.cpp:45-102) on the GPU:
NEWMARK_STRETCH through the NEWMARK drop-in, its pins following a moving
kinematic shape, against the reference's own recorded frames
(data/regression/newmark_stretch.json.gz, fixture copy); and the batch
state snapshot/restore."""
import os

import numpy as np
import pytest

from hobakv1_gb300 import _lib, hobak, replay, scenes

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def stretch_record():
    g = np.load(os.path.join(GOLDEN, "regression_newmark_stretch.npz"))
    rec = replay.SceneRecord(scene={"dt": float(g["dt"])}, frameNumber=g["frame_number"], position=g["position"],
                             velocity=g["velocity"], frameIndex=g["frames"], recordedFrames=int(g["total_frames"]))
    return g["rest"], g["tets"], rec


@pytest.mark.parametrize("precision,precond,tol", [
    (hobak.PRECISION_FP64, hobak.PRECOND_JACOBI, 1e-8),        # the reference's own tolerance
    (hobak.PRECISION_FP64, hobak.PRECOND_BLOCK_JACOBI, 1e-8),
    (hobak.PRECISION_MIXED, hobak.PRECOND_BLOCK_JACOBI, 1e-6),
], ids=["fp64_jacobi", "fp64_block", "mixed"])
def test_newmark_stretch_matches_the_reference_record(precision, precond, tol):
    rest, tets, rec = stretch_record()
    opts = hobak.solver_opts(precision=precision, preconditioner=precond, integrator=hobak.INTEGRATOR_NEWMARK)
    ok, err = replay.scene_regression(replay.NEWMARK_STRETCH(rest, tets, opts), rec, tol=tol)
    assert ok, err
    assert len(err) == len(rec.frameIndex)


def test_recorded_run_replays_through_the_reader(tmp_path):
    rest, tets, rec = stretch_record()
    sc = replay.NEWMARK_STRETCH(rest, tets)
    sc.buildScene()
    out = replay.SceneRecorder(sc)
    for _ in range(6):
        sc.stepSimulation()
        out.record_frame(sc)
    path = str(tmp_path / "stretch.json.gz")
    out.write(path)
    back = replay.read_scene_json(path)
    assert list(back.frameNumber) == [1, 2, 3, 4, 5, 6]
    assert np.array_equal(back.position[-1], sc.solver().position())
    assert np.array_equal(back.positionOld[-1], back.position[-2])
    for k in (0, 3):  # frames kept in the fixture
        r = rec.row(k)
        assert r is not None
        g = rec.position[r]
        if np.linalg.norm(g) > 1e-12:
            assert np.linalg.norm(back.position[k] - g) / np.linalg.norm(g) < 1e-8


@pytest.mark.parametrize("integrator", [hobak.INTEGRATOR_VELOCITY, hobak.INTEGRATOR_NEWMARK], ids=["bev", "newmark"])
@pytest.mark.parametrize("precision", [hobak.PRECISION_FP64, hobak.PRECISION_MIXED], ids=["fp64", "mixed"])
def test_snapshot_restore_replays_bitwise(integrator, precision):
    mix = scenes.config4_scenes(count=4, nmin=4, nmax=8)
    b = hobak.BATCH(mix, hobak.solver_opts(precision=precision, integrator=integrator))
    b.step(3)
    snap = b.snapshot()
    assert snap.size == b.snapshot_bytes()
    b.step(4)
    after = b.get_state_all()
    acc = b.get_acceleration(2)
    b.restore(snap)
    b.step(4)
    again = b.get_state_all()
    assert np.array_equal(after[0], again[0]) and np.array_equal(after[1], again[1])
    assert np.array_equal(acc, b.get_acceleration(2))
    b.close()


def test_device_snapshot_and_restore_into_another_batch():
    import torch
    mix = scenes.config4_scenes(count=3, nmin=4, nmax=7)
    a = hobak.BATCH(mix, hobak.solver_opts())
    a.step(2)
    a.set_active(1, 0)  # parked scenes stay parked after a restore
    buf = torch.empty(a.snapshot_bytes(), dtype=torch.uint8, device="cuda")
    a.snapshot(dst_ptr=buf.data_ptr())
    c = hobak.BATCH(mix, hobak.solver_opts())
    c.restore(src_ptr=buf.data_ptr(), nbytes=buf.numel())
    a.step(3)
    c.step(3)
    for i in range(3):
        xa, va = a.get_state(i)
        xc, vc = c.get_state(i)
        assert np.array_equal(xa, xc) and np.array_equal(va, vc), i
    other = hobak.BATCH(mix[:2], hobak.solver_opts())
    with pytest.raises(_lib.HobakError):
        other.restore(a.snapshot())
    with pytest.raises(_lib.HobakError):
        other.restore(np.zeros(other.snapshot_bytes(), dtype=np.uint8))


def test_pin_targets_move_the_pins():
    s = scenes.config1_scene(6)
    b = hobak.BATCH([s], hobak.solver_opts())
    t = np.tile([0.0, 0.05, 0.0], (len(s.pinned), 1))
    b.set_pin_targets(0, t)
    b.step(1)
    x, v = b.get_state(0)
    assert np.allclose(x.reshape(-1, 3)[s.pinned], t)
    with pytest.raises(_lib.HobakError):
        b.set_pin_targets(0, np.full_like(t, np.nan))


@pytest.mark.parametrize("precision,bound", [(hobak.PRECISION_FP64, 1e-8), (hobak.PRECISION_MIXED, 1e-5)],
                         ids=["fp64", "mixed"])  # mixed: 1e-8 per solve, grown over 200 frames of contact
@pytest.mark.parametrize("name", ["two_tet_drop_vf", "two_tet_kiss_vf", "two_tet_drop_ee", "two_tet_kiss_ee"])
def test_two_tet_contact_scenes_match_the_reference(name, precision, bound):
    """The reference's two-tet vertex-face regression scenes through the
    BACKWARD_EULER_POSITION drop-in with contact, frame by frame: against
    the reference built here (fixture) at `bound`, against the recorded file
    at 2e-7 (FP64; the reference itself is 2.5e-8 / 8.9e-8 from it here),
    and the vertex-face pair count of every frame equal to the record's."""
    g = np.load(os.path.join(GOLDEN, f"regression_{name}.npz"))
    cls = {"two_tet_drop_vf": replay.TWO_TET_DROP_VF, "two_tet_kiss_vf": replay.TWO_TET_KISS_VF,
           "two_tet_drop_ee": replay.TWO_TET_DROP_EE, "two_tet_kiss_ee": replay.TWO_TET_KISS_EE}[name]
    sc = cls(g["rest"], g["tets"], hobak.solver_opts(precision=precision, preconditioner=hobak.PRECOND_JACOBI,
                                                     integrator=hobak.INTEGRATOR_POSITION))
    sc.buildScene()
    for k in range(int(g["total_frames"])):
        sc.stepSimulation()
        x = sc.solver().position()
        xr = g["ref_position"][k]
        assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < bound, k
        if precision == hobak.PRECISION_FP64:
            assert np.linalg.norm(x - g["position"][k]) / np.linalg.norm(g["position"][k]) < 2e-7, k
        assert len(sc.vertexFaceCollisions()) == int(g["vf_pairs"][k]), k
        assert len(sc.edgeEdgeQuads()) == int(g["ee_pairs"][k]), k


@pytest.mark.parametrize("N", [4, 8])
def test_edge_edge_pairs_match_oracle_on_two_cubes(N):
    """Edge-edge pairs (vertex quadruples; the GPU's hashed broad phase
    against the oracle's scan over all edge pairs) and trajectory of two
    cubes pressed together with vertex-face and edge-edge contact."""
    from oracle import oracle
    two = scenes.two_cubes_scene(N)
    b = hobak.BATCH([two], hobak.solver_opts(integrator=hobak.INTEGRATOR_POSITION))
    b.set_collisions(0, True, 2e-2, 1e3, 0.001)
    b.set_edge_collisions(0, True)
    sim = oracle.Sim(two, precond=1, integrator="position")
    sim.set_collisions(True, 2e-2, 1e3, 0.001, ee=True)
    seen = 0
    for _ in range(5):
        b.step(1)
        sim.step(1)
        q, qo = b.edge_pairs(0), sim.ee_pairs()
        assert np.array_equal(q, qo)
        seen += len(q)
        x, _ = b.get_state(0)
        xo, _ = sim.state()
        r = two.rest.reshape(-1)
        assert np.linalg.norm(x - xo) / np.linalg.norm(xo + r) < 1e-9
    assert seen > 0
