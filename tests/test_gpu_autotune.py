"""Launch shapes and the autotuner: CTA sizes and the PCG chunk leave results
bitwise unchanged, the tile size changes them only by rounding, and
autotuning leaves the batch's state and trajectory untouched."""
import numpy as np
import pytest

from hobakv1_gb300 import _lib, hobak, scenes

pytestmark = pytest.mark.gpu


def mix():
    return scenes.config4_scenes(count=6, nmin=5, nmax=9)


def run(scene_list, precision, steps=6, **shape):
    b = hobak.BATCH(scene_list, hobak.solver_opts(precision=precision))
    if shape:
        b.set_tuning(**shape)
    b.step(steps)
    out = [b.get_state(i) for i in range(len(scene_list))]
    b.close()
    return out


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("precision", [hobak.PRECISION_FP64, hobak.PRECISION_MIXED], ids=["fp64", "mixed"])
def test_cta_sizes_and_chunk_do_not_change_results(precision):
    sc = mix()
    ref = run(sc, precision)
    for shape in (dict(element_threads=64), dict(assembly_threads=128), dict(assembly_threads=512),
                  dict(assembly_threads=1024),
                  dict(pcg_chunk=4), dict(pcg_chunk=16), dict(cluster_max=4)):
        got = run(sc, precision, **shape)
        for (x, v), (xr, vr) in zip(got, ref):
            assert np.array_equal(x, xr) and np.array_equal(v, vr), shape


@pytest.mark.parametrize("precision", [hobak.PRECISION_FP64, hobak.PRECISION_MIXED], ids=["fp64", "mixed"])
def test_tile_size_changes_results_only_by_rounding(precision):
    sc = mix()
    ref = run(sc, precision)
    got = run(sc, precision, tile_vertices=64)
    for k, ((x, _), (xr, _)) in enumerate(zip(got, ref)):
        pos, pos_r = x + sc[k].rest.reshape(-1), xr + sc[k].rest.reshape(-1)
        assert rel(pos, pos_r) < 1e-8, k


def test_autotune_keeps_state_and_trajectory():
    sc = mix()
    b = hobak.BATCH(sc, hobak.solver_opts(precision=hobak.PRECISION_MIXED))
    b.step(2)
    before = [b.get_state(i) for i in range(len(sc))]
    t = b.autotune(reps=2)
    assert t["tile_vertices"] in (64, 128) and t["element_threads"] in (64, 128)
    assert t["assembly_threads"] in (64, 128, 256, 512) and t["pcg_chunk"] in (4, 8, 16)
    assert t["cluster_pcg"] in (0, 1) and t["cluster_max"] in (4, 8, 16)
    assert t["step_ms"] > 0
    assert b.get_tuning()["tile_vertices"] == t["tile_vertices"]
    after = [b.get_state(i) for i in range(len(sc))]
    for (x, v), (xa, va) in zip(before, after):
        assert np.array_equal(x, xa) and np.array_equal(v, va)
    b.step(3)
    # the same trajectory as a batch that never autotuned but switches to the
    # chosen shape at the same point
    c = hobak.BATCH(sc, hobak.solver_opts(precision=hobak.PRECISION_MIXED))
    c.step(2)
    c.set_tuning(**{k: v for k, v in t.items() if k != "step_ms"})
    c.step(3)
    for i in range(len(sc)):
        xb, vb = b.get_state(i)
        xc, vc = c.get_state(i)
        assert np.array_equal(xb, xc) and np.array_equal(vb, vc), i


def test_bad_shapes_are_refused():
    b = hobak.BATCH(mix()[:1], hobak.solver_opts())
    for bad in (dict(tile_vertices=96), dict(element_threads=256), dict(assembly_threads=100),
                dict(pcg_chunk=0), dict(cluster_max=3), dict(cluster_max=32)):
        with pytest.raises(_lib.HobakError):
            b.set_tuning(**bad)
