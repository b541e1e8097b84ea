"""Parity on the benchmark workloads themselves, not only on small cases.

* A seeded 16-scene subset of the 256-scene batched mix (every 16th scene of
  scenes.config4_scenes(256): Kuhn cubes of 6..24 cells per side, random
  rotations, SNH/ARAP, log-uniform stiffness), batched exactly as the
  benchmark runs it (cluster-resident inner PCG), 20 steps against the FP64
  oracle run scene by scene: FP64 <= 1e-8 and mixed precision <= 1e-6
  relative L2 position error per scene.
* The serving mix's contact job that separates mixed precision from FP64
  (job 2 of scenes.config5_jobs(32): two 26^3 SNH cubes in vertex-face
  contact, 76 steps).  Contact makes the trajectory discontinuous in the
  state: a vertex crossing the detection distance adds or drops a spring.
  Mixed precision tracks FP64 within 1e-6 for as long as both runs find the
  same vertex-face pairs; the first step where the pair sets differ is
  recorded here (SPLIT_STEP) and checked."""
import numpy as np
import pytest

from hobakv1_gb300 import hobak, scenes
from oracle import oracle

pytestmark = pytest.mark.gpu

# first step after which the mixed and FP64 runs of serving job 2 detect
# different vertex-face pair sets
SPLIT_STEP = 22


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("precision,bound", [(hobak.PRECISION_FP64, 1e-8), (hobak.PRECISION_MIXED, 1e-6)],
                         ids=["fp64", "mixed"])
def test_mix256_subset_matches_oracle(precision, bound):
    mix = scenes.config4_scenes(256)[::16]
    assert len(mix) == 16
    b = hobak.BATCH(mix, hobak.solver_opts(precision=precision))
    b.set_tuning(cluster_pcg=1, cluster_max=8)
    sims = [oracle.Sim(s, precond=hobak.PRECOND_BLOCK_JACOBI) for s in mix]
    for k in (10, 20):
        st = b.step(10)
        assert all(s[1] == 1 for s in st), st
        for i, sim in enumerate(sims):
            sim.step(10)
            x, _ = b.get_state(i)
            xo, _ = sim.state()
            e = rel(x + mix[i].rest.reshape(-1), xo + mix[i].rest.reshape(-1))
            assert e < bound, (k, i, mix[i].name, e)
    b.close()


def pair_set(b):
    p, _ = b.collision_pairs(0)
    return set(map(tuple, p.tolist()))


def test_serving_contact_job_mixed_tracks_fp64_until_pair_sets_split():
    sc, nsteps, contact = scenes.config5_jobs(32)[2]
    assert sc.N == 26 and nsteps == 76 and contact is not None
    runs = {}
    for name, prec in (("mixed", hobak.PRECISION_MIXED), ("fp64", hobak.PRECISION_FP64)):
        b = hobak.BATCH([sc], hobak.solver_opts(precision=prec))
        b.set_collisions(0, True, *contact)
        runs[name] = b
    rest = sc.rest.reshape(-1)
    split = None
    worst_before = 0.0
    for k in range(1, nsteps + 1):
        for b in runs.values():
            b.step(1)
        if pair_set(runs["mixed"]) != pair_set(runs["fp64"]):
            split = k
            break
        xm, _ = runs["mixed"].get_state(0)
        xf, _ = runs["fp64"].get_state(0)
        e = rel(xm + rest, xf + rest)
        worst_before = max(worst_before, e)
        assert e < 1e-6, (k, e)
    for b in runs.values():
        b.close()
    print(f"serving job 2: pair sets split after step {split}; mixed vs FP64 before that <= {worst_before:.2e}")
    assert split == SPLIT_STEP, split
