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
  Mixed precision tracks FP64 within 1e-6 for as long as neither run's
  contact branches or pair sets split from the other's; the first step past
  1e-6 and the first steps where the contact branches and the pair sets
  differ are recorded here (SPLIT_STEPS) and checked."""
import numpy as np
import pytest

from hobakv1_gb300 import hobak, scenes
from oracle import oracle

pytestmark = pytest.mark.gpu

# serving job 2: the first step whose mixed-vs-FP64 difference exceeds 1e-6,
# the first step whose contact branches (a pair's reversal flag) differ, and
# the first step whose vertex-face pair sets differ (None: not within the
# job's 76 steps).  With the FP32 SVD of the SNH tets in mixed precision the
# two runs stay within 2.4e-8 of each other through all 76 steps; a build
# whose mixed element arithmetic differs may split at the impact step (21),
# where 58 pairs engage at once.
SPLIT_STEPS = (None, None, None)


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


def contact_branches(b, x_start, rest):
    """{collision tet: reversal flag} of the last detection.  The flag is
    VERTEX_FACE_SQRT_COLLISION::reverse (VERTEX_FACE_SQRT_COLLISION.cpp:73-86)
    at the state the detection saw: a vertex behind its face switches the
    spring from |t| - eps to |t| + eps."""
    tets, _, _ = b.collision_response(0)
    p = (x_start + rest).reshape(-1, 3)
    v = p[tets]  # [n, 4, 3]: vertex, face[2], face[1], face[0]
    e0, e1, e2 = v[:, 3] - v[:, 2], v[:, 0] - v[:, 2], v[:, 1] - v[:, 2]
    rev = np.einsum("ij,ij->i", np.cross(e2, e0), e1) < 0
    return {tuple(t): bool(r) for t, r in zip(tets.tolist(), rev)}


def test_serving_contact_job_mixed_tracks_fp64_until_the_impact_step():
    """Mixed precision, FP64 at tol 1e-8 and FP64 at tol 1e-12 side by side,
    step by step.  Recorded (SPLIT_STEPS): the first step whose mixed-vs-FP64
    difference exceeds 1e-6 (the impact step, where the cubes' contact springs
    engage), and the first steps whose contact branches and pair sets differ.
    Before the impact step the difference stays below 1e-6; at it, the FP64
    path's own sensitivity to its solver tolerance (1e-8 against 1e-12) is
    printed beside it."""
    sc, nsteps, contact = scenes.config5_jobs(32)[2]
    assert sc.N == 26 and nsteps == 76 and contact is not None
    runs = {}
    for name, prec, tol in (("mixed", hobak.PRECISION_MIXED, 1e-8), ("fp64", hobak.PRECISION_FP64, 1e-8),
                            ("fp64_tight", hobak.PRECISION_FP64, 1e-12)):
        b = hobak.BATCH([sc], hobak.solver_opts(precision=prec, tol=tol))
        b.set_collisions(0, True, *contact)
        runs[name] = b
    rest = sc.rest.reshape(-1)
    start = {n: b.get_state(0)[0] for n, b in runs.items()}
    split_err = split_branch = split_pairs = None
    worst_before = 0.0
    rows = []
    for k in range(1, nsteps + 1):
        for b in runs.values():
            b.step(1)
        br = {n: contact_branches(runs[n], start[n], rest) for n in ("mixed", "fp64")}
        if split_pairs is None and set(br["mixed"]) != set(br["fp64"]):
            split_pairs = k
        if split_branch is None and br["mixed"] != br["fp64"]:
            split_branch = k
        x = {n: b.get_state(0)[0] for n, b in runs.items()}
        e = rel(x["mixed"] + rest, x["fp64"] + rest)
        e_tol = rel(x["fp64"] + rest, x["fp64_tight"] + rest)
        rows.append((k, len(br["fp64"]), e, e_tol))
        if split_err is None and e > 1e-6:
            split_err = k
        if split_err is None:
            worst_before = max(worst_before, e)
        if split_err is not None and split_branch is not None and split_pairs is not None:
            break
        start = x
    for b in runs.values():
        b.close()
    at = rows[split_err - 1] if split_err else None
    print(f"serving job 2: mixed vs FP64 <= {worst_before:.2e} through step {(split_err or len(rows) + 1) - 1}; "
          f"step {split_err}: {at[1] if at else '-'} pairs, mixed vs FP64 {at[2] if at else 0:.2e}, "
          f"FP64 tol 1e-8 vs 1e-12 {at[3] if at else 0:.2e}; contact branches split at step {split_branch}, "
          f"pair sets at step {split_pairs}")
    assert worst_before < 1e-6
    assert (split_err, split_branch, split_pairs) == SPLIT_STEPS, (split_err, split_branch, split_pairs)
