"""Full-size accuracy of the FP64 and mixed-precision paths against the FP64
oracle: the 40^3 compressed and twisted Kuhn cube (68,921 vertices, 384,000
tets, E = 1e4, nu = 0.45), once with Stable Neo-Hookean and once with ARAP,
100 steps of BACKWARD_EULER_VELOCITY with block-Jacobi PCG to 1e-8 (about a
minute of oracle time per material on 16 host cores).

Bounds: FP64 relative L2 position error <= 1e-8 and mixed precision <= 1e-6,
at every checkpoint (steps 25, 50, 75, 100).  Measured per path and printed
(and written as JSON to $HOBAK_REPORT when set): relative L2 position error,
max per-vertex position error over the cube's extent, RMS position error over
the extent, and the relative difference of the hyperelastic energy
(TET_MESH::computeHyperelasticEnergy, TET_MESH.cpp:719-731)."""
import json
import os

import numpy as np
import pytest

from hobakv1_gb300 import hobak, scenes
from oracle import oracle

pytestmark = pytest.mark.gpu

STEPS = 100
CHECK = (25, 50, 75, 100)
BOUNDS = {"fp64": 1e-8, "mixed": 1e-6}


def errors(x, xo, rest, extent):
    px, po = x + rest, xo + rest
    d = (px - po).reshape(-1, 3)
    return {"rel_l2": float(np.linalg.norm(px - po) / np.linalg.norm(po)),
            "max_over_extent": float(np.linalg.norm(d, axis=1).max() / extent),
            "rms_over_extent": float(np.sqrt((d ** 2).sum(axis=1).mean()) / extent)}


@pytest.mark.parametrize("material", ["snh", "arap"])
def test_kuhn40_100_steps_fp64_and_mixed(material):
    s = scenes.config2_scene(40, material)
    rest = s.rest.reshape(-1)
    extent = float(np.linalg.norm(s.rest.max(axis=0) - s.rest.min(axis=0)))
    sim = oracle.Sim(s, precond=hobak.PRECOND_BLOCK_JACOBI)
    ref = {}
    done = 0
    for k in CHECK:
        sim.step(k - done)
        done = k
        ref[k] = (sim.state()[0], sim.energy())
    report = {"scene": f"kuhn40_{material}_twist", "steps": STEPS, "tol": 1e-8}
    for name, prec in (("fp64", hobak.PRECISION_FP64), ("mixed", hobak.PRECISION_MIXED)):
        b = hobak.BATCH([s], hobak.solver_opts(precision=prec))
        done = 0
        rows = {}
        for k in CHECK:
            b.step(k - done)
            done = k
            x, _ = b.get_state(0)
            e = errors(x, ref[k][0], rest, extent)
            e["energy_rel"] = float(abs(b.energy(0) - ref[k][1]) / abs(ref[k][1]))
            rows[k] = e
        b.close()
        report[name] = rows
    print(json.dumps(report))
    if os.environ.get("HOBAK_REPORT"):
        path = os.environ["HOBAK_REPORT"]
        prev = json.load(open(path)) if os.path.exists(path) else {}
        prev[material] = report
        with open(path, "w") as f:
            json.dump(prev, f, indent=1)
    for name, bound in BOUNDS.items():
        for k in CHECK:
            assert report[name][k]["rel_l2"] < bound, (name, k, report[name][k])
