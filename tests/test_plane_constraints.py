"""Plane constraints (kinematic collision objects) on the reference's two-tet
contact scenes.

The scenes register their lower cube as a collision object
(addKinematicCollisionObject; TWO_TET_DROP_VF.h:72, TWO_TET_DROP_EE.h:72,
TWO_TET_KISS_VF.h:77, TWO_TET_KISS_EE.h:77).  Every solve,
TIMESTEPPER::findNewSurfaceConstraints (TIMESTEPPER.cpp:446-524) adds a plane
constraint only for a surface vertex that is inside such an object
(CUBE::inside, CUBE.cpp:44-55) and moving into it, and buildConstraintMatrix
(TIMESTEPPER.cpp:128-171) lets the kinematic pins override it.  So a vertex
that is pinned, or never inside a collision object, never carries one.

This checks, on the trajectories of the reference built from its own
sources (the golden fixtures, every frame), that no unpinned vertex is ever
inside a collision object, and by how much: the constraint set stays empty
on these scenes, which is why the drop-in builds no plane constraints.  The
GPU trajectories match these to 1e-8 (test_gpu_regression.py), far inside
the margin."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
LOWER, UPPER = ((0.0, -4.90, 0.0), 10.0), ((0.0, 6.9, 0.0), 10.0)
# (kinematic shapes the surface vertices inside are pinned to, collision objects)
SCENES = {
    "two_tet_drop_vf": ((LOWER,), (LOWER,)),
    "two_tet_drop_ee": ((LOWER,), (LOWER,)),
    "two_tet_kiss_vf": ((LOWER, UPPER), (LOWER,)),
    "two_tet_kiss_ee": ((LOWER, UPPER), (LOWER,)),
}


def cube_gap(p, shape):
    """How far outside the axis-aligned cube (center, scale) the points are,
    in the max norm: <= 0 means inside (CUBE::inside on the local unit cube)."""
    center, scale = shape
    return np.max(np.abs(p - np.asarray(center)), axis=-1) - 0.5 * scale


@pytest.mark.parametrize("name", sorted(SCENES))
def test_no_unpinned_vertex_enters_a_collision_object(name):
    g = np.load(os.path.join(GOLDEN, f"regression_{name}.npz"))
    pins, objects = SCENES[name]
    rest = g["rest"]
    # attachKinematicSurfaceConstraints: the surface vertices inside a shape
    # at rest are pinned (every vertex of these two-tet meshes is on the surface)
    pinned = np.zeros(len(rest), bool)
    for s in pins:
        pinned |= cube_gap(rest, s) <= 0
    free = ~pinned
    assert pinned.any() and free.any()
    margin = np.inf
    for k in range(int(g["total_frames"])):
        world = rest + g["ref_position"][k].reshape(-1, 3)
        for s in objects:
            margin = min(margin, float(cube_gap(world[free], s).min()))
    print(f"{name}: closest approach of an unpinned vertex to a collision object {margin:.4f}")
    assert margin > 0.25, margin
