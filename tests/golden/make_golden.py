"""Generate the golden fixtures in this directory from the reference itself.

Runs the UNMODIFIED reference (HOBAK) through the harness built by
oracle/ref/Makefile (binary oracle/_ref/hobak_ref; needs the reference sources,
so this only runs where they are).  Inputs come from hobakv1_gb300.scenes, so
they are regenerated bit-identically anywhere.  Usage:

    make -C oracle/ref REF=<reference checkout> -j8
    python tests/golden/make_golden.py [elements] [trajectories] [aniso] [position] [newmark] [green] [newmark_contact] [collisions]
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from hobakv1_gb300 import scenes  # noqa: E402
from oracle import refrun  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def element_states(N):
    """Named displacement fields on the N^3 Kuhn cube: rest (F = I up to
    jitter), compressed+twisted, and a seeded large perturbation that inverts
    some tets."""
    rest, tets = scenes.kuhn_cube(N)
    h = 1.0 / N
    twisted = scenes.compress_and_twist(rest, N) - rest
    rng = np.random.default_rng(scenes.BASE_SEED + 77)
    wild = rng.uniform(-0.6 * h, 0.6 * h, size=rest.shape)
    return rest, tets, {"rest": np.zeros_like(rest), "twist": twisted, "wild": wild}


def make_elements():
    """Per-element terms of every material at three states; the anisotropic
    energies with the fibre direction scenes.FIBER (stored as `fiber`)."""
    for mat in scenes.MATERIALS:
        N = 3 if mat in ("snh", "arap") else 2
        rest, tets, states = element_states(N)
        mu, lam = scenes.lame(1e4, 0.45)
        fiber = np.array(scenes.FIBER) if mat in scenes.ANISOTROPIC else None
        for name, x in states.items():
            if mat == "neo_hookean_bw" and name == "wild":
                continue  # log(J) of inverted tets is undefined for this energy
            r = refrun.elements(rest, tets, x, mat, mu, lam, fiber=fiber)
            extra = {"fiber": fiber} if fiber is not None else {}
            np.savez_compressed(os.path.join(OUT, f"elements_{mat}_{name}.npz"),
                                rest=rest, tets=tets, x=x, mu=mu, lam=lam, **extra,
                                **{k: r[k] for k in ["F", "U", "Sigma", "V", "psi", "P", "H9", "H9u", "fe", "He", "R",
                                                     "K_colptr", "K_rowidx", "K_values", "energy",
                                                     "restVolume", "oneRingVolume"]})
            print("elements", mat, name, len(tets))


def make_aniso_trajectories():
    """BACKWARD_EULER_VELOCITY on the 6^3 compressed and twisted cube with
    each anisotropic energy (fibre scenes.FIBER, no gravity), 40 steps."""
    for mat in scenes.ANISOTROPIC:
        s = scenes.aniso_scene(6, mat)
        r = refrun.run(s, 40, stride=10)
        np.savez_compressed(os.path.join(OUT, f"traj_{s.name}.npz"), x=r["x"], v=r["v"],
                            iters=r["iters"], cg_error=r["cg_error"], energy=r["energy"],
                            steps=40, stride=10, fiber=np.array(s.fiber))
        print("aniso trajectory", s.name, r["iters"].sum())


def make_trajectories():
    cases = [(scenes.config1_scene(10), 100, 25),
             (scenes.config2_scene(6, "snh"), 100, 25),
             (scenes.config2_scene(6, "arap"), 100, 25)]
    for s, steps, stride in cases:
        r = refrun.run(s, steps, stride=stride)
        np.savez_compressed(os.path.join(OUT, f"traj_{s.name}.npz"), x=r["x"], v=r["v"],
                            iters=r["iters"], cg_error=r["cg_error"], energy=r["energy"],
                            steps=steps, stride=stride)
        print("trajectory", s.name, r["iters"].sum())


def make_position_trajectories():
    """BACKWARD_EULER_POSITION (Rayleigh damped, alpha = beta = 0.01, the
    reference's defaults) on the same pinned, compressed and twisted cubes."""
    cases = [(scenes.config2_scene(6, "snh"), 100, 25),
             (scenes.config2_scene(6, "arap"), 100, 25),
             (scenes.config1_scene(8), 60, 20)]
    for s, steps, stride in cases:
        r = refrun.run(s, steps, stride=stride, integrator="position", rayleigh=(0.01, 0.01))
        np.savez_compressed(os.path.join(OUT, f"traj_{s.name}_position.npz"), x=r["x"], v=r["v"],
                            iters=r["iters"], cg_error=r["cg_error"], energy=r["energy"],
                            steps=steps, stride=stride, rayleigh=np.array([0.01, 0.01]))
        print("position trajectory", s.name, r["iters"].sum())


def make_newmark_trajectories():
    """NEWMARK (beta 1/4, gamma 1/2, Newton to |rhs|^2 <= 1e-7, at most 10
    iterations) on the pinned, compressed and twisted cubes."""
    cases = [(scenes.config2_scene(6, "snh"), 40, 10),
             (scenes.config2_scene(6, "arap"), 40, 10)]
    for s, steps, stride in cases:
        r = refrun.run(s, steps, stride=stride, integrator="newmark")
        np.savez_compressed(os.path.join(OUT, f"traj_{s.name}_newmark.npz"), x=r["x"], v=r["v"],
                            iters=r["iters"], cg_error=r["cg_error"], energy=r["energy"],
                            steps=steps, stride=stride)
        print("newmark trajectory", s.name, r["iters"].sum())


def make_green_damping():
    """NEWMARK's energy-damped solve with GREEN_DAMPING(mu) (NEWMARK.cpp:
    344-420) on the 5^3 cube hanging under gravity, mu = 0.05 and 1.0, six
    steps each (every step recorded)."""
    s = scenes.config1_scene(5)
    out = {}
    for mu in (0.05, 1.0):
        r = refrun.run(s, 6, integrator="newmark", green_damping=mu)
        tag = f"mu{mu:g}".replace(".", "p")
        out[f"x_{tag}"] = r["x"]
        out[f"v_{tag}"] = r["v"]
        out[f"iters_{tag}"] = r["iters"]
    np.savez_compressed(os.path.join(OUT, f"traj_{s.name}_newmark_green.npz"), steps=6, mus=np.array([0.05, 1.0]),
                        **out)
    print("green damping", s.name)


def make_newmark_contact():
    """NEWMARK with vertex-face contact (detection and response inside the
    Newton loop, NEWMARK.cpp:226-242) on the two 6^3 cubes, collision distance
    1e-3, stiffness 1e3, beta 1e-3, 40 steps."""
    s = scenes.two_cubes_scene(6)
    r = refrun.run(s, 40, stride=10, vf=True, coll_eps=1e-3, coll_mu=1e3, coll_beta=0.001, integrator="newmark")
    np.savez_compressed(os.path.join(OUT, f"traj_{s.name}_newmark_vf.npz"), x=r["x"], v=r["v"], iters=r["iters"],
                        steps=40, stride=10)
    print("newmark contact", s.name, r["iters"].sum())


def make_collisions():
    """Two cubes in contact: vertex-face pairs (reference AABB broad phase +
    narrow phase) at the start and along a 40-step trajectory with collisions."""
    s = scenes.two_cubes_scene(6)
    r = refrun.run(s, 40, stride=10, vf=True, coll_eps=1e-3, coll_mu=1e3, coll_beta=0.001)
    pairs = {}
    for k in range(r["x"].shape[0]):
        c = refrun.collide(s.rest, s.tets, r["x"][k], 1e-3)
        pairs[f"pairs_{k}"] = c["vf_pairs"]
    np.savez_compressed(os.path.join(OUT, f"traj_{s.name}_vf.npz"), x=r["x"], v=r["v"], iters=r["iters"],
                        steps=40, stride=10, surface_triangles=c["surface_triangles"],
                        surface_vertices=c["surface_vertices"], **pairs)
    print("collisions", s.name, [len(v) for v in pairs.values()])


if __name__ == "__main__":
    if not refrun.available():
        sys.exit("reference build missing: make -C oracle/ref REF=<reference checkout>")
    which = set(sys.argv[1:]) or {"elements", "trajectories", "aniso", "position", "newmark", "green",
                                  "newmark_contact", "collisions"}
    if "elements" in which:
        make_elements()
    if "trajectories" in which:
        make_trajectories()
    if "aniso" in which:
        make_aniso_trajectories()
    if "position" in which:
        make_position_trajectories()
    if "newmark" in which:
        make_newmark_trajectories()
    if "green" in which:
        make_green_damping()
    if "newmark_contact" in which:
        make_newmark_contact()
    if "collisions" in which:
        make_collisions()
