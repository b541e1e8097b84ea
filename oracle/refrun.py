"""Runs the reference build (oracle/_ref/hobak_ref) on a scene.

Test infrastructure (oracle): used only by tests/golden/make_golden.py and the
oracle validation tests, never by the product library.  The binary exists only
where the reference sources are present (the build recipe is
oracle/ref/Makefile).
"""
from __future__ import annotations

import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_BIN = os.path.join(HERE, "_ref", "hobak_ref")


def available() -> bool:
    return os.path.exists(REF_BIN)


def _write_mesh(d, rest, tets):
    np.save(os.path.join(d, "rest.npy"), np.ascontiguousarray(rest, dtype=np.float64))
    np.save(os.path.join(d, "tets.npy"), np.ascontiguousarray(tets, dtype=np.int32))


def _read_dir(d):
    return {f[:-4]: np.load(os.path.join(d, f)) for f in os.listdir(d) if f.endswith(".npy")}


def elements(rest, tets, x, material, mu, lam, fiber=None):
    """Per-tet F, svd_rv, psi, PK1, clamped and unclamped Hessians, element
    force/Hessian, R and CSC K (fiber: the anisotropic energies' direction)."""
    with tempfile.TemporaryDirectory() as tin, tempfile.TemporaryDirectory() as tout:
        _write_mesh(tin, rest, tets)
        if fiber is not None:
            np.save(os.path.join(tin, "fiber.npy"), np.asarray(fiber, dtype=np.float64))
        np.save(os.path.join(tin, "x.npy"), np.ascontiguousarray(x, dtype=np.float64).reshape(-1))
        subprocess.run([REF_BIN, "elements", tin, tout, material, repr(float(mu)), repr(float(lam))],
                       check=True, stdout=subprocess.DEVNULL)
        return _read_dir(tout)


def run(scene, steps, stride=1, tol=1e-8, maxit=1000, vf=False, ee=False,
        coll_eps=0.01, coll_mu=1.0, coll_beta=0.001, threads=None, integrator="velocity",
        rayleigh=(0.01, 0.01), green_damping=0.0):
    """BACKWARD_EULER_VELOCITY::solve (integrator "velocity"),
    BACKWARD_EULER_POSITION::solve (integrator "position", Rayleigh damped
    with alpha, beta = rayleigh) or NEWMARK::solve (integrator "newmark")
    for `steps` steps on `scene`."""
    with tempfile.TemporaryDirectory() as tin, tempfile.TemporaryDirectory() as tout:
        _write_mesh(tin, scene.rest, scene.tets)
        if getattr(scene, "fiber", None) is not None:
            np.save(os.path.join(tin, "fiber.npy"), np.asarray(scene.fiber, dtype=np.float64))
        np.save(os.path.join(tin, "x0.npy"), scene.x0.reshape(-1).astype(np.float64))
        np.save(os.path.join(tin, "v0.npy"), scene.v0.reshape(-1).astype(np.float64))
        np.save(os.path.join(tin, "pinned.npy"), scene.pinned.astype(np.int32))
        g = scene.gravity
        params = np.array([scene.density, g[0], g[1], g[2], scene.dt, tol, maxit,
                           float(vf), float(ee), coll_eps, coll_mu, coll_beta,
                           {"velocity": 0.0, "position": 1.0, "newmark": 2.0}[integrator], rayleigh[0], rayleigh[1],
                           green_damping],
                          dtype=np.float64)
        np.save(os.path.join(tin, "params.npy"), params)
        env = dict(os.environ)
        if threads:
            env["OMP_NUM_THREADS"] = str(threads)
        subprocess.run([REF_BIN, "run", tin, tout, scene.material, repr(float(scene.mu)),
                        repr(float(scene.lam)), str(steps), str(stride)],
                       check=True, stdout=subprocess.DEVNULL, env=env)
        return _read_dir(tout)


def collide(rest, tets, x, eps):
    """Vertex-face collision pairs at displacement x."""
    with tempfile.TemporaryDirectory() as tin, tempfile.TemporaryDirectory() as tout:
        _write_mesh(tin, rest, tets)
        np.save(os.path.join(tin, "x.npy"), np.ascontiguousarray(x, dtype=np.float64).reshape(-1))
        subprocess.run([REF_BIN, "collide", tin, tout, repr(float(eps))], check=True,
                       stdout=subprocess.DEVNULL)
        return _read_dir(tout)
