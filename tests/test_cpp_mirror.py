"""The C++ mirror of the reference interface (hobakv1_gb300/cpp/HOBAK_GPU.h):
compiles and links against libhobak_gpu.so here; on a GPU it steps a scene
the way the reference's scenes do and matches the oracle."""
import os
import subprocess

import numpy as np
import pytest

from hobakv1_gb300 import build, scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "bev_gpu_example.cpp")


def compile_example(tmp_path):
    lib = build.build()
    exe = str(tmp_path / "bev_gpu_example")
    cmd = ["g++", "-O2", "-std=c++17", SRC, "-o", exe, "-L" + os.path.dirname(lib), "-lhobak_gpu",
           "-Wl,-rpath," + os.path.dirname(lib)]
    subprocess.run(cmd, check=True)
    return exe


def test_cpp_mirror_compiles_and_links(tmp_path):
    assert os.path.exists(compile_example(tmp_path))


@pytest.mark.gpu
def test_cpp_mirror_solve_matches_oracle(tmp_path):
    from oracle import oracle
    exe = compile_example(tmp_path)
    s = scenes.config2_scene(6, "arap")
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        np.array([s.nv, s.nt, len(s.pinned), 1], dtype=np.int32).tofile(f)
        np.array([s.mu, s.lam, s.density, s.dt], dtype=np.float64).tofile(f)
        s.rest.astype(np.float64).tofile(f)
        s.tets.astype(np.int32).tofile(f)
        s.pinned.astype(np.int32).tofile(f)
        s.x0.astype(np.float64).tofile(f)
    for integrator in ("velocity", "position", "newmark"):
        subprocess.run([exe, str(inp), str(out), "10"] + ([integrator] if integrator != "velocity" else []),
                       check=True)
        xv = np.fromfile(out, dtype=np.float64)
        x, v = xv[:3 * s.nv], xv[3 * s.nv:]
        sim = oracle.Sim(s, precond=1, integrator=integrator)
        sim.step(10)
        xo, vo = sim.state()
        assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-9, integrator
        assert np.linalg.norm(v - vo) / np.linalg.norm(vo) < 1e-8, integrator


@pytest.mark.gpu
def test_cpp_mirror_moving_pins_match_the_reference_regression_record(tmp_path):
    """NEWMARK_STRETCH through the C++ mirror (pins attached to two cube
    shapes with attachKinematicSurfaceConstraints, one cube moved between
    solves) against the reference's recorded last frame, at its 1e-8."""
    exe = compile_example(tmp_path)
    g = np.load(os.path.join(ROOT, "tests", "golden", "regression_newmark_stretch.npz"))
    rest, tets = g["rest"], g["tets"]
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        np.array([len(rest), len(tets), 0, 0], dtype=np.int32).tofile(f)
        np.array([1.0, 10.0, 1.0, float(g["dt"])], dtype=np.float64).tofile(f)
        rest.astype(np.float64).tofile(f)
        tets.astype(np.int32).tofile(f)
        np.zeros(3 * len(rest)).tofile(f)
    n = int(g["total_frames"])
    subprocess.run([exe, str(inp), str(out), str(n), "stretch"], check=True)
    xv = np.fromfile(out, dtype=np.float64)
    x, v = xv[:3 * len(rest)], xv[3 * len(rest):]
    assert int(g["frames"][-1]) == n - 1
    assert np.linalg.norm(x - g["position"][-1]) / np.linalg.norm(g["position"][-1]) < 1e-8
    assert np.linalg.norm(v - g["velocity"][-1]) / np.linalg.norm(g["velocity"][-1]) < 1e-6
