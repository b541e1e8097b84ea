"""A C++ host serving jobs with the library's server (hobak_server_*):
tests/cpp/serve_example.cpp compiles and links here; on a GPU its jobs, two
arriving first and the rest while those run (small cohorts, so arrivals are
merged into running ones), end bitwise equal to each scene run alone in its
own batch."""
import os
import subprocess

import numpy as np
import pytest

from hobakv1_gb300 import build, scenes
from hobakv1_gb300.hobak import make_material

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "serve_example.cpp")


def compile_example(tmp_path):
    lib = build.build()
    exe = str(tmp_path / "serve_example")
    cmd = ["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L" + os.path.dirname(lib), "-lhobak_gpu", "-Wl,-rpath," + os.path.dirname(lib)]
    subprocess.run(cmd, check=True)
    return exe


def test_cpp_serve_example_compiles_and_links(tmp_path):
    assert os.path.exists(compile_example(tmp_path))


@pytest.mark.gpu
def test_cpp_served_jobs_equal_alone(tmp_path):
    exe = compile_example(tmp_path)
    mix = scenes.config4_scenes(count=5, nmin=5, nmax=8)
    nsteps = [7, 3, 11, 6, 4]
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        np.array([len(mix)], dtype=np.int32).tofile(f)
        for s, n in zip(mix, nsteps):
            m = make_material(s.material, s.mu, s.lam)._c()
            np.array([s.nv, s.nt, len(s.pinned), n, m.kind], dtype=np.int32).tofile(f)
            np.array([m.mu, m.lambda_, s.density, s.dt, *s.gravity], dtype=np.float64).tofile(f)
            s.rest.astype(np.float64).tofile(f)
            s.tets.astype(np.int32).tofile(f)
            np.asarray(s.pinned, dtype=np.int32).tofile(f)
            (s.x0 if s.x0 is not None else np.zeros(3 * s.nv)).astype(np.float64).tofile(f)
    r = subprocess.run([exe, str(inp), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    print(r.stdout.strip())
    data = np.fromfile(out, dtype=np.float64)
    at = 0
    for s in mix:
        n = 3 * s.nv
        served_x, served_v, alone_x, alone_v = (data[at + k * n:at + (k + 1) * n] for k in range(4))
        at += 4 * n
        assert np.array_equal(served_x, alone_x) and np.array_equal(served_v, alone_v)
    assert at == len(data)
