"""hobak_element_eval_noalloc: the entry point for callers that cannot let the
library allocate device memory (plugins in hosts that own the GPU memory
budget, per-frame loops where cudaMalloc would synchronise the device).

The caller owns every device buffer (torch tensors here); the call must give
the same element terms as the allocating hobak_element_eval on the same inputs,
call after call, even though all calls share one static scratch array.  This
file sorts last so a failure here cannot hide the other tests' results."""
import ctypes

import numpy as np
import pytest

from hobakv1_gb300 import _lib, hobak, scenes

pytestmark = pytest.mark.gpu
MAX_TETS = 131072  # HOBAK_NOALLOC_MAX_TETS in include/hobak_gpu.h


def relmax(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def noalloc_eval(rest, tets, x, material):
    import torch
    dev = torch.device("cuda")
    nv, nt = rest.shape[0], tets.shape[0]
    d_rest = torch.from_numpy(np.ascontiguousarray(rest, dtype=np.float64).reshape(-1)).to(dev)
    d_tets = torch.from_numpy(np.ascontiguousarray(tets, dtype=np.int32).reshape(-1)).to(dev)
    d_x = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64).reshape(-1)).to(dev)
    out = {k: torch.zeros(nt * n, dtype=torch.float64, device=dev)
           for k, n in [("F", 9), ("Sigma", 3), ("force", 12), ("hessian", 144)]}
    mat = material._c()
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    rc = _lib.load().hobak_element_eval_noalloc(nv, nt, d_rest.data_ptr(), d_tets.data_ptr(), d_x.data_ptr(),
                                                ctypes.byref(mat), out["F"].data_ptr(), out["Sigma"].data_ptr(),
                                                out["force"].data_ptr(), out["hessian"].data_ptr(), stream)
    return rc, {k: v.cpu().numpy().reshape(nt, -1) for k, v in out.items()}


def allocating_eval(rest, tets, x, material):
    mesh = hobak.TET_MESH(rest, tets)
    mesh.setDisplacement(x)
    return mesh.computeElements(material)


def test_noalloc_matches_allocating_entry_point_on_consecutive_calls():
    # call 1: 6^3 compressed/twisted SNH; call 2: a smaller, different ARAP
    # mesh and state, so stale scratch from call 1 would show up as a mismatch
    s1 = scenes.config2_scene(6, "snh")
    rest2, tets2 = scenes.kuhn_cube(3)
    rng = np.random.default_rng(5)
    x2 = rng.uniform(-0.15, 0.15, size=rest2.shape)
    cases = [(s1.rest, s1.tets, s1.x0, hobak.SNH(s1.mu, s1.lam)),
             (rest2, tets2, x2, hobak.ARAP(3448.0, 31034.0))]
    for rest, tets, x, mat in cases:
        rc, got = noalloc_eval(rest, tets, x, mat)
        assert rc == 0, _lib.load().hobak_last_error().decode()
        ref = allocating_eval(rest, tets, x, mat)
        for k in ("F", "Sigma", "force", "hessian"):
            assert relmax(got[k], ref[k]) < 1e-10, (k, relmax(got[k], ref[k]))


def test_noalloc_rejects_oversize_and_bad_indices_then_still_works():
    import torch
    L = _lib.load()
    s = scenes.config1_scene(2)
    mat = hobak.SNH(s.mu, s.lam)
    cm = mat._c()
    buf = torch.zeros(1024, dtype=torch.float64, device="cuda")
    tbuf = torch.zeros(1024, dtype=torch.int32, device="cuda")
    rc = L.hobak_element_eval_noalloc(s.nv, MAX_TETS + 1, buf.data_ptr(), tbuf.data_ptr(), buf.data_ptr(),
                                      ctypes.byref(cm), None, None, None, None, None)
    assert rc == -1 and b"scratch limit" in L.hobak_last_error()
    bad = s.tets.copy()
    bad[5, 1] = s.nv + 7  # caught by the kernel's bounds check before any element work
    rc, _ = noalloc_eval(s.rest, bad, s.x0, mat)
    assert rc == -1 and b"outside [0, nv)" in L.hobak_last_error()
    rc, got = noalloc_eval(s.rest, s.tets, s.x0, mat)
    assert rc == 0
    ref = allocating_eval(s.rest, s.tets, s.x0, mat)
    assert relmax(got["hessian"], ref["hessian"]) < 1e-10
