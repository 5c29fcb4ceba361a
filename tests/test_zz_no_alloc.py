"""The allocation-free Dirichlet entry point (vpmg_dirichlet_static).

Some callers cannot let a library allocate GPU memory (their own pool
owns the device, or they run under a fixed memory budget).  For them the
library exports one solve whose temporaries live in a static device array.
This test calls it through the C-ABI on device buffers the caller owns and
checks it against the allocating entry point (vpmg_pmesh with iynbc = 0) on
two calls in a row, with the tolerance of the other Dirichlet parity tests.
It sits in a file of its own that pytest collects last.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _static_fn(V):
    L = V.load_library()
    f = L.vpmg_dirichlet_static
    f.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_int,
                  C.c_void_p]
    f.restype = C.c_int
    return f


def _reference(V, rhs, sol, d):
    nz, ny, nx = rhs.shape
    cfg = V.VPMConfig.make(dpm=d, box=(0, 0, 0, 8 * d[0], 8 * d[1], 8 * d[2]))
    with V.VPM(cfg) as h:
        out = [sol.copy(), sol.copy(), sol.copy()]
        h.pmesh(out, [rhs, rhs, rhs], (0.0, 0.0, 0.0, 1.0, 1.0, 1.0), d, iynbc=0, NN_bl=(1, 1, 1, nx, ny, nz))
    return out[0]


def test_static_dirichlet_matches_allocating_entry(gpulib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    V = gpulib
    fn = _static_fn(V)
    rng = np.random.default_rng(2024)
    shape = (37, 29, 33)  # (nz, ny, nx)
    nz, ny, nx = shape
    d = (0.05, 0.07, 0.06)
    dims = (C.c_int * 3)(nx, ny, nz)
    box = (C.c_int * 6)(0, 0, 0, nx - 1, ny - 1, nz - 1)
    hh = (C.c_double * 3)(*d)
    for call in range(2):  # two calls in a row share the static array
        rhs = rng.standard_normal(shape)
        sol = rng.standard_normal(shape)  # faces = Dirichlet values
        ref = _reference(V, rhs, sol, d)
        d_rhs = torch.from_numpy(rhs).cuda()
        d_sol = torch.from_numpy(sol).cuda()
        torch.cuda.synchronize()
        rc = fn(C.c_void_p(d_rhs.data_ptr()), C.c_void_p(d_sol.data_ptr()), dims, box, hh, 0, None)
        assert rc == 0, V.load_library().vpmg_status_string(rc)
        torch.cuda.synchronize()
        got = d_sol.cpu().numpy()
        assert rel_l2(got, ref) <= TOL, call
        assert np.array_equal(got[0], sol[0]) and np.array_equal(got[:, :, -1], sol[:, :, -1])


def test_static_dirichlet_rejects_oversize(gpulib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    V = gpulib
    fn = _static_fn(V)
    nx, ny, nz = 1000, 1000, 10  # 998 interior nodes along x: over the 900 limit
    a = torch.zeros(nx * ny * nz, dtype=torch.float64, device="cuda")
    b = torch.zeros(nx * ny * nz, dtype=torch.float64, device="cuda")
    dims = (C.c_int * 3)(nx, ny, nz)
    box = (C.c_int * 6)(0, 0, 0, nx - 1, ny - 1, nz - 1)
    hh = (C.c_double * 3)(0.1, 0.1, 0.1)
    rc = fn(C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()), dims, box, hh, 0, None)
    torch.cuda.synchronize()
    assert rc == -1
    assert float(b.abs().max()) == 0.0  # refused before any GPU work
