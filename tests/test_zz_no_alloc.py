"""The allocation-free Dirichlet entry point (vpmg_dirichlet_static).

Some callers cannot let a library allocate GPU memory: a host code whose
own pool allocator owns the whole device, or one that runs inside a fixed
memory budget where one more cudaMalloc would fail.  For them the library
exports one solve whose temporaries live in a static device array.  These
tests call it through the C-ABI on device buffers the caller owns and
check it against the oracle's Dirichlet solve and the allocating entry
point (vpmg_pmesh with iynbc = 0), with the tolerance of the other
Dirichlet parity tests, on calls in a row that share the static array:
an even and an odd line length (the real-symmetric and the odd-extension
transforms), zero and given boundary values, a smaller grid after a larger
one, and long lines along x near the array's bounds.  They also check that
the calls allocate nothing.  The file sits last in pytest's collection
order.
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


def _allocating(V, rhs, sol, d, zero_bc):
    """The same solve through vpmg_pmesh(iynbc = 0); zero_bc: faces zeroed first."""
    nz, ny, nx = rhs.shape
    cfg = V.VPMConfig.make(dpm=d, box=(0, 0, 0, 8 * d[0], 8 * d[1], 8 * d[2]))
    s0 = sol.copy()
    if zero_bc:
        s0[0], s0[-1], s0[:, 0], s0[:, -1], s0[:, :, 0], s0[:, :, -1] = 0, 0, 0, 0, 0, 0
    with V.VPM(cfg) as h:
        out = [s0.copy(), s0.copy(), s0.copy()]
        h.pmesh(out, [rhs, rhs, rhs], (0.0, 0.0, 0.0, 1.0, 1.0, 1.0), d, iynbc=0, NN_bl=(1, 1, 1, nx, ny, nz))
    return out[0]


def _call(V, torch, fn, rhs, sol, d, zero_bc):
    nz, ny, nx = rhs.shape
    dims = (C.c_int * 3)(nx, ny, nz)
    box = (C.c_int * 6)(0, 0, 0, nx - 1, ny - 1, nz - 1)
    hh = (C.c_double * 3)(*d)
    d_rhs = torch.from_numpy(rhs).cuda()
    d_sol = torch.from_numpy(sol).cuda()
    torch.cuda.synchronize()
    rc = fn(C.c_void_p(d_rhs.data_ptr()), C.c_void_p(d_sol.data_ptr()), dims, box, hh, int(zero_bc), None)
    assert rc == 0, V.load_library().vpmg_status_string(rc)
    torch.cuda.synchronize()
    return d_sol.cpu().numpy()


# (nz, ny, nx), spacings, zero_bc: even N, odd N (nx = 34: 32 interior, N = 33,
# transform length 66), zero faces, a smaller grid after the larger ones, and
# long lines along x near the array's bounds: 899 interior nodes (N = 900 =
# 2^2 3^2 5^2, the longest accepted line whose transform factors into radices
# up to 17) and 874 (N = 875 odd, transform length 1750 of the 1802 the twiddle
# tables hold)
CASES = [((37, 29, 33), (0.05, 0.07, 0.06), 0),
         ((21, 26, 34), (0.04, 0.05, 0.03), 0),
         ((23, 19, 27), (0.06, 0.05, 0.07), 1),
         ((9, 11, 13), (0.1, 0.2, 0.15), 0),
         ((4, 4, 901), (0.01, 0.3, 0.2), 0),
         ((4, 5, 876), (0.01, 0.3, 0.2), 1)]


def _need_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_static_dirichlet_matches_oracle_and_allocating_entry(gpulib, oracle):
    torch = _need_cuda()
    V = gpulib
    fn = _static_fn(V)
    rng = np.random.default_rng(2024)
    for k, (shape, d, zero_bc) in enumerate(CASES):  # consecutive calls share the static array
        rhs = rng.standard_normal(shape)
        sol = rng.standard_normal(shape)  # faces = Dirichlet values unless zero_bc
        got = _call(V, torch, fn, rhs, sol, d, zero_bc)
        ref_o = sol.copy()
        oracle.dirichlet(rhs, ref_o, d, zero_bc=bool(zero_bc))
        assert rel_l2(got, ref_o) <= TOL, (k, rel_l2(got, ref_o))
        assert rel_l2(got, _allocating(V, rhs, sol, d, zero_bc)) <= TOL, k
        faces = [np.s_[0], np.s_[-1], np.s_[:, 0], np.s_[:, -1], np.s_[:, :, 0], np.s_[:, :, -1]]
        for f in faces:
            assert np.array_equal(got[f], np.zeros_like(sol[f]) if zero_bc else sol[f]), (k, f)


def test_static_dirichlet_two_calls_in_a_row_agree(gpulib):
    """The same solve twice in a row returns the same bits (the second call
    starts from whatever the first left in the array)."""
    torch = _need_cuda()
    V = gpulib
    fn = _static_fn(V)
    rng = np.random.default_rng(7)
    shape, d = (25, 31, 29), (0.05, 0.06, 0.07)
    rhs, sol = rng.standard_normal(shape), rng.standard_normal(shape)
    a = _call(V, torch, fn, rhs, sol, d, 0)
    b = _call(V, torch, fn, rhs, sol, d, 0)
    assert np.array_equal(a, b)


def test_static_dirichlet_allocates_nothing(gpulib):
    """After a first call (the device's set-up), further calls leave the
    device's free memory unchanged: nothing is allocated."""
    torch = _need_cuda()
    V = gpulib
    fn = _static_fn(V)
    shape = (33, 35, 31)
    nz, ny, nx = shape
    dims = (C.c_int * 3)(nx, ny, nz)
    box = (C.c_int * 6)(0, 0, 0, nx - 1, ny - 1, nz - 1)
    hh = (C.c_double * 3)(0.1, 0.1, 0.1)
    a = torch.randn(nz * ny * nx, dtype=torch.float64, device="cuda")
    b = torch.randn(nz * ny * nx, dtype=torch.float64, device="cuda")
    assert fn(C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()), dims, box, hh, 0, None) == 0
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for zbc in (0, 1, 0, 1):
        assert fn(C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()), dims, box, hh, zbc, None) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_static_dirichlet_rejects_oversize(gpulib):
    torch = _need_cuda()
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
    nx, ny, nz = 140, 140, 140  # 138^3 interior nodes: over the 2^21 limit
    dims = (C.c_int * 3)(nx, ny, nz)
    box = (C.c_int * 6)(0, 0, 0, nx - 1, ny - 1, nz - 1)
    rc = fn(C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()), dims, box, hh, 0, None)
    torch.cuda.synchronize()
    assert rc == -1
    assert float(b.abs().max()) == 0.0
