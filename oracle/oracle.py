"""ctypes binding of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
the checker, and by bench.py's cpu_baseline / reference arm.  The product
package vpm_free_gb300 never imports this module.

The oracle restates the reference's Fortran hot path (source/vpm.f90,
pmproject.f90, pmlib.f90, pmsolve.f90, pinfdomain.f90, pmbound.f90,
yaps3d.f90, vpm_gcalc.f90, vpm_time.f90, vpm_remesh.f90, test.f90) in C++;
each routine cites the reference lines it follows.
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


class Config(C.Structure):
    """pm.inp contents (source/vpm.f90:132-152) plus an explicit-box option."""
    _fields_ = [
        ("dpm", C.c_double * 3), ("interf_iproj", C.c_int), ("ibctyp", C.c_int), ("idvpm", C.c_int),
        ("epsvol", C.c_double), ("ncoarse", C.c_int), ("nbi", C.c_int), ("nbj", C.c_int), ("nbk", C.c_int),
        ("nremesh", C.c_int), ("ncell_rem", C.c_int), ("iyntree", C.c_int), ("ilevmax", C.c_int),
        ("ompthreads", C.c_int), ("idefine", C.c_int), ("iynslice", C.c_int), ("use_box", C.c_int),
        ("box", C.c_double * 6),
    ]


class Sizes(C.Structure):
    """Mesh descriptors of define_sizes (source/vpm.f90:477-660)."""
    _fields_ = [
        ("xbound", C.c_double * 6), ("dpm", C.c_double * 3), ("nn", C.c_int * 3), ("nn_bl", C.c_int * 6),
        ("xbound_bl", C.c_double * 6), ("nnbl", C.c_int * 3), ("nnbl_bl", C.c_int * 6),
        ("xbound_coarse", C.c_double * 6), ("dpm_coarse", C.c_double * 3), ("nn_coarse", C.c_int * 3),
        ("nn_bl_coarse", C.c_int * 6), ("ilevmax", C.c_int), ("dvpm", C.c_double), ("defined", C.c_int),
    ]


F_RHS, F_SOL, F_VEL, F_DEF, F_BL_SOL1, F_COARSE_RHS, F_COARSE_SOL, F_BL_FINAL = range(8)

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_PP = C.POINTER(C.c_double) * 3


def build():
    """Compile liboracle.so from oracle/vpm_oracle.cpp (make)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        L.vpmo_definepm.argtypes = [C.c_int, _dp, _dp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.vpmo_define_sizes.argtypes = [C.POINTER(Config), C.c_void_p, C.c_int, C.c_int, C.POINTER(Sizes)]
        L.vpmo_projection_fun.argtypes = [C.c_int, C.c_double]
        L.vpmo_projection_fun.restype = C.c_double
        L.vpmo_project_particles.argtypes = [C.POINTER(Sizes), C.c_int, _dp, _dp, C.c_int, _dp, _dp, _dp, C.c_int]
        L.vpmo_dirichlet.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), _dp, _dp, _dp, C.c_int, C.c_int]
        L.vpmo_pmesh.argtypes = [_PP, _PP, _dp, _dp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int, C.c_int, C.c_int, C.c_int]
        L.vpmo_step_fields.argtypes = [C.POINTER(Config), C.POINTER(Sizes), _dp, _dp, _dp, _dp, C.c_int, C.c_int]
        L.vpmo_get_field.argtypes = [C.c_int, C.c_void_p, C.c_long]
        L.vpmo_get_field.restype = C.c_long
        L.vpmo_euler.argtypes = [_dp, _dp, _dp, _dp, C.c_int, C.c_double, _dp]
        L.vpmo_remesh.argtypes = [C.POINTER(Config), C.POINTER(Sizes), _dp, _dp, C.c_int, _dp, _dp, C.c_long, C.c_int]
        L.vpmo_remesh.restype = C.c_long
        L.vpmo_diffuse.argtypes = [C.POINTER(Config), C.POINTER(Sizes), _dp, _dp, C.c_double, _dp, C.c_int, C.c_int]
        L.vpmo_whattodo4.argtypes = [C.POINTER(Config), C.POINTER(Sizes), _dp, _dp, _dp, _dp, C.c_int, C.c_int]
        L.vpmo_remesh_masked.argtypes = [C.POINTER(Config), C.POINTER(Sizes), _dp, _dp, C.c_int, _dp, _dp, C.c_long,
                                         C.c_int, C.POINTER(C.c_int), C.c_int]
        L.vpmo_remesh_masked.restype = C.c_long
        L.vpmo_boundary_values.argtypes = [_PP, _PP, _dp, _dp, C.POINTER(C.c_int), C.c_int, C.c_int, C.c_int]
        L.vpmo_boundary_values.restype = C.c_long
        L.vpmo_boundary_values_bc.argtypes = [_PP, _PP, _dp, _dp, C.POINTER(C.c_int), C.c_int, C.c_int, C.c_int,
                                              C.c_int]
        L.vpmo_boundary_values_bc.restype = C.c_long
        L.vpmo_pmesh_bc.argtypes = [_PP, _PP, _dp, _dp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int, C.c_int,
                                    C.c_int, C.c_int, C.c_int]
        L.vpmo_fsour_a4.argtypes = [_dp, _dp, C.c_int, _dp, C.c_double]
        L.vpmo_fsour_a4.restype = C.c_double
        L.vpmo_yaps_seam.restype = C.c_double
        _LIB = L
    return _LIB


def _ivec(v):
    return (C.c_int * len(v))(*[int(x) for x in v])


def _pp(arrs):
    return _PP(*[a.ctypes.data_as(C.POINTER(C.c_double)) for a in arrs])


def make_config(dpm=(0.05, 0.05, 0.05), interf_iproj=4, ibctyp=2, idvpm=1, epsvol=0.0, ncoarse=8, nb=(1, 1, 1),
                nremesh=1, ncell_rem=1, iyntree=1, ilevmax=3, ompthreads=1, idefine=1, iynslice=0, box=None):
    c = Config()
    c.dpm[:] = list(dpm)
    c.interf_iproj, c.ibctyp, c.idvpm, c.epsvol, c.ncoarse = interf_iproj, ibctyp, idvpm, epsvol, ncoarse
    c.nbi, c.nbj, c.nbk = nb
    c.nremesh, c.ncell_rem, c.iyntree, c.ilevmax = nremesh, ncell_rem, iyntree, ilevmax
    c.ompthreads, c.idefine, c.iynslice = ompthreads, idefine, iynslice
    if box is not None:
        c.use_box = 1
        c.box[:] = list(box)
    return c


def definepm(itype, xbound, dpm, ndum, nsize):
    xb = np.array(xbound, dtype=np.float64)
    d = np.array(dpm, dtype=np.float64)
    nn = (C.c_int * 3)()
    nnbl = (C.c_int * 6)()
    lib().vpmo_definepm(itype, xb, d, ndum, _ivec(nsize), nn, nnbl)
    return xb, d, list(nn), list(nnbl)


def define_sizes(cfg, xp, ntime=0, sizes=None):
    """xp: (nvr, 3) C-order (= Fortran XP(3,nvr))."""
    s = sizes if sizes is not None else Sizes()
    xp = np.ascontiguousarray(xp, dtype=np.float64)
    rc = lib().vpmo_define_sizes(C.byref(cfg), xp.ctypes.data if xp.size else None, int(xp.shape[0]), ntime, C.byref(s))
    if rc != 0:
        raise RuntimeError(f"vpmo_define_sizes failed: {rc}")
    return s


def dirichlet(rhs, sol, d, box=None, zero_bc=False, nthreads=0):
    """rhs, sol: arrays shaped (nz, ny, nx) (x fastest); sol modified in place."""
    nz, ny, nx = rhs.shape
    if box is None:
        box = (1, 1, 1, nx, ny, nz)
    lib().vpmo_dirichlet(nx, ny, nz, _ivec(box), np.asarray(d, dtype=np.float64),
                         np.ascontiguousarray(rhs), sol, 1 if zero_bc else 0, nthreads)
    return sol


def pmesh(sol, rhs, xbound, dpm, iynbc, itree, levmax, nn_bl=None, nthreads=0, ibctyp=2):
    """sol, rhs: lists of 3 arrays (nz, ny, nx); sol modified in place."""
    nz, ny, nx = rhs[0].shape
    nn_bl = nn_bl if nn_bl is not None else (1, 1, 1, nx, ny, nz)
    rc = lib().vpmo_pmesh_bc(_pp(sol), _pp(rhs), np.asarray(xbound, dtype=np.float64),
                             np.asarray(dpm, dtype=np.float64), _ivec((nx, ny, nz)), _ivec(nn_bl), iynbc, itree,
                             levmax, nthreads, ibctyp)
    if rc != 0:
        raise RuntimeError(f"vpmo_pmesh failed: {rc}")
    return sol


def boundary_values(sol0, xbound, dpm, levmax, direct=False, nthreads=0, ibctyp=2):
    nz, ny, nx = sol0[0].shape
    bnd = [np.zeros_like(sol0[0]) for _ in range(3)]
    n = lib().vpmo_boundary_values_bc(_pp(sol0), _pp(bnd), np.asarray(xbound, dtype=np.float64),
                                      np.asarray(dpm, dtype=np.float64), _ivec((nx, ny, nz)), levmax,
                                      1 if direct else 0, nthreads, ibctyp)
    if n < 0:
        raise RuntimeError(f"vpmo_boundary_values failed: {n}")
    return bnd, n


def fsour_a4(xo, rg, iplane, dpm, area):
    """FSOUR_A4 (source/pmbound.f90:1540-1620) in the frame of target plane iplane."""
    return lib().vpmo_fsour_a4(np.asarray(xo, dtype=np.float64), np.asarray(rg, dtype=np.float64), int(iplane),
                               np.asarray(dpm, dtype=np.float64), float(area))


def step_fields(cfg, sizes, xp, qp, nthreads=0):
    """WhatToDo = 2 on one block. xp (nvr,3), qp (nvr,4). Returns (up, gp)."""
    xp = np.ascontiguousarray(xp, dtype=np.float64)
    qp = np.ascontiguousarray(qp, dtype=np.float64)
    n = xp.shape[0]
    up = np.zeros((n, 3))
    gp = np.zeros((n, 3))
    rc = lib().vpmo_step_fields(C.byref(cfg), C.byref(sizes), xp, qp, up, gp, n, nthreads)
    if rc != 0:
        raise RuntimeError(f"vpmo_step_fields failed: {rc}")
    return up, gp


def diffuse(cfg, sizes, xp, qp, ni, nthreads=0):
    """vpm(WhatToDo = 5) on one block: returns GP (nvr, 3) = vol * sum W (-NI Lap_h RHS)."""
    xp = np.ascontiguousarray(xp, dtype=np.float64)
    qp = np.ascontiguousarray(qp, dtype=np.float64)
    gp = np.zeros((xp.shape[0], 3))
    rc = lib().vpmo_diffuse(C.byref(cfg), C.byref(sizes), xp, qp, float(ni), gp, xp.shape[0], nthreads)
    if rc != 0:
        raise RuntimeError(f"vpmo_diffuse failed: {rc}")
    return gp


def whattodo4(cfg, sizes, xp, qp, up, nthreads=0):
    """vpm(WhatToDo = 4) after step_fields on the same mesh: returns (up + sum W vel, GP)."""
    xp = np.ascontiguousarray(xp, dtype=np.float64)
    qp = np.ascontiguousarray(qp, dtype=np.float64)
    up = np.array(up, dtype=np.float64, order="C", copy=True)
    gp = np.zeros((xp.shape[0], 3))
    rc = lib().vpmo_whattodo4(C.byref(cfg), C.byref(sizes), xp, qp, up, gp, xp.shape[0], nthreads)
    if rc != 0:
        raise RuntimeError(f"vpmo_whattodo4 failed: {rc}")
    return up, gp


def get_field(which):
    """Returns (3, NZ, NY, NX) array of the last step's field."""
    n = lib().vpmo_get_field(which, None, 0)
    out = np.empty(3 * n)
    lib().vpmo_get_field(which, out.ctypes.data, 3 * n)
    return out


def euler(xp, qp, up, gp, dt, uinf=(0.0, 0.0, 0.0)):
    lib().vpmo_euler(xp, qp, np.ascontiguousarray(up), np.ascontiguousarray(gp), xp.shape[0], dt,
                     np.asarray(uinf, dtype=np.float64))


def remesh(cfg, sizes, xp, qp, nthreads=0):
    xp = np.ascontiguousarray(xp, dtype=np.float64)
    qp = np.ascontiguousarray(qp, dtype=np.float64)
    cap = int(np.prod(list(sizes.nn)))
    xo = np.empty((cap, 3))
    qo = np.empty((cap, 4))
    n = lib().vpmo_remesh(C.byref(cfg), C.byref(sizes), xp, qp, xp.shape[0], xo, qo, cap, nthreads)
    if n < 0:
        raise RuntimeError(f"vpmo_remesh failed: {n}")
    return xo[:n].copy(), qo[:n].copy()


def remesh_masked(cfg, sizes, xp, qp, mask, mode, nthreads=0):
    """remesh with the |w| cut recorded into (mode 1) or replaced by (mode 2)
    the int32 node mask `mask` of NN1*NN2*NN3 entries."""
    xp = np.ascontiguousarray(xp, dtype=np.float64)
    qp = np.ascontiguousarray(qp, dtype=np.float64)
    cap = int(np.prod(list(sizes.nn)))
    assert mask.dtype == np.int32 and mask.size == cap and mask.flags.c_contiguous
    xo = np.empty((cap, 3))
    qo = np.empty((cap, 4))
    n = lib().vpmo_remesh_masked(C.byref(cfg), C.byref(sizes), xp, qp, xp.shape[0], xo, qo, cap, nthreads,
                                 mask.ctypes.data_as(C.POINTER(C.c_int)), int(mode))
    if n < 0:
        raise RuntimeError(f"vpmo_remesh_masked failed: {n}")
    return xo[:n].copy(), qo[:n].copy()
