"""vpm_free_gb300 -- GB300 (sm_103a) particle-mesh time step of vpm_free.

Host-side mirror of the reference's Fortran interface for this path, over
the C-ABI of libvpmg.so (include/vpmg.h):

  * ``read_pm_inp(path)``          -- pm.inp, positional (source/vpm.f90:132-152)
  * ``VPM(cfg)``                   -- the vpm_lib module state as an object:
      ``.vpm(XP, QP, UP, GP, NVR, neqpm, WhatToDo, NTIME, NI, NVRM)``
                                      (source/vpm.f90:54-475, WhatToDo 0 and 2)
      ``.remesh_particles_3d(iflag, XP, QP)``  (source/vpm_remesh.f90:5-225)
      ``.pmesh(...)``, ``.project_particles_3D(...)`` (pmlib / projlib calls)
      plus a device-resident loop (``set_particles``/``step``) for
      test.f90-style time stepping without host copies.

Particle arrays use the reference's layout in C order: XP(3,NVR) is a
(NVR, 3) float64 array, QP(4,NVR) a (NVR, 4) array with QP(:,1:3) =
-omega*vol and QP(:,4) = vol.  By default everything computes in IEEE FP64
on the GPU, as the reference does; ``VPM(cfg, arith="ff48")`` (or
``set_arithmetic``) runs the heavy kernels in float-float instead (about
48 significant bits, FP32's exponent range).  There is no CPU fallback:
without the compiled library or a GPU every call raises.
"""
import ctypes as C
import os

import numpy as np

__all__ = ["VPMConfig", "VPM", "VPMError", "read_pm_inp", "read_particles_bin", "write_particles_bin", "load_library",
           "library_path", "FIELDS", "ARITH"]

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

FIELDS = {"rhs": 0, "sol": 1, "vel": 2, "def": 3, "bl_sol1": 4, "coarse_rhs": 5, "coarse_sol": 6, "bl_final": 7}
ARITH = {"fp64": 0, "ff48": 1}  # VPMG_ARITH_FP64 (default), VPMG_ARITH_FF48

EXPORTS = [
    "vpmg_read_pm_inp", "vpmg_create", "vpmg_destroy", "vpmg_last_error", "vpmg_status_string", "vpmg_vpm",
    "vpmg_remesh_particles_3d", "vpmg_pmesh", "vpmg_project_particles_3d", "vpmg_define_sizes", "vpmg_get_sizes",
    "vpmg_set_particles", "vpmg_get_particles", "vpmg_get_particle_velocity", "vpmg_step", "vpmg_remesh_device",
    "vpmg_num_particles", "vpmg_get_field", "vpmg_kernel_launches", "vpmg_phase_times", "vpmg_tree_stats",
    "vpmg_set_profiling", "vpmg_set_operator_budget", "vpmg_run", "vpmg_bench_kernel", "vpmg_fp64_peak", "vpmg_batch_run",
    "vpmg_read_particles_bin", "vpmg_write_particles_bin", "vpmg_write_solution", "vpmg_write_hist", "vpmg_set_output",
    "vpmg_dst_tiles", "vpmg_apply_poisson", "vpmg_adjoint_poisson", "vpmg_vjp_fields", "vpmg_vjp_remesh", "vpmg_adjoint_loss",
    "vpmg_adjoint_run", "vpmg_batch_create", "vpmg_batch_info", "vpmg_batch_step", "vpmg_batch_destroy",
    "vpmg_batch_set_schedule", "vpmg_batch_get_schedule", "vpmg_host_euler", "vpmg_set_arithmetic",
    "vpmg_get_arithmetic", "vpmg_dirichlet_static", "vpmg_projection_fun", "vpmg_farfield_stats",
]


class VPMError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"vpmg status {status}: {msg}")
        self.status = status


class VPMConfig(C.Structure):
    """vpmg_config: pm.inp plus an explicit mesh box."""
    _fields_ = [
        ("dpm", C.c_double * 3), ("interf_iproj", C.c_int), ("ibctyp", C.c_int), ("idvpm", C.c_int),
        ("epsvol", C.c_double), ("ncoarse", C.c_int), ("nbi", C.c_int), ("nbj", C.c_int), ("nbk", C.c_int),
        ("nremesh", C.c_int), ("ncell_rem", C.c_int), ("iyntree", C.c_int), ("ilevmax", C.c_int),
        ("ompthreads", C.c_int), ("idefine", C.c_int), ("iynslice", C.c_int), ("use_box", C.c_int),
        ("box", C.c_double * 6), ("ipmwrite", C.c_int), ("ipmwstart", C.c_int * 10), ("ipmwsteps", C.c_int * 10),
    ]

    @classmethod
    def make(cls, dpm=(0.05, 0.05, 0.05), interf_iproj=4, ibctyp=2, idvpm=1, epsvol=0.0, ncoarse=8, nb=(1, 1, 1),
             nremesh=1, ncell_rem=1, iyntree=1, ilevmax=3, ompthreads=1, idefine=1, iynslice=0, box=None):
        c = cls()
        c.dpm[:] = list(dpm)
        c.interf_iproj, c.ibctyp, c.idvpm, c.epsvol, c.ncoarse = interf_iproj, ibctyp, idvpm, epsvol, ncoarse
        c.nbi, c.nbj, c.nbk = nb
        c.nremesh, c.ncell_rem, c.iyntree, c.ilevmax = nremesh, ncell_rem, iyntree, ilevmax
        c.ompthreads, c.idefine, c.iynslice = ompthreads, idefine, iynslice
        if box is not None:
            c.use_box = 1
            c.box[:] = list(box)
        return c


class VPMSizes(C.Structure):
    _fields_ = [
        ("xbound", C.c_double * 6), ("dpm", C.c_double * 3), ("nn", C.c_int * 3), ("nn_bl", C.c_int * 6),
        ("xbound_bl", C.c_double * 6), ("nnbl", C.c_int * 3), ("nnbl_bl", C.c_int * 6),
        ("xbound_coarse", C.c_double * 6), ("dpm_coarse", C.c_double * 3), ("nn_coarse", C.c_int * 3),
        ("nn_bl_coarse", C.c_int * 6), ("ilevmax", C.c_int), ("dvpm", C.c_double), ("defined", C.c_int),
    ]


_dp = C.POINTER(C.c_double)
_PP = _dp * 3


def library_path():
    return os.path.join(_HERE, "libvpmg.so")


def load_library():
    """Loads libvpmg.so (built in tree by vpm_free_gb300/build.py)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not os.path.exists(path):
        raise VPMError(-2, f"{path} is missing: run vpm_free_gb300/build.py (there is no CPU fallback)")
    L = C.CDLL(path)
    L.vpmg_read_pm_inp.argtypes = [C.c_char_p, C.POINTER(VPMConfig)]
    L.vpmg_create.argtypes = [C.POINTER(VPMConfig), C.c_int, C.POINTER(C.c_void_p)]
    L.vpmg_destroy.argtypes = [C.c_void_p]
    L.vpmg_last_error.argtypes = [C.c_void_p]
    L.vpmg_last_error.restype = C.c_char_p
    L.vpmg_status_string.argtypes = [C.c_int]
    L.vpmg_status_string.restype = C.c_char_p
    L.vpmg_vpm.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, C.POINTER(C.c_int), C.c_int, C.c_int, C.c_int, C.c_double,
                           C.c_int]
    L.vpmg_remesh_particles_3d.argtypes = [C.c_void_p, C.c_int, _dp, _dp, C.POINTER(C.c_int), C.c_int]
    L.vpmg_pmesh.argtypes = [C.c_void_p, _PP, _PP, _dp, _dp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int, C.c_int,
                             C.c_int]
    L.vpmg_project_particles_3d.argtypes = [C.c_void_p, _dp, _dp, C.c_int, _PP]
    L.vpmg_define_sizes.argtypes = [C.c_void_p, _dp, C.c_int, C.c_int]
    L.vpmg_get_sizes.argtypes = [C.c_void_p, C.POINTER(VPMSizes)]
    L.vpmg_set_particles.argtypes = [C.c_void_p, _dp, _dp, C.c_int, C.c_int]
    L.vpmg_get_particles.argtypes = [C.c_void_p, _dp, _dp, C.POINTER(C.c_int), C.c_int]
    L.vpmg_get_particle_velocity.argtypes = [C.c_void_p, _dp, _dp, C.c_int]
    L.vpmg_step.argtypes = [C.c_void_p, C.c_double, _dp, C.c_int]
    L.vpmg_remesh_device.argtypes = [C.c_void_p]
    L.vpmg_num_particles.argtypes = [C.c_void_p, C.POINTER(C.c_int)]
    L.vpmg_get_field.argtypes = [C.c_void_p, C.c_int, _dp, C.c_size_t, C.POINTER(C.c_size_t)]
    L.vpmg_kernel_launches.argtypes = [C.c_void_p]
    L.vpmg_kernel_launches.restype = C.c_longlong
    L.vpmg_phase_times.argtypes = [C.c_void_p, _dp]
    L.vpmg_tree_stats.argtypes = [C.c_void_p, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), C.POINTER(C.c_int)]
    L.vpmg_farfield_stats.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_longlong), _dp]
    L.vpmg_set_profiling.argtypes = [C.c_void_p, C.c_int]
    L.vpmg_set_operator_budget.argtypes = [C.c_void_p, C.c_longlong]
    L.vpmg_run.argtypes = [C.c_void_p, C.c_int, C.c_double, _dp, C.c_int, _dp, C.POINTER(C.c_longlong)]
    L.vpmg_bench_kernel.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, _dp, _dp]
    L.vpmg_fp64_peak.argtypes = [C.c_void_p, _dp]
    L.vpmg_batch_run.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_double, C.c_int, _dp,
                                 C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
    L.vpmg_batch_create.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.POINTER(C.c_void_p)]
    L.vpmg_batch_info.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_longlong)]
    L.vpmg_batch_step.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_int, _dp, C.POINTER(C.c_longlong),
                                  C.POINTER(C.c_longlong)]
    L.vpmg_batch_destroy.argtypes = [C.c_void_p]
    L.vpmg_host_euler.argtypes = [_dp, _dp, _dp, _dp, C.c_int, C.c_double, _dp]
    L.vpmg_batch_set_schedule.argtypes = [C.c_void_p, C.c_int]
    L.vpmg_batch_get_schedule.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_float)]
    L.vpmg_read_particles_bin.argtypes = [C.c_char_p, C.POINTER(C.c_int), _dp, _dp, _dp, C.c_int]
    L.vpmg_write_particles_bin.argtypes = [C.c_char_p, C.c_int, C.c_double, _dp, _dp]
    L.vpmg_write_solution.argtypes = [C.c_void_p, C.c_char_p, C.c_int]
    L.vpmg_write_hist.argtypes = [C.c_void_p, C.c_char_p, C.c_int]
    L.vpmg_set_output.argtypes = [C.c_void_p, C.c_char_p, C.c_int]
    L.vpmg_dst_tiles.argtypes = [C.c_void_p, C.POINTER(C.c_int)]
    L.vpmg_apply_poisson.argtypes = [C.c_void_p, _dp, _dp]
    L.vpmg_adjoint_poisson.argtypes = [C.c_void_p, _dp, _dp]
    L.vpmg_vjp_fields.argtypes = [C.c_void_p, _dp, _dp, C.c_int, _dp, _dp, _dp, _dp]
    L.vpmg_vjp_remesh.argtypes = [C.c_void_p, _dp, _dp, C.c_int, _dp, C.c_int, _dp, _dp]
    L.vpmg_adjoint_loss.argtypes = [C.c_void_p, C.c_int, C.c_double, _dp, C.c_int, C.c_double, C.c_int, _dp]
    L.vpmg_adjoint_run.argtypes = [C.c_void_p, C.c_int, C.c_double, _dp, C.c_int, C.c_double, _dp, _dp, _dp, _dp, _dp]
    L.vpmg_projection_fun.argtypes = [C.c_int, C.c_double]
    L.vpmg_projection_fun.restype = C.c_double
    L.vpmg_set_arithmetic.argtypes = [C.c_void_p, C.c_int]
    L.vpmg_get_arithmetic.argtypes = [C.c_void_p, C.POINTER(C.c_int)]
    _LIB = L
    return L


def _p(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None and a.shape != shape:
        raise ValueError(f"expected shape {shape}, got {a.shape}")
    return a


def read_pm_inp(path):
    """pm.inp -> VPMConfig (positional list-directed reads of source/vpm.f90:132-152)."""
    L = load_library()
    cfg = VPMConfig()
    rc = L.vpmg_read_pm_inp(os.fsencode(path), C.byref(cfg))
    if rc != 0:
        raise VPMError(rc, f"cannot parse {path}")
    return cfg


def read_particles_bin(path):
    """particles.bin (source/test.f90:24-37) -> (XP (NVR,3), QP (NVR,4), Vref),
    QP[:, :3] = -w * Vref and QP[:, 3] = Vref.  Needs no GPU."""
    L = load_library()
    n, vref = C.c_int(0), C.c_double(0.0)
    rc = L.vpmg_read_particles_bin(os.fsencode(path), C.byref(n), C.byref(vref), None, None, 0)
    if rc != 0:
        raise VPMError(rc, f"cannot read {path}")
    xp, qp = np.zeros((max(n.value, 1), 3)), np.zeros((max(n.value, 1), 4))
    rc = L.vpmg_read_particles_bin(os.fsencode(path), C.byref(n), C.byref(vref), _p(xp), _p(qp), xp.shape[0])
    if rc != 0:
        raise VPMError(rc, f"cannot read {path}")
    return xp[:n.value], qp[:n.value], vref.value


def write_particles_bin(path, XP, QP, vref):
    """Writes particles.bin so that read_particles_bin returns XP, QP[:, :3] (QP[:, 3] = vref)."""
    L = load_library()
    n = XP.shape[0]
    rc = L.vpmg_write_particles_bin(os.fsencode(path), n, float(vref), _p(_f64(XP, (n, 3))), _p(_f64(QP, (n, 4))))
    if rc != 0:
        raise VPMError(rc, f"cannot write {path}")


class VPM:
    """The vpm_lib module state (source/vpm.f90:1-32) on one GPU."""

    def __init__(self, cfg, device=-1, arith="fp64"):
        self._L = load_library()
        self.cfg = cfg
        h = C.c_void_p()
        rc = self._L.vpmg_create(C.byref(cfg), device, C.byref(h))
        if rc != 0:
            raise VPMError(rc, self._L.vpmg_status_string(rc).decode())
        self._h = h
        if arith != "fp64":
            self.set_arithmetic(arith)

    def set_arithmetic(self, arith):
        """'fp64' (default, the reference's arithmetic) or 'ff48' (float-float
        heavy kernels).  On a sized handle the plans and the recorded
        boundary operator are rebuilt."""
        self._chk(self._L.vpmg_set_arithmetic(self._h, ARITH[arith] if isinstance(arith, str) else int(arith)))

    @property
    def arithmetic(self):
        a = C.c_int(-1)
        self._chk(self._L.vpmg_get_arithmetic(self._h, C.byref(a)))
        return {v: k for k, v in ARITH.items()}[a.value]

    def close(self):
        if getattr(self, "_h", None):
            self._L.vpmg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _chk(self, rc):
        if rc != 0:
            msg = self._L.vpmg_last_error(self._h)
            raise VPMError(rc, (msg or b"").decode() or self._L.vpmg_status_string(rc).decode())

    # ---- the reference's calls ------------------------------------------
    def vpm(self, XP, QP, UP, GP, NVR, neqpm=3, WhatToDo=2, NTIME=0, NI=0.0, NVRM=None):
        """vpm(XP,QP,UP,GP,NVR,neqpm,WhatToDo,...,NTIME,NI,NVRM).  WhatToDo 2
        and 4 add the interpolated velocity to UP (the caller zeroes it, as
        test.f90:90-91 does) and overwrite GP.  Returns NVR."""
        nvrm = XP.shape[0] if NVRM is None else NVRM
        for a, w in ((XP, 3), (QP, 4), (UP, 3), (GP, 3)):
            if a is not None and (a.dtype != np.float64 or not a.flags.c_contiguous or a.shape[1] != w):
                raise ValueError("particle arrays must be C-contiguous float64 (NVRM, 3|4)")
        n = C.c_int(int(NVR))
        self._chk(self._L.vpmg_vpm(self._h, _p(XP), _p(QP), _p(UP), _p(GP), C.byref(n), neqpm, WhatToDo, NTIME,
                                   float(NI), int(nvrm)))
        return n.value

    def define_sizes(self, XP, NTIME=0):
        XP = _f64(XP)
        self._chk(self._L.vpmg_define_sizes(self._h, _p(XP), XP.shape[0], NTIME))
        return self.sizes()

    def sizes(self):
        s = VPMSizes()
        self._chk(self._L.vpmg_get_sizes(self._h, C.byref(s)))
        return s

    def remesh_particles_3d(self, iflag, XP, QP, capacity=None):
        """remesh_particles_3d(iflag) on (XP, QP); returns new (XP, QP) arrays.
        The in/out arrays of the C call (capacity = mesh nodes, the most a
        remesh can emit) are kept by the handle and reused."""
        nn = list(self.sizes().nn)
        cap = int(capacity or max(int(np.prod(nn)), XP.shape[0]))
        if getattr(self, "_rbuf", None) is None or self._rbuf[0].shape[0] < cap:
            self._rbuf = (np.empty((cap, 3)), np.empty((cap, 4)))
        xb, qb = self._rbuf
        xb[:XP.shape[0]] = XP
        qb[:QP.shape[0]] = QP
        n = C.c_int(XP.shape[0])
        self._chk(self._L.vpmg_remesh_particles_3d(self._h, iflag, _p(xb), _p(qb), C.byref(n), cap))
        return xb[:n.value].copy(), qb[:n.value].copy()

    @staticmethod
    def host_euler(XP, QP, UP, GP, n, dt, uinf=None):
        """Forward Euler of the reference's time loop (test.f90:104-117) on
        host arrays in one compiled pass: XP += (UP + uinf) dt, QP[:, :3] -= GP dt."""
        for a, c in ((XP, 3), (QP, 4), (UP, 3), (GP, 3)):
            if a.dtype != np.float64 or not a.flags.c_contiguous or a.shape[1] != c or a.shape[0] < n:
                raise ValueError("host_euler wants C-contiguous float64 (>= n, 3/4) arrays")
        u = (C.c_double * 3)(*uinf) if uinf is not None else None
        rc = load_library().vpmg_host_euler(_p(XP), _p(QP), _p(UP), _p(GP), int(n), float(dt), u)
        if rc != 0:
            raise ValueError("vpmg_host_euler: bad arguments")

    def remesh_in_place(self, XP, QP, n, iflag=1):
        """remesh_particles_3d(iflag) on caller-owned arrays of NVRM rows, as a
        Fortran host passes XPR/QPR: reads n particles, writes the new set in
        place and returns its count (VPMGError if it exceeds NVRM)."""
        if XP.dtype != np.float64 or QP.dtype != np.float64 or not (XP.flags.c_contiguous and QP.flags.c_contiguous):
            raise ValueError("XP, QP must be C-contiguous float64 (NVRM, 3) / (NVRM, 4)")
        m = C.c_int(int(n))
        self._chk(self._L.vpmg_remesh_particles_3d(self._h, iflag, _p(XP), _p(QP), C.byref(m), XP.shape[0]))
        return m.value

    def pmesh(self, SOL, RHS, Xbound, Dpm, iynbc, itree=1, levmax=3, NN_bl=None):
        """pmesh (source/pmlib.f90:69-192), 3 components, the handle's ibctyp.
        SOL, RHS: lists of 3 arrays shaped (NZ, NY, NX); SOL updated in place."""
        nz, ny, nx = RHS[0].shape
        sol = [_f64(s) for s in SOL]
        rhs = [_f64(r) for r in RHS]
        nn = (C.c_int * 3)(nx, ny, nz)
        nnbl = (C.c_int * 6)(*(NN_bl if NN_bl is not None else (1, 1, 1, nx, ny, nz)))
        self._chk(self._L.vpmg_pmesh(self._h, _PP(*[_p(s) for s in sol]), _PP(*[_p(r) for r in rhs]),
                                     _p(_f64(Xbound)), _p(_f64(Dpm)), nn, nnbl, iynbc, itree, levmax))
        for dst, src in zip(SOL, sol):
            if dst is not src:
                dst[...] = src
        return SOL

    def project_particles_3D(self, XP, QP):
        """project_particles_3D + project_vol3d(IDVPM=1) on the current mesh;
        returns RHS(1:3) as 3 arrays (NZ, NY, NX)."""
        nx, ny, nz = list(self.sizes().nn)
        XP, QP = _f64(XP), _f64(QP)
        out = [np.empty((nz, ny, nx)) for _ in range(3)]
        self._chk(self._L.vpmg_project_particles_3d(self._h, _p(XP), _p(QP), XP.shape[0], _PP(*[_p(o) for o in out])))
        return out

    # ---- device-resident loop -------------------------------------------
    def set_particles(self, XP, QP):
        XP, QP = _f64(XP), _f64(QP)
        self._chk(self._L.vpmg_set_particles(self._h, _p(XP), _p(QP), XP.shape[0], XP.shape[0]))

    def get_particles(self):
        n = self.num_particles()
        xp, qp = np.empty((max(n, 1), 3)), np.empty((max(n, 1), 4))
        m = C.c_int(0)
        self._chk(self._L.vpmg_get_particles(self._h, _p(xp), _p(qp), C.byref(m), max(n, 1)))
        return xp[:m.value], qp[:m.value]

    def get_particle_velocity(self, n=None):
        n = self.num_particles() if n is None else n
        up, gp = np.empty((max(n, 1), 3)), np.empty((max(n, 1), 3))
        self._chk(self._L.vpmg_get_particle_velocity(self._h, _p(up), _p(gp), n))
        return up[:n], gp[:n]

    def num_particles(self):
        n = C.c_int(0)
        self._chk(self._L.vpmg_num_particles(self._h, C.byref(n)))
        return n.value

    def step(self, dt, uinf=(0.0, 0.0, 0.0), remesh=True):
        u = np.asarray(uinf, dtype=np.float64)
        self._chk(self._L.vpmg_step(self._h, float(dt), _p(u), 1 if remesh else 0))

    def run(self, nsteps, dt, uinf=(0.0, 0.0, 0.0), remesh=True):
        """nsteps device-resident steps timed with CUDA events on the handle's
        stream.  Returns (device ms, sum of particle counts)."""
        u = np.asarray(uinf, dtype=np.float64)
        ms = C.c_double(0.0)
        ps = C.c_longlong(0)
        self._chk(self._L.vpmg_run(self._h, int(nsteps), float(dt), _p(u), 1 if remesh else 0, C.byref(ms),
                                   C.byref(ps)))
        return ms.value, ps.value

    @staticmethod
    def batch_run(handles, nsteps, dt, remesh=True):
        """Advances independent problems together (one graph per problem,
        replayed concurrently).  Returns (device ms, solves, particle-steps)."""
        L = load_library()
        arr = (C.c_void_p * len(handles))(*[h._h for h in handles])
        ms, sv, ps = C.c_double(0), C.c_longlong(0), C.c_longlong(0)
        rc = L.vpmg_batch_run(arr, len(handles), int(nsteps), float(dt), 1 if remesh else 0, C.byref(ms), C.byref(sv),
                              C.byref(ps))
        if rc != 0:
            handles[0]._chk(rc)
        return ms.value, sv.value, ps.value

    @staticmethod
    def batch(handles):
        """Batch object over `handles` (problems sharing a boundary operator
        are grouped); see Batch."""
        return Batch(handles)

    def bench_kernel(self, which, reps=5):
        """(ms per replay, algorithmic flops, algorithmic bytes) of one kernel."""
        ms, fl, by = C.c_double(0), C.c_double(0), C.c_double(0)
        self._chk(self._L.vpmg_bench_kernel(self._h, int(which), int(reps), C.byref(ms), C.byref(fl), C.byref(by)))
        return ms.value, fl.value, by.value

    def fp64_peak(self):
        t = C.c_double(0)
        self._chk(self._L.vpmg_fp64_peak(self._h, C.byref(t)))
        return t.value

    def remesh(self):
        self._chk(self._L.vpmg_remesh_device(self._h))

    def field(self, name):
        """Resident field (3, NZ, NY, NX) of the last step."""
        which = FIELDS[name]
        cnt = C.c_size_t(0)
        self._chk(self._L.vpmg_get_field(self._h, which, None, 0, C.byref(cnt)))
        out = np.empty(3 * cnt.value)
        self._chk(self._L.vpmg_get_field(self._h, which, _p(out), out.size, C.byref(cnt)))
        s = self.sizes()
        if which in (0, 1, 2, 3):
            dims = list(s.nn)
        elif which in (4, 7):
            dims = list(s.nnbl)
        else:
            dims = list(s.nn_coarse)
        return out.reshape(3, dims[2], dims[1], dims[0])

    # ---- instrumentation --------------------------------------------------
    def kernel_launches(self):
        return int(self._L.vpmg_kernel_launches(self._h))

    def phase_times(self):
        ms = (C.c_double * 9)()
        self._chk(self._L.vpmg_phase_times(self._h, ms))
        return list(ms)

    def tree_stats(self):
        a, b, c = C.c_longlong(0), C.c_longlong(0), C.c_int(0)
        self._chk(self._L.vpmg_tree_stats(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return {"interactions": a.value, "bytes": b.value, "precomputed": bool(c.value)}

    def farfield_stats(self):
        """{'on': the coarsest tree level goes by FFT convolutions, 'corrections':
        opened coarsest cells subtracted as rows, 'flops': FP64 flops of one
        apply of the FFT part}."""
        a, b, c = C.c_int(0), C.c_longlong(0), C.c_double(0.0)
        self._chk(self._L.vpmg_farfield_stats(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return {"on": bool(a.value), "corrections": b.value, "flops": c.value}

    def write_solution(self, ntime, directory=None):
        """NNNNNsolution.bin of the last field step (writesol, source/vpm.f90:662-709)."""
        d = os.fsencode(directory) if directory else None
        self._chk(self._L.vpmg_write_solution(self._h, d, int(ntime)))

    def write_hist(self, ntime, directory=None):
        """Appends the nine velocity lines to NNhist.bin (writeline, source/vpm.f90:789-833)."""
        d = os.fsencode(directory) if directory else None
        self._chk(self._L.vpmg_write_hist(self._h, d, int(ntime)))

    def set_output(self, directory=None, solution=True, hist=True):
        """The writers vpm(WhatToDo = 2) calls after the velocity, as the reference does."""
        d = os.fsencode(directory) if directory else None
        self._chk(self._L.vpmg_set_output(self._h, d, (1 if solution else 0) | (2 if hist else 0)))

    def dst_tiles(self):
        """Autotuned DST tile shapes (line pairs per CTA) of the block x/y, inner-box x/y and coarse x/y plans."""
        t = (C.c_int * 6)()
        self._chk(self._L.vpmg_dst_tiles(self._h, t))
        keys = ["block_x", "block_y", "inner_x", "inner_y", "coarse_x", "coarse_y"]
        return dict(zip(keys, list(t)))

    def set_profiling(self, level):
        self._chk(self._L.vpmg_set_profiling(self._h, int(level)))

    def set_operator_budget(self, nbytes):
        self._chk(self._L.vpmg_set_operator_budget(self._h, int(nbytes)))

    # ---- reverse mode -------------------------------------------------------
    def _mesh_shape(self):
        s = self.sizes()
        return (3, s.nn[2], s.nn[1], s.nn[0])

    def apply_poisson(self, r):
        """psi = L r: the vector-potential solve of one step on a (3, NZ, NY, NX) RHS."""
        r = _f64(r, self._mesh_shape())
        psi = np.empty_like(r)
        self._chk(self._L.vpmg_apply_poisson(self._h, _p(r), _p(psi)))
        return psi

    def adjoint_poisson(self, psibar):
        """rbar = L^T psibar (exact transpose of apply_poisson)."""
        psibar = _f64(psibar, self._mesh_shape())
        rbar = np.empty_like(psibar)
        self._chk(self._L.vpmg_adjoint_poisson(self._h, _p(psibar), _p(rbar)))
        return rbar

    def vjp_fields(self, XP, QP, UPbar, GPbar):
        """(xbar, qbar) = (d(UP, GP) / d(XP, QP[:, :3]))^T (UPbar, GPbar) of vpm(WhatToDo = 2)."""
        n = XP.shape[0]
        XP, QP = _f64(XP, (n, 3)), _f64(QP, (n, 4))
        UPbar, GPbar = _f64(UPbar, (n, 3)), _f64(GPbar, (n, 3))
        xb, qb = np.zeros((max(n, 1), 3)), np.zeros((max(n, 1), 3))
        self._chk(self._L.vpmg_vjp_fields(self._h, _p(XP), _p(QP), n, _p(UPbar), _p(GPbar), _p(xb), _p(qb)))
        return xb[:n], qb[:n]

    def vjp_remesh(self, XP, QP, Qbar_new):
        """(xbar, qbar) of remesh_particles_3d(1) for the adjoint Qbar_new (nnew, 3) of the emitted strengths."""
        n = XP.shape[0]
        XP, QP = _f64(XP, (n, 3)), _f64(QP, (n, 4))
        qn = _f64(Qbar_new)
        xb, qb = np.zeros((max(n, 1), 3)), np.zeros((max(n, 1), 3))
        self._chk(self._L.vpmg_vjp_remesh(self._h, _p(XP), _p(QP), n, _p(qn), qn.shape[0], _p(xb), _p(qb)))
        return xb[:n], qb[:n]

    @staticmethod
    def _probes(probes):
        if probes is None or len(probes) == 0:
            return np.zeros((1, 3)), 0
        pr = _f64(probes)
        if pr.ndim != 2 or pr.shape[1] != 3:
            raise ValueError("probes must be (nprobe, 3)")
        return pr, pr.shape[0]

    def adjoint_loss(self, nsteps, dt, probes=None, ke_weight=0.0, mask_mode=0):
        """Loss of nsteps steps from the current particles (which are kept):
        sum |u(probe)|^2 + ke_weight * 0.5 * DV * sum |u|^2 on the final field.
        mask_mode 0: the reference's remesh cut; 1: record its masks; 2: the
        masks of the last adjoint_run (the map its gradient differentiates)."""
        pr, n = self._probes(probes)
        loss = C.c_double(0.0)
        self._chk(self._L.vpmg_adjoint_loss(self._h, int(nsteps), float(dt), _p(pr), n, float(ke_weight),
                                            int(mask_mode), C.byref(loss)))
        return loss.value

    def adjoint_run(self, nsteps, dt, probes=None, ke_weight=0.0):
        """(loss, dloss/dXP (NVR, 3), dloss/dQP[:, :3] (NVR, 3), forward ms, backward ms)."""
        pr, n = self._probes(probes)
        nvr = self.num_particles()
        xbar, qbar = np.zeros((max(nvr, 1), 3)), np.zeros((max(nvr, 1), 3))
        loss, tf, tb = C.c_double(0.0), C.c_double(0.0), C.c_double(0.0)
        self._chk(self._L.vpmg_adjoint_run(self._h, int(nsteps), float(dt), _p(pr), n, float(ke_weight),
                                           C.byref(loss), _p(xbar), _p(qbar), C.byref(tf), C.byref(tb)))
        return loss.value, xbar[:nvr], qbar[:nvr], tf.value, tb.value


class Batch:
    """Independent problems advanced together (vpmg_batch_create): problems
    whose fine-block boundary operators agree up to the mesh spacing share
    one operator apply per step; every group and every other problem is one
    captured graph, replayed concurrently.  The handles must stay open."""

    def __init__(self, handles, release_shared=False):
        """release_shared: free the followers' own recorded operators (their
        standalone applies then walk the tree)."""
        self._L = load_library()
        self._hs = list(handles)
        arr = (C.c_void_p * len(self._hs))(*[h._h for h in self._hs])
        self._b = C.c_void_p()
        rc = self._L.vpmg_batch_create(arr, len(self._hs), 1 if release_shared else 0, C.byref(self._b))
        if rc != 0:
            self._hs[0]._chk(rc)

    def info(self):
        """(graphs replayed per step, problems in shared-operator groups)"""
        return self.details()[:2]

    def details(self):
        """(graphs per step, problems sharing an operator, corrected rows)"""
        u, s, r = C.c_int(0), C.c_int(0), C.c_longlong(0)
        self._L.vpmg_batch_info(self._b, C.byref(u), C.byref(s), C.byref(r))
        return u.value, s.value, r.value

    def run(self, nsteps, dt, remesh=True):
        """Returns (device ms, solves, particle-steps)."""
        ms, sv, ps = C.c_double(0), C.c_longlong(0), C.c_longlong(0)
        rc = self._L.vpmg_batch_step(self._b, int(nsteps), float(dt), 1 if remesh else 0, C.byref(ms), C.byref(sv),
                                     C.byref(ps))
        if rc != 0:
            self._hs[0]._chk(rc)
        return ms.value, sv.value, ps.value

    def set_schedule(self, mode):
        """0 concurrent, 1 in sequence, -1 tuned on the next run of >= 2 steps."""
        rc = self._L.vpmg_batch_set_schedule(self._b, int(mode))
        if rc != 0:
            raise ValueError("schedule must be -1, 0 or 1")

    def schedule(self):
        """(mode, [ms of the tuning step run concurrently, in sequence])"""
        m, t = C.c_int(0), (C.c_float * 2)()
        self._L.vpmg_batch_get_schedule(self._b, C.byref(m), t)
        return m.value, [t[0], t[1]]

    def close(self):
        if self._b:
            self._L.vpmg_batch_destroy(self._b)
            self._b = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
