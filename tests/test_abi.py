"""C-ABI checks that need no GPU: the library loads, exports every entry
point declared in include/vpmg.h, parses pm.inp like the reference and
fails with status codes (never aborts) where a GPU is required."""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            text = open(os.path.join(inc, f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(vpmg_[a-z0-9_]+)\s*\(", text))
    return names


def test_library_exports_every_declared_symbol(gpulib):
    path = gpulib.library_path()
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (vpmg_[a-z0-9_]+)", out))
    declared = _declared()
    assert len(declared) >= 25
    assert declared <= exported, declared - exported
    L = gpulib.load_library()
    for n in declared:
        assert hasattr(L, n)


def test_read_pm_inp_reference_format(gpulib):
    cfg = gpulib.read_pm_inp(os.path.join(ROOT, "tests", "golden", "pm.inp"))
    assert list(cfg.dpm) == [4.0, 4.0, 4.0]
    assert (cfg.interf_iproj, cfg.ibctyp, cfg.idvpm, cfg.ncoarse) == (4, 2, 1, 8)
    assert (cfg.nbi, cfg.nbj, cfg.nbk, cfg.nremesh, cfg.ncell_rem) == (6, 1, 1, 1, 1)
    assert (cfg.iyntree, cfg.ilevmax, cfg.idefine, cfg.iynslice) == (1, 3, 1, 0)


def test_read_pm_inp_rejects_bad_input(gpulib, tmp_path):
    p = tmp_path / "pm.inp"
    p.write_text("1.0 1.0\n")
    with pytest.raises(gpulib.VPMError):
        gpulib.read_pm_inp(str(p))
    lines = open(os.path.join(ROOT, "tests", "golden", "pm.inp")).read().splitlines()
    lines[12] = " 11   ! more than 10 write windows stops the reference (vpm.f90:146)"
    p.write_text("\n".join(lines) + "\n")
    with pytest.raises(gpulib.VPMError):
        gpulib.read_pm_inp(str(p))


def test_status_strings_and_bad_configs(gpulib):
    L = gpulib.load_library()
    for st in range(0, -9, -1):
        assert L.vpmg_status_string(st)
    cfg = gpulib.VPMConfig.make(dpm=(0.1, 0.1, 0.1))
    for field, val, code in (("interf_iproj", 9, -1), ("ibctyp", 1, -6), ("ibctyp", 4, -6), ("idvpm", 0, -6), ("ncell_rem", 2, -6)):
        c = gpulib.VPMConfig.make(dpm=(0.1, 0.1, 0.1))
        setattr(c, field, val)
        h = C.c_void_p()
        assert L.vpmg_create(C.byref(c), -1, C.byref(h)) == code
    assert L.vpmg_destroy(None) == -1
    assert L.vpmg_step(None, 0.1, None, 1) == -1


def test_no_gpu_means_error_not_abort(gpulib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(gpulib.VPMError):
        gpulib.VPM(gpulib.VPMConfig.make(dpm=(0.1, 0.1, 0.1), box=(0, 0, 0, 0.8, 0.8, 0.8)))


def test_host_euler_is_the_reference_update(gpulib):
    """vpmg_host_euler (host only) against the test.f90:104-117 update
    written out in numpy: XP += (UP + UINF) dt, QP[:, :3] -= GP dt, rows
    past n untouched."""
    import numpy as np
    V = gpulib
    rng = np.random.default_rng(5)
    n, rows, dt, uinf = 1000, 1200, 0.005, (0.3, -0.1, 0.2)
    XP, QP = rng.normal(size=(rows, 3)), rng.normal(size=(rows, 4))
    UP, GP = rng.normal(size=(rows, 3)), rng.normal(size=(rows, 3))
    x0, q0 = XP.copy(), QP.copy()
    V.VPM.host_euler(XP, QP, UP, GP, n, dt, uinf)
    ex = x0.copy()
    ex[:n] = x0[:n] + (UP[:n] + np.array(uinf)) * dt
    eq = q0.copy()
    eq[:n, :3] = q0[:n, :3] - GP[:n] * dt
    assert np.array_equal(XP, ex) and np.array_equal(QP, eq)
    with pytest.raises(ValueError):
        V.VPM.host_euler(XP, QP, UP, GP, rows + 1, dt)


def test_batch_entry_points_reject_bad_arguments(gpulib):
    """The batch object's C-ABI checks its arguments before any device work."""
    L = gpulib.load_library()
    out = C.c_void_p()
    assert L.vpmg_batch_create(None, 1, 0, C.byref(out)) == -1
    arr = (C.c_void_p * 1)(None)
    assert L.vpmg_batch_create(arr, 1, 0, C.byref(out)) == -1
    assert L.vpmg_batch_create(arr, 0, 0, C.byref(out)) == -1
    u, s, r = C.c_int(0), C.c_int(0), C.c_longlong(0)
    assert L.vpmg_batch_info(None, C.byref(u), C.byref(s), C.byref(r)) == -1
    ms, sv, ps = C.c_double(0), C.c_longlong(0), C.c_longlong(0)
    assert L.vpmg_batch_step(None, 1, 0.01, 1, C.byref(ms), C.byref(sv), C.byref(ps)) == -1
    assert L.vpmg_batch_set_schedule(None, 0) == -1
    assert L.vpmg_batch_get_schedule(None, None, None) == -1
    assert L.vpmg_batch_destroy(None) == -1
    assert L.vpmg_host_euler(None, None, None, None, 5, 0.1, None) == -1
    assert L.vpmg_host_euler(None, None, None, None, 0, 0.1, None) == 0


def test_projection_fun_matches_oracle(gpulib, oracle):
    """vpmg_projection_fun (projlib's projection_fun, pmproject.f90:391-431)
    equals the oracle's restatement for every kernel type, both signs of x."""
    L = gpulib.load_library()
    O = oracle.lib()
    xs = [i / 64.0 for i in range(-160, 161)] + [0.5, 1.0, 1.5, 2.0, 1e-9, 2.0000001]
    for itype in (2, 3, 4, 5, 6):
        for x in xs:
            assert L.vpmg_projection_fun(itype, x) == O.vpmo_projection_fun(itype, x), (itype, x)
    assert L.vpmg_projection_fun(7, 0.1) == 0.0


def test_fortran_shim_declares_what_test_f90_uses():
    """The Fortran binding declares, in modules that vpm_lib re-exports (as
    the reference's vpm_lib re-exports vpm_vars and vpm_size, vpm.f90:42-44),
    the names source/test.f90 takes from them: mrem (test.f90:47), st and et
    (:54, :57), interf_iproj (:202), neqpm (:234), Dpm (:438); and a projlib
    module with projection_fun (:187).  No Fortran compiler exists here, so
    this reads the source."""
    src = open(os.path.join(ROOT, "vpm_free_gb300", "fortran", "vpm_gb300.f90")).read().lower()

    def module(name):
        m = re.search(r"^module %s\b(.*?)^end module %s" % (name, name), src, flags=re.S | re.M)
        assert m, name
        return m.group(1)

    lib = module("vpm_lib")
    for used in ("vpm_vars", "vpm_size", "openmpth"):
        assert re.search(r"^\s*use %s\b" % used, lib, flags=re.M), used
    decl = module("vpm_vars") + module("vpm_size")
    for name in ("mrem", "st", "et", "interf_iproj", "neqpm", "dpm", "nn_bl", "xbound"):
        assert re.search(r"::[^\n]*\b%s\b" % name, decl), name
    assert "function projection_fun" in module("projlib")
    assert "velvrx_pm" in module("pmgrid")
