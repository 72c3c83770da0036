"""libgDMR without a GPU: it loads, exports every symbol include/*.h declares,
validates arguments the way the reference does, and links a reference-style
control program.  No compute calls."""
import ctypes
import os
import re
import shutil
import subprocess

import pytest

import gdmr

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
# The reference source tree (holding progDMR.c) is named by GDMR_REFERENCE_DIR; the link test
# skips when it is unset.
REFERENCE_DIR = os.environ.get("GDMR_REFERENCE_DIR", "")
REFERENCE_PROG = os.path.join(REFERENCE_DIR, "progDMR.c") if REFERENCE_DIR else ""


def declared_functions():
    names = set()
    for h in ("gDMR.h", "gDMRC.h", "gdmr_ext.h"):
        text = open(os.path.join(INCLUDE, h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(\w+)\s*\([^;{]*\)\s*;", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert {"initDMR", "freeDMR", "solverDMR", "impSVDMR", "expSVDMR", "initLS", "solveLS", "linOptLS",
            "solverDMR_z", "gdmr_solve_batch"} <= names
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol():
    assert declared_functions() == set(gdmr.SIGNATURES)


def test_soname_and_links():
    libdir = os.path.join(ROOT, "gdmr-solver_gb300", "lib")
    assert os.readlink(os.path.join(libdir, "libgDMR.so")) == "libgDMR.so.1"
    assert os.readlink(os.path.join(libdir, "libgDMR.so.1")) == "libgDMR.so.1.0.1"
    out = subprocess.run(["readelf", "-d", os.path.join(libdir, "libgDMR.so.1.0.1")], capture_output=True, text=True)
    if out.returncode == 0:
        assert "libgDMR.so.1" in out.stdout


def test_version_and_status(lib):
    assert lib.gdmrVersion().decode().startswith("1.0.1")
    assert isinstance(lib.gdmrLastStatus(), int)


@pytest.mark.parametrize("basis,deflat,ndev,needle", [
    (10, 9, 1, "too small"),             # gDMR.cu:856-860
    (10, 4, 2, "basisDim + 1"),          # gDMR.cu:844-848
    (11, 3, 2, "deflation space"),       # gDMR.cu:850-854
])
def test_init_validation_matches_reference(lib, basis, deflat, ndev, needle):
    devs = (ctypes.c_int * ndev)(*([0] * ndev))
    hook = ctypes.CFUNCTYPE(None)(lambda: None)
    lib.initDMR(32, 512, devs, ndev, 100, basis, deflat, ctypes.cast(hook, ctypes.c_void_p))
    assert lib.gdmrLastStatus() == 1
    assert needle in gdmr.last_error()


def test_solver_before_init_reports_not_initialised(lib):
    its = ctypes.c_int(-1)
    r = lib.solverDMR_z(0, None, None, None, 0, 1e-10, 10, ctypes.byref(its))
    assert r == 1.0
    assert lib.gdmrLastStatus() == 6


def test_process_settings_read_set_and_restore(lib):
    """The process-wide settings that take a count (multi-solve hand-over point, residual grid
    cap) read with -1, return the previous value when set, and clamp the cap."""
    tail = gdmr.multi_tail()
    assert tail == 48
    assert gdmr.multi_tail(3) == 48 and gdmr.multi_tail() == 3
    assert gdmr.multi_tail(tail) == 3 and gdmr.multi_tail() == tail
    cap = gdmr.overlap_residual()
    assert cap == 0
    assert gdmr.overlap_residual(20) == 0 and gdmr.overlap_residual() == 8
    assert gdmr.overlap_residual(cap) == 8 and gdmr.overlap_residual() == cap


@pytest.mark.skipif(not REFERENCE_PROG or not os.path.exists(REFERENCE_PROG) or shutil.which("gcc") is None,
                    reason="GDMR_REFERENCE_DIR unset or without progDMR.c, or no gcc")
def test_reference_control_program_links_unchanged(tmp_path):
    """progDMR.c, compiled from the reference tree as it is, against this library's
    gDMRC.h, links with -lgDMR (it is not run: it needs a GPU)."""
    libdir = os.path.join(ROOT, "gdmr-solver_gb300", "lib")
    exe = tmp_path / "progDMR.exe"
    cmd = ["gcc", "-std=c99", "-o", str(exe), REFERENCE_PROG, f"-I{INCLUDE}", f"-L{libdir}",
           f"-Wl,-rpath,{libdir}", "-lgDMR", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert exe.exists()
