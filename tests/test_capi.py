"""The C-ABI library loads and exports every entry point include/*.h declares
(no GPU needed: nothing here launches work), and argument validation fails
cleanly without a device."""
import ctypes
import glob
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"\b(?:int|const char \*|void)\s*\*?\s*(gev_[A-Za-z0-9_]+)\s*\(", txt):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def libpath():
    import sys
    sys.path.insert(0, os.path.join(ROOT, "gevolution-1.2_gb300"))
    import build
    return build.build()


def test_headers_declare_the_hot_path():
    names = declared()
    for must in ("gev_projection_T00", "gev_projection_T0i", "gev_projection_Tij", "gev_prepare_source_scalar",
                 "gev_prepare_source_tensor", "gev_fft_r2c", "gev_fft_c2r", "gev_solve_poisson", "gev_project_scalar",
                 "gev_evolve_vector", "gev_project_vector", "gev_project_tensor", "gev_update_q", "gev_update_pos",
                 "gev_sim_step"):
        assert must in names


def test_library_exports_every_declared_symbol(libpath):
    out = subprocess.run(["nm", "-D", "--defined-only", libpath], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = sorted(declared() - exported)
    assert not missing, missing


def test_loads_and_validates_without_device(libpath):
    L = ctypes.CDLL(libpath)
    L.gev_strerror.restype = ctypes.c_char_p
    assert L.gev_strerror(0) == b"ok"
    assert L.gev_strerror(-1) == b"invalid argument"
    h = ctypes.c_void_p()
    # bad sizes are rejected before any CUDA call: odd N, N with a prime factor 5, bad precision
    assert L.gev_ctx_create(0, 15, 0, ctypes.byref(h)) == -1
    assert L.gev_ctx_create(0, 20, 0, ctypes.byref(h)) == -1
    assert L.gev_ctx_create(0, 16, 7, ctypes.byref(h)) == -1
    assert L.gev_ctx_destroy(None) == 0
    assert L.gev_field_upload(None, None) == -1
