"""The C-ABI library loads and exports every function include/*.h declares
(no compute calls: no GPU needed)."""
import ctypes
import glob
import os
import re

from conftest import ROOT

from activemodelbplus.integrator import _native


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(amb_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("amb_integrator_create", "amb_integrator_run", "amb_integrator_get_field",
                     "amb_integrator_get_current", "amb_step_f64", "amb_step_f32", "amb_terms_f64",
                     "amb_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol():
    lib = _native.lib()
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_python_binding_covers_the_header():
    assert declared_functions() <= set(_native.SIGNATURES)


def test_cpu_only_calls():
    lib = _native.lib()
    assert lib.amb_version().decode().startswith("amb_gb300")
    assert lib.amb_mass_scratch_bytes(0) == 0
    assert lib.amb_mass_scratch_bytes(1 << 20) > 0
    # argument checking happens before any CUDA call
    s = _native.amb_stencil(1e-3, 1, 1)
    m = _native.amb_model(0, 0, 0, 0, 0, 0, 0)
    rc = lib.amb_step_f64(ctypes.byref(s), ctypes.byref(m), 0, 0, 16, None, None, 0, 1, None, None, None)
    assert rc == _native.AMB_ERR_INVALID
    assert "grid shape" in _native.last_error()
    h = ctypes.c_void_p()
    rc = lib.amb_integrator_create(None, 8, 8, ctypes.byref(s), ctypes.byref(m), 0, 0, ctypes.byref(h))
    assert rc == _native.AMB_ERR_INVALID and not h.value
