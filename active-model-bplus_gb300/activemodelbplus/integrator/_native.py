"""ctypes binding of ``libamb_gb300.so`` (C ABI declared in include/amb_gb300.h).

The library is built in-tree by ``active-model-bplus_gb300/build.py``. There is
no fallback: if the library cannot be built or loaded, importing the
integrator raises, so nothing silently runs on the CPU.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libamb_gb300.so")

AMB_OK = 0
AMB_ERR_INVALID = 1
AMB_ERR_CUDA = 2
AMB_ERR_NONFINITE = 3
AMB_ERR_NOMEM = 4
AMB_ERR_UNSUPPORTED = 5

AMB_F64, AMB_F32, AMB_F32C = 0, 1, 2
AMB_KERNEL_AUTO, AMB_KERNEL_TILE, AMB_KERNEL_SLIDING = 0, 1, 2
AMB_NTERMS = 10
AMB_EPI_GELU, AMB_EPI_F32, AMB_EPI_GELU_BWD = 0, 1, 2
CURRENTS = {"total": 0, "deterministic": 1, "passive": 2, "active": 3, "lambda": 4, "circulating": 5, "random": 6}
MUS = {"total": 0, "passive": 1, "active": 2}


class amb_stencil(ctypes.Structure):
    _fields_ = [("dt", ctypes.c_double), ("dx", ctypes.c_double), ("dy", ctypes.c_double)]


class amb_model(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("a", "b", "c", "kappa", "lamb", "zeta", "temperature")]


class amb_kernel_config(ctypes.Structure):
    _fields_ = [("kernel", ctypes.c_int), ("seg_rows", ctypes.c_int), ("pairs_per_cta", ctypes.c_int),
                ("flags", ctypes.c_int)]


AMB_FLAG_PERSISTENT = 1
AMB_FLAG_FUSED = 2
AMB_FLAG_TILE_ROWS_28 = 4


_VP = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_U64 = ctypes.c_uint64
_SP = ctypes.POINTER(amb_stencil)
_MP = ctypes.POINTER(amb_model)
_IP = ctypes.POINTER(ctypes.c_int)

# name -> (restype, argtypes)
SIGNATURES = {
    "amb_version": (ctypes.c_char_p, []),
    "amb_last_error": (ctypes.c_char_p, []),
    "amb_integrator_create": (_I, [_VP, _I, _I, _SP, _MP, _I, _U64, ctypes.POINTER(_VP)]),
    "amb_integrator_destroy": (None, [_VP]),
    "amb_integrator_run": (_I, [_VP, _I]),
    "amb_integrator_get_field": (_I, [_VP, _VP]),
    "amb_integrator_set_field": (_I, [_VP, _VP]),
    "amb_integrator_get_chemical_potential": (_I, [_VP, _I, _VP]),
    "amb_integrator_get_current": (_I, [_VP, _I, _VP, _VP]),
    "amb_integrator_get_timestep": (_I, [_VP, ctypes.POINTER(_I64)]),
    "amb_integrator_get_time": (_I, [_VP, ctypes.POINTER(ctypes.c_double)]),
    "amb_integrator_set_timestep": (_I, [_VP, _I64]),
    "amb_integrator_get_stencil": (_I, [_VP, _SP]),
    "amb_integrator_get_model": (_I, [_VP, _MP]),
    "amb_integrator_get_shape": (_I, [_VP, _IP, _IP, _IP]),
    "amb_step_f64": (_I, [_SP, _MP, _U64, _I, _I, _VP, _VP, _I64, _I, _VP, _VP, _IP]),
    "amb_step_f64_ex": (_I, [_SP, _MP, _U64, _I, _I, _VP, _VP, _I64, _I, _VP, ctypes.POINTER(amb_kernel_config),
                             _VP, _IP]),
    "amb_step_f32": (_I, [_SP, _MP, _U64, _I, _I, _VP, _VP, _VP, _I64, _I, _VP, _I, _VP, _IP]),
    "amb_step_f32_ex": (_I, [_SP, _MP, _U64, _I, _I, _VP, _VP, _VP, _I64, _I, _VP, ctypes.POINTER(amb_kernel_config),
                             _VP, _IP]),
    "amb_autotune_f32": (_I, [_SP, _MP, _I, _I, _I, _I, _VP, ctypes.POINTER(amb_kernel_config),
                              ctypes.POINTER(ctypes.c_double)]),
    "amb_terms_f64": (_I, [_SP, _MP, _U64, _I, _I, _VP, _I64, _VP, _VP, _VP]),
    "amb_terms_f32": (_I, [_SP, _MP, _U64, _I, _I, _VP, _I64, _VP, _VP, _VP]),
    "amb_mass_scratch_bytes": (ctypes.c_size_t, [_I64]),
    "amb_mass_f64": (_I, [_VP, _I64, _VP, _VP, ctypes.c_size_t, _VP]),
    "amb_mass_f32": (_I, [_VP, _I64, _VP, _VP, ctypes.c_size_t, _VP]),
    "amb_mass_f32_noalloc": (_I, [_VP, _I64, _VP, _VP]),
    "amb_ensemble_create": (_I, [_I, _IP, _IP, ctypes.POINTER(ctypes.POINTER(ctypes.c_double)), _SP, _MP,
                                 ctypes.POINTER(ctypes.c_uint64), _I, _I, ctypes.POINTER(_VP)]),
    "amb_ensemble_destroy": (None, [_VP]),
    "amb_ensemble_run": (_I, [_VP, _I]),
    "amb_ensemble_get_field": (_I, [_VP, _I, _VP]),
    "amb_ensemble_info": (_I, [_VP, ctypes.POINTER(_I64), _IP, _IP]),
    "amb_ensemble_form": (_I, [_VP, _I, _IP]),
    "amb_radial_spectrum": (_I, [_VP, _I, _I, ctypes.c_double, ctypes.c_double, _VP, _I, _VP, _VP, _VP]),
    "amb_label_components_f64": (_I, [_VP, _I, _I, ctypes.c_double, _VP, _VP, _VP]),
    "amb_label_components_f32": (_I, [_VP, _I, _I, ctypes.c_double, _VP, _VP, _VP]),
    "amb_check_finite_f64": (_I, [_VP, _I64, _VP, _VP]),
    "amb_check_finite_f32": (_I, [_VP, _I64, _VP, _VP]),
    "amb_ensemble_gather": (_I, [_VP, _VP]),
    "amb_ensemble_scatter": (_I, [_VP, _VP]),
    "amb_tc_selftest": (_I, [_VP, _VP, _VP, _I, _I, _I, _I, _VP, _VP]),
    "amb_conv5x5_forward": (_I, [_VP, _I, _I, _I, _I, _VP, _VP, _I, _I, _I, _VP, _VP, _VP, _VP, _VP, _VP]),
    "amb_conv5x5_wgrad_scratch_bytes": (ctypes.c_size_t, [_I, _I, _I, _I, _I]),
    "amb_conv5x5_wgrad": (_I, [_VP, _VP, _I, _I, _I, _I, _I, _VP, _VP, ctypes.c_size_t, _VP, _VP]),
    "amb_learned_input": (_I, [_VP, _VP, _I, _I, _I, _VP, _VP]),
    "amb_learned_spectral_combine": (_I, [_VP, _VP, _VP, _VP, _VP, _VP, ctypes.c_double, _I64, _VP, _VP, _VP]),
    "amb_learned_noise_spectral": (_I, [_I, _I, _U64, _VP, _VP, _I64, _I64, _VP]),
    "amb_learned_spectral_combine_noise": (_I, [_VP, _VP, _VP, _VP, _VP, ctypes.c_double, _I, _I, _I64, _I64, _U64,
                                                _VP, _VP, _VP, _VP]),
    "amb_learned_noise": (_I, [_I, _I, _U64, _VP, _VP, _VP]),
    "amb_learned_fft_create": (_I, [_I, _I, ctypes.POINTER(_VP)]),
    "amb_learned_fft_forward": (_I, [_VP, _VP, _VP, _VP]),
    "amb_learned_fft_inverse2": (_I, [_VP, _VP, _VP, _VP]),
    "amb_learned_fft_destroy": (None, [_VP]),
    "amb_learned_update": (_I, [_VP, _VP, _I, _I, ctypes.c_double, ctypes.c_double, ctypes.c_double, _VP,
                                ctypes.c_double, _VP, _VP, ctypes.c_double, _VP, _VP, _VP]),
    "amb_learned_update_input": (_I, [_VP, _VP, _I, _I, ctypes.c_double, ctypes.c_double, ctypes.c_double, _VP,
                                      ctypes.c_double, _VP, _VP, ctypes.c_double, _VP, _VP, _VP, _VP, _VP]),
}

_lib = None


def _build_if_needed() -> None:
    import importlib.util
    build_py = os.path.abspath(os.path.join(_HERE, "..", "..", "build.py"))
    spec = importlib.util.spec_from_file_location("_amb_gb300_build", build_py)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()


def lib() -> ctypes.CDLL:
    """The loaded CUDA library (built on first use if the toolkit is present)."""
    global _lib
    if _lib is None:
        try:
            _build_if_needed()
        except Exception as exc:  # no toolkit: only a prebuilt library can be used
            if not os.path.exists(LIB_PATH):
                raise ImportError(f"libamb_gb300.so is missing and could not be built: {exc}") from exc
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def last_error() -> str:
    return lib().amb_last_error().decode()


def stencil_struct(s) -> amb_stencil:
    return amb_stencil(float(s.dt), float(s.dx), float(s.dy))


def model_struct(m) -> amb_model:
    return amb_model(float(m.a), float(m.b), float(m.c), float(m.kappa), float(m.lamb), float(m.zeta), float(m.T))
