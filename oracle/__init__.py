"""ORACLE — test infrastructure, not the product.

ctypes front end to the CPU restatement in ``amb_oracle.c`` (and, where it was
built, to the reference's own CPU scheme compiled into ``oracle/_ref``). Only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use
this module, always as the checker of the CUDA library, never in its place.

Field layout: numpy float64 arrays of shape (ny, nx), row-major, axis 0 = y.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from . import build as _build

TERM_NAMES = ("mu_p", "mu_a", "jp_y", "jp_x", "jl_y", "jl_x", "jc_y", "jc_x", "jr_y", "jr_x")
NOISE_MODES = {"none": 0, "philox": 1, "injected": 2}


@dataclass
class Params:
    """Stencil + model parameters (reference src/parameters.h:23-91)."""
    dt: float = 0.0
    dx: float = 1.0
    dy: float = 1.0
    a: float = 0.0
    b: float = 0.0
    c: float = 0.0
    kappa: float = 0.0
    lamb: float = 0.0
    zeta: float = 0.0
    T: float = 0.0


class _CParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ("dt", "dx", "dy", "a", "b", "c", "kappa", "lamb", "zeta", "T")]


def _cparams(p: Params) -> _CParams:
    return _CParams(p.dt, p.dx, p.dy, p.a, p.b, p.c, p.kappa, p.lamb, p.zeta, p.T)


_lib = None
_ref = {}
_DP = ctypes.POINTER(ctypes.c_double)


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    return a.ctypes.data_as(_DP)


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = ctypes.CDLL(path)
        L.orc_terms.argtypes = [ctypes.c_int, ctypes.c_int, _DP, ctypes.POINTER(_CParams), _DP, _DP, _DP, ctypes.c_int]
        L.orc_divergence.argtypes = [ctypes.c_int, ctypes.c_int, _DP, ctypes.POINTER(_CParams), _DP, _DP, ctypes.c_int]
        L.orc_run.argtypes = [ctypes.c_int, ctypes.c_int, _DP, ctypes.POINTER(_CParams), ctypes.c_int64, ctypes.c_int,
                              ctypes.c_int, ctypes.c_uint64, _DP, ctypes.c_int]
        L.orc_philox4x32_10.argtypes = [ctypes.POINTER(ctypes.c_uint32)] * 3
        L.orc_noise_bits.argtypes = [ctypes.c_uint64, ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_uint32)]
        L.orc_noise_normal.argtypes = [ctypes.c_uint64, ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_noise_normal.restype = ctypes.c_double
        L.orc_normals.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint64, ctypes.c_int64, _DP, _DP]
        L.orc_sum.argtypes = [_DP, ctypes.c_long]
        L.orc_sum.restype = ctypes.c_double
        _lib = L
    return _lib


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def terms(phi, p: Params, xi_y=None, xi_x=None, nthreads: int = 1) -> dict[str, np.ndarray]:
    """All per-term fields of the reference's forces/currents kernels at ``phi``."""
    phi = _f64(phi)
    ny, nx = phi.shape
    out = np.empty((len(TERM_NAMES), ny, nx))
    xy = None if xi_y is None else _f64(xi_y)
    xx = None if xi_x is None else _f64(xi_x)
    rc = lib().orc_terms(ny, nx, _ptr(phi), ctypes.byref(_cparams(p)), _ptr(xy), _ptr(xx), _ptr(out), nthreads)
    if rc:
        raise ValueError(f"orc_terms failed ({rc})")
    return dict(zip(TERM_NAMES, out))


def divergence(phi, p: Params, xi_y=None, xi_x=None, nthreads: int = 1) -> np.ndarray:
    """divJ of one step at ``phi`` (the update is phi -= dt * divJ)."""
    phi = _f64(phi)
    ny, nx = phi.shape
    out = np.empty((len(TERM_NAMES), ny, nx))
    xy = None if xi_y is None else _f64(xi_y)
    xx = None if xi_x is None else _f64(xi_x)
    lib().orc_terms(ny, nx, _ptr(phi), ctypes.byref(_cparams(p)), _ptr(xy), _ptr(xx), _ptr(out), nthreads)
    div = np.empty((ny, nx))
    work = np.empty((4, ny, nx))
    lib().orc_divergence(ny, nx, _ptr(out), ctypes.byref(_cparams(p)), _ptr(div), _ptr(work), nthreads)
    return div


def run(phi, p: Params, nsteps: int, noise: str = "none", seed: int = 0, step0: int = 0,
        injected=None, nthreads: int = 1) -> np.ndarray:
    """``nsteps`` explicit-Euler steps from ``phi``; returns the new field."""
    phi = _f64(phi).copy()
    ny, nx = phi.shape
    inj = None
    if noise == "injected":
        inj = _f64(injected)
        if inj.shape != (nsteps, 2, ny, nx):
            raise ValueError("injected noise must have shape (nsteps, 2, ny, nx)")
    rc = lib().orc_run(ny, nx, _ptr(phi), ctypes.byref(_cparams(p)), step0, nsteps, NOISE_MODES[noise],
                       seed, _ptr(inj), nthreads)
    if rc:
        raise ValueError(f"orc_run failed ({rc})")
    return phi


def philox4x32_10(ctr, key) -> np.ndarray:
    c = (ctypes.c_uint32 * 4)(*[int(v) & 0xFFFFFFFF for v in ctr])
    k = (ctypes.c_uint32 * 2)(*[int(v) & 0xFFFFFFFF for v in key])
    o = (ctypes.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return np.array(list(o), dtype=np.uint32)


def noise_bits(seed: int, step: int, row: int, col: int, comp: int) -> np.ndarray:
    o = (ctypes.c_uint32 * 4)()
    lib().orc_noise_bits(seed, step, row, col, comp, o)
    return np.array(list(o), dtype=np.uint32)


def normals(ny: int, nx: int, seed: int, step: int) -> tuple[np.ndarray, np.ndarray]:
    """Standard normals (xi_y, xi_x) of the (seed, step) noise field."""
    xy = np.empty((ny, nx))
    xx = np.empty((ny, nx))
    lib().orc_normals(ny, nx, seed, step, _ptr(xy), _ptr(xx))
    return xy, xx


def mass(phi) -> float:
    phi = _f64(phi)
    return lib().orc_sum(_ptr(phi), phi.size)


# ------------------------------------------------- the reference's own CPU scheme

def reference_lib(fast: bool = False):
    """ctypes handle on oracle/_ref (the compiled test/tjhung_ambplus.h), or None."""
    key = "fast" if fast else "exact"
    if key not in _ref:
        path = _build.TJHUNG_FAST_LIB if fast else _build.TJHUNG_LIB
        try:
            _build.build_reference()  # from the staged reference sources, where they exist
        except RuntimeError:
            pass
        L = None
        if os.path.exists(path):
            try:
                L = ctypes.CDLL(path)
            except OSError:  # built for another architecture
                L = None
        if L is not None:
            L.tjhung_ref_dphi.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_double] * 6 + [_DP] * 8
            L.tjhung_ref_run.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_double] * 6 + [_DP, ctypes.c_int]
            L.tjhung_ref_run_noisy.argtypes = ([ctypes.c_int, ctypes.c_int] + [ctypes.c_double] * 7
                                               + [_DP, ctypes.c_int, ctypes.c_long])
        _ref[key] = L
    return _ref[key]


def tjhung_dphi(phi, dt: float, h: float, A: float, K: float, lamb: float, zeta: float) -> dict[str, np.ndarray]:
    """One TjhungIntegrator::calculate_dphi (model a=-A, b=0, c=A) on a (ny, nx) field."""
    L = reference_lib()
    if L is None:
        raise RuntimeError("reference CPU scheme not built here")
    phi = _f64(phi)
    ny, nx = phi.shape
    names = ("dphi", "mueq", "muact", "jxeq", "jyeq", "jxact", "jyact")
    outs = {k: np.empty((ny, nx)) for k in names}
    rc = L.tjhung_ref_dphi(ny, nx, dt, h, A, K, lamb, zeta, _ptr(phi), *[_ptr(outs[k]) for k in names])
    if rc:
        raise ValueError("tjhung_ref_dphi rejected the sizes")
    return outs


def tjhung_run(phi, nsteps: int, dt: float, h: float, A: float, K: float, lamb: float, zeta: float,
               fast: bool = False) -> np.ndarray:
    L = reference_lib(fast)
    if L is None:
        raise RuntimeError("reference CPU scheme not built here")
    phi = _f64(phi).copy()
    ny, nx = phi.shape
    rc = L.tjhung_ref_run(ny, nx, dt, h, A, K, lamb, zeta, _ptr(phi), nsteps)
    if rc:
        raise ValueError("tjhung_ref_run rejected the arguments")
    return phi


def tjhung_run_noisy(phi, nsteps: int, dt: float, h: float, A: float, K: float, lamb: float, zeta: float,
                     D: float, seed: int = 1, fast: bool = True) -> np.ndarray:
    """TjhungIntegrator::run with its own noise (D = T; drand48 seeded with ``seed``). No test can
    pin this noise; it serves the timed CPU baseline, which must run the scheme as it ships."""
    L = reference_lib(fast)
    if L is None:
        raise RuntimeError("reference CPU scheme not built here")
    phi = _f64(phi).copy()
    ny, nx = phi.shape
    rc = L.tjhung_ref_run_noisy(ny, nx, dt, h, A, K, lamb, zeta, D, _ptr(phi), nsteps, seed)
    if rc:
        raise ValueError("tjhung_ref_run_noisy rejected the arguments")
    return phi


# ------------------------------------------------- the reference's own CUDA integrator

class ReferenceGpuIntegrator:
    """The reference's CUDA Integrator (src/integrator.cu) run from its compiled cubin
    (oracle/_ref/ref_integrator.cubin) by oracle/ref_gpu_driver.cc: FP64, three launches per
    step, curand XORWOW noise seeded with ``seed``. Baseline and parity infrastructure."""

    _lib = None

    @classmethod
    def available(cls) -> bool:
        return os.path.exists(_build.REF_GPU_CUBIN)

    @classmethod
    def _load(cls):
        if cls._lib is None:
            path = _build.build_ref_gpu_driver()
            L = ctypes.CDLL(path)
            L.refgpu_last_error.restype = ctypes.c_char_p
            L.refgpu_load.argtypes = [ctypes.c_char_p]
            L.refgpu_create.argtypes = [_DP, ctypes.c_int, ctypes.c_int, _DP, _DP, ctypes.c_ulonglong,
                                        ctypes.POINTER(ctypes.c_void_p)]
            L.refgpu_run.argtypes = [ctypes.c_void_p, ctypes.c_int]
            L.refgpu_get_field.argtypes = [ctypes.c_void_p, _DP]
            L.refgpu_time_steps.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]
            L.refgpu_destroy.argtypes = [ctypes.c_void_p]
            if L.refgpu_load(_build.REF_GPU_CUBIN.encode()):
                raise RuntimeError(L.refgpu_last_error().decode())
            cls._lib = L
        return cls._lib

    def __init__(self, field, p: Params, seed: int = 0):
        L = self._load()
        f = _f64(field)
        self.shape = f.shape
        st = np.array([p.dt, p.dx, p.dy])
        md = np.array([p.a, p.b, p.c, p.kappa, p.lamb, p.zeta, p.T])
        self._h = ctypes.c_void_p()
        if L.refgpu_create(_ptr(f), f.shape[0], f.shape[1], _ptr(st), _ptr(md), seed, ctypes.byref(self._h)):
            raise RuntimeError(L.refgpu_last_error().decode())

    def run(self, nsteps: int) -> None:
        rc = self._lib.refgpu_run(self._h, nsteps)
        if rc:
            raise RuntimeError(self._lib.refgpu_last_error().decode())

    def time_steps(self, nsteps: int) -> float:
        """Milliseconds (CUDA events) for nsteps of the run loop."""
        ms = ctypes.c_float()
        if self._lib.refgpu_time_steps(self._h, nsteps, ctypes.byref(ms)):
            raise RuntimeError(self._lib.refgpu_last_error().decode())
        return ms.value

    @property
    def field(self) -> np.ndarray:
        out = np.empty(self.shape)
        if self._lib.refgpu_get_field(self._h, _ptr(out)):
            raise RuntimeError(self._lib.refgpu_last_error().decode())
        return out

    def close(self):
        if self._h:
            self._lib.refgpu_destroy(self._h)
            self._h = ctypes.c_void_p()

    __del__ = close
