"""GB300-native drop-in for the reference's ``activemodelbplus.integrator``.

Same public names and behaviour as the reference package
(tranqui/active-model-bplus, ``activemodelbplus/integrator/__init__.py`` over the
pybind11 module ``src/integrator.cc``): ``Model``, ``Stencil``, ``Integrator``
(``run``, ``run_for_time``, ``field``, the current getters, ``time``,
``timestep``), ``CudaException``, ``steps_from_time``, ``step_iterator`` and
``plot_field``.

Behind the API: device buffers are torch CUDA tensors, and every step is one
launch of a hand-written sm_103a kernel in ``libamb_gb300.so`` (C ABI,
include/amb_gb300.h) on the current torch stream. There is no CPU path.

Additions with no reference counterpart (all keyword-only or new names):
``precision`` ("f64" default, "f32", "f32c"), ``seed`` (Philox noise key; the
reference seeds non-deterministically), ``kernel``, the chemical-potential
getters the reference leaves unbound, ``mass()``, ``field_tensor``,
``checkpoint()`` / ``Integrator.from_checkpoint()``, ``sample_trajectory()``
(see ``activemodelbplus.trajectory`` for the ``.npz`` trajectory format),
``Ensemble``.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

from . import _native as N

__all__ = ["Model", "Stencil", "Integrator", "Ensemble", "CudaException", "steps_from_time", "step_iterator",
           "plot_field"]


class CudaException(RuntimeError):
    """Raised on CUDA errors and on a non-finite field after ``run``
    (the reference's ``kernel::CudaError``, src/integrator.h:10-14, src/integrator.cc:33)."""


def _check(rc: int) -> None:
    if rc == N.AMB_OK:
        return
    msg = N.last_error()
    if rc == N.AMB_ERR_INVALID:
        raise ValueError(msg)
    raise CudaException(msg)


# ------------------------------------------------------------------ parameters

class Model:
    """Active Model B+ parameters (src/parameters.h:54-77, bound at src/integrator.cc:35-72).

    ``Model()``, ``Model(a, b, c, kappa, lamb, zeta, T)`` or ``Model(model)`` (copy).
    ``as_dict()`` uses the key ``"temperature"`` for ``T`` as the reference does.
    """
    _names = ("a", "b", "c", "kappa", "lamb", "zeta", "T")
    __slots__ = _names

    def __init__(self, *args, **kwargs):
        if len(args) == 1 and not kwargs and isinstance(args[0], Model):
            vals = args[0].as_tuple()
        elif not args and set(kwargs) == {"model"}:
            vals = Model(kwargs["model"]).as_tuple()
        else:
            if len(args) > len(self._names):
                raise TypeError("Model takes at most 7 parameters")
            given = dict(zip(self._names, args))
            for k, v in kwargs.items():
                if k not in self._names or k in given:
                    raise TypeError(f"unexpected or repeated argument {k!r}")
                given[k] = v
            vals = tuple(float(given.get(k, 0.0)) for k in self._names)
        for k, v in zip(self._names, vals):
            object.__setattr__(self, k, float(v))

    def __setattr__(self, k, v):
        if k not in self._names:
            raise AttributeError(k)
        object.__setattr__(self, k, float(v))

    def as_tuple(self):
        return tuple(getattr(self, k) for k in self._names)

    def as_dict(self):
        d = {k: getattr(self, k) for k in ("a", "b", "c", "kappa", "lamb", "zeta")}
        d["temperature"] = self.T
        return d

    def __eq__(self, other):
        return isinstance(other, Model) and self.as_tuple() == other.as_tuple()

    __hash__ = None

    def __str__(self):
        return str(self.as_dict())

    def __repr__(self):
        return "<Model " + str(self.as_dict()) + ">"


class Stencil:
    """Discretisation parameters (src/parameters.h:23-41, bound at src/integrator.cc:74-103).

    ``Stencil()``, ``Stencil(dt, dx, dy)`` or ``Stencil(stencil)`` (copy).
    """
    _names = ("dt", "dx", "dy")
    __slots__ = _names

    def __init__(self, *args, **kwargs):
        if len(args) == 1 and not kwargs and isinstance(args[0], Stencil):
            vals = args[0].as_tuple()
        elif not args and set(kwargs) == {"stencil"}:
            vals = Stencil(kwargs["stencil"]).as_tuple()
        else:
            if len(args) > 3:
                raise TypeError("Stencil takes at most 3 parameters")
            given = dict(zip(self._names, args))
            for k, v in kwargs.items():
                if k not in self._names or k in given:
                    raise TypeError(f"unexpected or repeated argument {k!r}")
                given[k] = v
            vals = tuple(float(given.get(k, 0.0)) for k in self._names)
        for k, v in zip(self._names, vals):
            object.__setattr__(self, k, float(v))

    def __setattr__(self, k, v):
        if k not in self._names:
            raise AttributeError(k)
        object.__setattr__(self, k, float(v))

    def as_tuple(self):
        return tuple(getattr(self, k) for k in self._names)

    def as_dict(self):
        return {k: getattr(self, k) for k in self._names}

    def __eq__(self, other):
        return isinstance(other, Stencil) and self.as_tuple() == other.as_tuple()

    __hash__ = None

    def __str__(self):
        return str(self.as_dict())

    def __repr__(self):
        return "<Stencil " + str(self.as_dict()) + ">"


# ------------------------------------------------------------------ integrator

_PRECISIONS = {"f64": N.AMB_F64, "f32": N.AMB_F32, "f32c": N.AMB_F32C}
_KERNELS = {"auto": N.AMB_KERNEL_AUTO, "tile": N.AMB_KERNEL_TILE, "sliding": N.AMB_KERNEL_SLIDING}


def _torch():
    import torch
    return torch


def _random_seed() -> int:
    return int.from_bytes(os.urandom(8), "little")


class Integrator:
    """Explicit-Euler Active Model B+ integrator on one GPU
    (the reference's ``Integrator``, src/integrator.h:24-81, src/integrator.cc:105-123).

    Args:
        field: initial field, array-like of shape (ny, nx) (axis 0 = y).
        stencil: :class:`Stencil`.
        model: :class:`Model`.
        precision: "f64" (default; the reference's arithmetic), "f32" or "f32c"
            (float field with a bf16 Kahan residual: compensated update).
        seed: 64-bit key of the Philox noise; ``None`` draws one from the OS,
            like the reference's non-deterministic seed.
        device: CUDA device (default: current).
        kernel: "auto", "tile" or "sliding" (FP32 kernel choice; FP64 always runs the tile kernel).
        autotune: with kernel="auto" and FP32 storage, time the candidate kernels and
            launch shapes for this grid once per process (``amb_autotune_f32``) and use
            the fastest; otherwise a shape heuristic decides. The FP32 kernels give
            bitwise equal fields (the same arithmetic at every site), so the choice
            changes the time, never the result.
        launch: explicit launch shape: for kernel="sliding" (FP32 storage) {"seg_rows": h,
            "pairs_per_cta": p, "fused": bool (one warp per strip runs every stage; p then counts
            warps)}; for kernel="tile" {"pairs_per_cta": g (256-thread groups per CTA),
            "persistent": bool (all steps of a run() in one launch), "tile_rows": 32 or 28
            (output tile height)}; e.g. a configuration the autotuner reported.
    """

    def __init__(self, field, stencil, model, *, precision: str = "f64", seed: int | None = None,
                 device=None, kernel: str = "auto", autotune: bool = True, launch: dict | None = None):
        torch = _torch()
        if not torch.cuda.is_available():
            raise CudaException("no CUDA device is available")
        lib = N.lib()  # raises if the CUDA library is missing
        if precision not in _PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(_PRECISIONS)}")
        if kernel not in _KERNELS:
            raise ValueError(f"kernel must be one of {sorted(_KERNELS)}")
        host = np.asarray(field, dtype=np.float64)
        if host.ndim != 2:
            raise TypeError("field must be a 2D array (ny, nx)")
        self._stencil = Stencil(stencil)
        self._model = Model(model)
        self._precision = precision
        self._kernel = kernel
        self._seed = _random_seed() if seed is None else int(seed) & 0xFFFFFFFFFFFFFFFF
        self._device = torch.device("cuda", torch.cuda.current_device() if device is None else
                                    torch.device(device).index or 0)
        self._ny, self._nx = host.shape
        if self._ny < 1 or self._nx < 1:
            raise ValueError("field must have at least one site")
        dtype = torch.float64 if precision == "f64" else torch.float32
        self._buf = [torch.empty((self._ny, self._nx), dtype=dtype, device=self._device) for _ in range(2)]
        self._cur = 0
        self._residual = (torch.zeros((self._ny, self._nx), dtype=torch.int16, device=self._device)
                          if precision == "f32c" else None)
        self._flag = torch.zeros(1, dtype=torch.int32, device=self._device)
        self._timestep = 0
        self._terms_step = None
        self._terms_dev = None
        self._terms_host = None
        self._events = None  # optional (start, end) CUDA events recorded around the step launches
        self._s = N.stencil_struct(self._stencil)
        self._m = N.model_struct(self._model)
        self.set_field(host)
        self._launch_cfg = None
        if launch is not None:
            if kernel not in ("sliding", "tile") or (precision == "f64" and kernel != "tile"):
                raise ValueError('launch= applies to kernel="sliding" (FP32 storage) or kernel="tile"')
            if int(launch.get("tile_rows", 32)) not in (28, 32):
                raise ValueError("tile_rows must be 32 or 28")
            flags = ((N.AMB_FLAG_PERSISTENT if launch.get("persistent", False) else 0)
                     | (N.AMB_FLAG_FUSED if launch.get("fused", False) else 0)
                     | (N.AMB_FLAG_TILE_ROWS_28 if int(launch.get("tile_rows", 32)) == 28 else 0))
            self._launch_cfg = N.amb_kernel_config(_KERNELS[kernel], int(launch.get("seg_rows", 0)),
                                                   int(launch.get("pairs_per_cta", 0)), flags)
        self._tuned = None
        if autotune and kernel == "auto" and precision != "f64":
            cfg, us = N.amb_kernel_config(), ctypes.c_double()
            _check(lib.amb_autotune_f32(ctypes.byref(self._s), ctypes.byref(self._m), self._ny, self._nx,
                                        int(precision == "f32c"), 8, self._stream(), ctypes.byref(cfg),
                                        ctypes.byref(us)))
            names = {N.AMB_KERNEL_TILE: "tile", N.AMB_KERNEL_SLIDING: "sliding"}
            self._tuned = {"kernel": names.get(cfg.kernel, "auto"), "seg_rows": cfg.seg_rows,
                           "pairs_per_cta": cfg.pairs_per_cta,
                           "persistent": bool(cfg.flags & N.AMB_FLAG_PERSISTENT),
                           "fused": bool(cfg.flags & N.AMB_FLAG_FUSED),
                           "tile_rows": 28 if cfg.flags & N.AMB_FLAG_TILE_ROWS_28 else 32, "us_per_step": us.value}
        del lib

    # -------------------------------------------------------------- plumbing
    def _stream(self) -> int:
        return _torch().cuda.current_stream(self._device).cuda_stream

    @property
    def kernel_config(self):
        """The autotuned FP32 kernel configuration (dict) or None."""
        return None if self._tuned is None else dict(self._tuned)

    @property
    def field_tensor(self):
        """The field as a device tensor (no copy; valid until the next ``run``)."""
        return self._buf[self._cur]

    def set_field(self, field) -> None:
        """Replace the field (no reference counterpart; clears the residual)."""
        torch = _torch()
        host = np.asarray(field, dtype=np.float64)
        if host.shape != (self._ny, self._nx):
            raise ValueError(f"field shape {host.shape} != {(self._ny, self._nx)}")
        self._buf[self._cur].copy_(torch.from_numpy(np.ascontiguousarray(host)))
        if self._residual is not None:
            self._residual.zero_()
        self._terms_step = None

    # ------------------------------------------------------------ reference API
    @property
    def stencil(self) -> Stencil:
        return Stencil(self._stencil)

    @property
    def model(self) -> Model:
        return Model(self._model)

    @property
    def timestep(self) -> int:
        return self._timestep

    @property
    def time(self) -> float:
        return self._timestep * self._stencil.dt

    @property
    def field(self) -> np.ndarray:
        """A fresh float64 host copy of the field (src/integrator.cu:378-383)."""
        return self._buf[self._cur].to(dtype=_torch().float64).cpu().numpy()

    def run(self, nsteps: int) -> None:
        """Advance ``nsteps`` explicit-Euler steps (src/integrator.cu:497-538).

        Blocks until done and raises :class:`CudaException` if the field is no
        longer finite. As in the reference, ``timestep`` advances by ``nsteps``
        even when ``nsteps <= 0``.
        """
        self._launch(int(nsteps))
        self._check_finite()

    def _launch(self, nsteps: int) -> None:
        """Enqueue ``nsteps`` steps on the current stream and advance ``timestep``
        (no host synchronisation)."""
        lib = N.lib()
        stream = self._stream()
        if nsteps > 0:
            in_spare = ctypes.c_int(0)
            cur, other = self._buf[self._cur], self._buf[1 - self._cur]
            if self._events is not None:
                self._events[0].record()
            if self._precision == "f64":
                rc = lib.amb_step_f64_ex(ctypes.byref(self._s), ctypes.byref(self._m), self._seed, self._ny,
                                         self._nx, cur.data_ptr(), other.data_ptr(), self._timestep, nsteps, None,
                                         ctypes.byref(self._launch_cfg) if self._launch_cfg is not None else None,
                                         stream, ctypes.byref(in_spare))
            else:
                res = self._residual.data_ptr() if self._residual is not None else None
                if self._launch_cfg is not None:
                    rc = lib.amb_step_f32_ex(ctypes.byref(self._s), ctypes.byref(self._m), self._seed, self._ny,
                                             self._nx, cur.data_ptr(), other.data_ptr(), res, self._timestep, nsteps,
                                             None, ctypes.byref(self._launch_cfg), stream, ctypes.byref(in_spare))
                else:
                    rc = lib.amb_step_f32(ctypes.byref(self._s), ctypes.byref(self._m), self._seed, self._ny,
                                          self._nx, cur.data_ptr(), other.data_ptr(), res, self._timestep, nsteps,
                                          None, _KERNELS[self._kernel], stream, ctypes.byref(in_spare))
            if self._events is not None:
                self._events[1].record()
            _check(rc)
            if in_spare.value:
                self._cur = 1 - self._cur
        self._timestep += nsteps

    def _enqueue_finite_check(self) -> None:
        """OR a non-finite flag for the current field into ``self._flag`` (stream-ordered)."""
        lib = N.lib()
        f = self._buf[self._cur]
        fn = lib.amb_check_finite_f64 if self._precision == "f64" else lib.amb_check_finite_f32
        _check(fn(f.data_ptr(), f.numel(), self._flag.data_ptr(), self._stream()))

    def _raise_if_flagged(self) -> None:
        """Read the accumulated flag (one host synchronisation) and clear it."""
        bad = int(self._flag.item())
        self._flag.zero_()
        if bad:
            raise CudaException("an unknown numerical error occurred during simulation")

    def _check_finite(self) -> None:
        self._enqueue_finite_check()
        self._raise_if_flagged()

    # ------------------------------------------------------------- getters
    def _terms(self) -> np.ndarray:
        """The ten FP64 term planes at the current timestep, cached per timestep
        like the reference's lazy current recompute (src/integrator.cu:477-495)."""
        if self._terms_step != self._timestep:
            torch = _torch()
            if self._terms_dev is None:
                self._terms_dev = torch.empty((N.AMB_NTERMS, self._ny, self._nx), dtype=torch.float64,
                                              device=self._device)
            lib = N.lib()
            fn = lib.amb_terms_f64 if self._precision == "f64" else lib.amb_terms_f32
            _check(fn(ctypes.byref(self._s), ctypes.byref(self._m), self._seed, self._ny, self._nx,
                      self._buf[self._cur].data_ptr(), self._timestep, None, self._terms_dev.data_ptr(),
                      self._stream()))
            self._terms_host = self._terms_dev.cpu().numpy()
            self._terms_step = self._timestep
        return self._terms_host

    def _current(self, which: str):
        t = self._terms()
        out = []
        for c in range(2):
            jp, jl, jc, jr = t[2 + c], t[4 + c], t[6 + c], t[8 + c]
            # sums in the reference's order (src/integrator.cu:406-465)
            if which == "passive":
                v = jp.copy()
            elif which == "lambda":
                v = jl.copy()
            elif which == "circulating":
                v = jc.copy()
            elif which == "random":
                v = jr.copy()
            else:
                active = jc + jl
                if which == "active":
                    v = active
                else:
                    det = active + jp
                    v = det if which == "deterministic" else det + jr
            out.append(v)
        return out

    @property
    def current(self):
        """Total current [J_y, J_x] (src/integrator.cu:406-412)."""
        return self._current("total")

    @property
    def deterministic_current(self):
        return self._current("deterministic")

    @property
    def passive_current(self):
        return self._current("passive")

    @property
    def active_current(self):
        return self._current("active")

    @property
    def lambda_current(self):
        return self._current("lambda")

    @property
    def circulating_current(self):
        return self._current("circulating")

    @property
    def random_current(self):
        return self._current("random")

    @property
    def chemical_potential(self) -> np.ndarray:
        """mu_p + mu_a (src/integrator.cu:385-388; not bound in the reference's module)."""
        t = self._terms()
        return t[0] + t[1]

    @property
    def passive_chemical_potential(self) -> np.ndarray:
        return self._terms()[0].copy()

    @property
    def active_chemical_potential(self) -> np.ndarray:
        return self._terms()[1].copy()

    # ---------------------------------------------------------- additions
    @property
    def precision(self) -> str:
        return self._precision

    @property
    def seed(self) -> int:
        return self._seed

    @property
    def shape(self) -> tuple[int, int]:
        return (self._ny, self._nx)

    def mass(self) -> float:
        """Sum of the field, FP64 with compensation, on the device."""
        torch = _torch()
        lib = N.lib()
        f = self._buf[self._cur]
        nbytes = lib.amb_mass_scratch_bytes(f.numel())
        scratch = torch.empty(max(1, (nbytes + 7) // 8), dtype=torch.float64, device=self._device)
        out = torch.empty(1, dtype=torch.float64, device=self._device)
        fn = lib.amb_mass_f64 if self._precision == "f64" else lib.amb_mass_f32
        _check(fn(f.data_ptr(), f.numel(), out.data_ptr(), scratch.data_ptr(), nbytes, self._stream()))
        return float(out.item())

    def checkpoint(self) -> dict:
        """Everything needed to resume exactly: field (native dtype), residual, timestep, seed."""
        d = {
            "field": self._buf[self._cur].cpu().numpy().copy(),
            "timestep": self._timestep,
            "seed": self._seed,
            "precision": self._precision,
            "stencil": self._stencil.as_tuple(),
            "model": self._model.as_tuple(),
        }
        if self._residual is not None:
            d["residual"] = self._residual.cpu().numpy().copy()
        return d

    @classmethod
    def from_checkpoint(cls, ckpt: dict, **kwargs) -> "Integrator":
        torch = _torch()
        sim = cls(np.asarray(ckpt["field"], dtype=np.float64), Stencil(*ckpt["stencil"]), Model(*ckpt["model"]),
                  precision=ckpt["precision"], seed=int(ckpt["seed"]), **kwargs)
        sim._buf[sim._cur].copy_(torch.from_numpy(np.ascontiguousarray(ckpt["field"])))
        if sim._residual is not None and "residual" in ckpt:
            sim._residual.copy_(torch.from_numpy(np.ascontiguousarray(ckpt["residual"])))
        sim._timestep = int(ckpt["timestep"])
        return sim

    def save_checkpoint(self, path: str) -> None:
        np.savez(path, **{k: np.asarray(v) for k, v in self.checkpoint().items()})

    @classmethod
    def load_checkpoint(cls, path: str, **kwargs) -> "Integrator":
        z = np.load(path, allow_pickle=False)
        d = {k: z[k] for k in z.files}
        d["precision"] = str(d["precision"])
        d["stencil"] = tuple(d["stencil"].tolist())
        d["model"] = tuple(d["model"].tolist())
        return cls.from_checkpoint(d, **kwargs)

    # ---------------------------------------------------- trajectories
    def sample_trajectory(self, t_samples, *, to: str = "host"):
        """Run forward and record the field at each of ``t_samples`` (no reference
        counterpart; it does what the analysis notebook does with ``run_for_time``
        interrupts, examples/structureFactor.ipynb cell 1, without host round trips).

        Args:
            t_samples: non-decreasing times measured from the current time, each a
                multiple of dt (0 records the current field).
            to: "host" (float64 arrays, the ``.npz`` layout) or "device" (a device
                tensor (n, ny, nx) of the storage dtype, e.g. for on-device S(k)).

        The host waits once, at the end. Each sample is a device-to-device snapshot
        taken on the compute stream; for ``to="host"`` the snapshot goes to pinned
        memory on a copy stream that overlaps the next chunk of steps (two snapshot
        buffers in rotation). The non-finite flag accumulates on the device and is
        read once: :class:`CudaException` is raised at the end if any sample was
        non-finite.

        Returns:
            :class:`activemodelbplus.trajectory.Trajectory`.
        """
        from ..trajectory import Trajectory

        torch = _torch()
        if to not in ("host", "device"):
            raise ValueError('to must be "host" or "device"')
        ts = np.atleast_1d(np.asarray(t_samples, dtype=np.float64))
        steps = np.atleast_1d(steps_from_time(self._stencil.dt, ts)).astype(np.int64)
        if steps.size == 0:
            raise ValueError("no sample times given")
        if np.any(steps < 0) or np.any(np.diff(steps) < 0):
            raise ValueError("sample times must be non-negative and non-decreasing")
        n = int(steps.size)
        shape = (n, self._ny, self._nx)
        dtype = self._buf[0].dtype
        compute = torch.cuda.current_stream(self._device)
        start = self._timestep
        times = np.empty(n, dtype=np.float64)

        if to == "device":
            out = torch.empty(shape, dtype=dtype, device=self._device)
            for i, st in enumerate(steps):
                self._launch(int(start + st - self._timestep))
                self._enqueue_finite_check()
                out[i].copy_(self._buf[self._cur])
                times[i] = self.time
            self._raise_if_flagged()
            return Trajectory(times, out, self.model, self.stencil)

        host = torch.empty(shape, dtype=dtype, pin_memory=True)
        nstage = min(2, n)
        stage = [torch.empty((self._ny, self._nx), dtype=dtype, device=self._device) for _ in range(nstage)]
        drained = [None] * nstage  # copy-stream event: the D2H out of stage[k] has finished
        copier = torch.cuda.Stream(self._device)
        for i, st in enumerate(steps):
            self._launch(int(start + st - self._timestep))
            self._enqueue_finite_check()
            k = i % nstage
            if drained[k] is not None:
                compute.wait_event(drained[k])
            stage[k].copy_(self._buf[self._cur])
            ready = torch.cuda.Event()
            ready.record(compute)
            copier.wait_event(ready)
            with torch.cuda.stream(copier):
                host[i].copy_(stage[k], non_blocking=True)
                done = torch.cuda.Event()
                done.record(copier)
            drained[k] = done
            times[i] = self.time
        copier.synchronize()
        self._raise_if_flagged()
        return Trajectory(times, host.numpy().astype(np.float64), self.model, self.stencil)

    # ---------------------------------------------------- run_for_time
    def run_for_time(self, t, show_progress=False, t_interrupt=None, f_interrupt=None,
                     max_updates=100, min_update_time=10):
        """Run for simulation time ``t`` in chunks, calling ``f_interrupt(self)`` at
        ``t_interrupt`` (activemodelbplus/integrator/__init__.py:105-161).

        Chunks are enqueued without a host wait between them; a non-finite field
        raises :class:`CudaException` at the next interrupt or at the end, where the
        reference raises after the chunk. For sampling without host round trips use
        :meth:`sample_trajectory`.

        Raises:
            ValueError: if ``t`` or an interrupt time is not a multiple of dt.
        """
        nsteps = steps_from_time(self.stencil.dt, t)
        if t_interrupt is not None:
            assert f_interrupt is not None
            ti = np.asarray(t_interrupt)
            if np.any(ti < 0) or np.any(ti > t):
                raise ValueError("interrupt outside sim time window!")

        initial_timestep = self.timestep
        initial_time = self.time
        plot = None
        if show_progress:
            plot = _ProgressPlot(self.field)

        steps = step_iterator(self.stencil.dt, t, max_updates, min_update_time, t_interrupt=t_interrupt)
        if show_progress:
            steps = _progress(steps)

        for n in steps:
            if show_progress:
                for out in (sys.stdout, sys.stderr):
                    out.flush()
            if t_interrupt is not None and np.any(np.isclose(self.time - initial_time, t_interrupt)):
                self._raise_if_flagged()
                f_interrupt(self)
            assert n > 0
            # chunks are enqueued without waiting; the non-finite flag is read at
            # the next interrupt or at the end
            self._launch(int(n))
            self._enqueue_finite_check()
            if plot is not None:
                plot.update(self.field)

        if plot is not None:
            plot.close()
        self._raise_if_flagged()
        assert (self.timestep - initial_timestep) == nsteps
        if t_interrupt is not None and np.any(np.isclose(self.time - initial_time, t_interrupt)):
            f_interrupt(self)


# ------------------------------------------------------------------ ensemble

class Ensemble:
    """Many independent replicas advanced together on one GPU (no reference counterpart).

    Each replica has its own field (any size with ncols >= 112 and ncols % 4 == 0), stencil,
    model and Philox seed; storage is FP32 ("f32") or compensated FP32 ("f32c"). One kernel
    launch per step covers every replica, and ``graph_steps`` steps are captured once into a
    CUDA graph and replayed (C ABI ``amb_ensemble_*``).
    """

    def __init__(self, fields, stencils, models, *, precision: str = "f32c", seeds=None, graph_steps: int = 64):
        torch = _torch()
        if not torch.cuda.is_available():
            raise CudaException("no CUDA device is available")
        L = N.lib()
        fields = [np.ascontiguousarray(np.asarray(f, dtype=np.float64)) for f in fields]
        n = len(fields)
        if n == 0:
            raise ValueError("an ensemble needs at least one replica")
        stencils = [Stencil(stencils)] * n if isinstance(stencils, Stencil) else [Stencil(s) for s in stencils]
        models = [Model(models)] * n if isinstance(models, Model) else [Model(m) for m in models]
        if len(stencils) != n or len(models) != n:
            raise ValueError("one stencil and one model per replica (or a single shared one)")
        if precision not in ("f32", "f32c"):
            raise ValueError("ensemble precision must be 'f32' or 'f32c'")
        seeds = [_random_seed() for _ in range(n)] if seeds is None else [int(x) & 0xFFFFFFFFFFFFFFFF for x in seeds]
        self._shapes = [f.shape for f in fields]
        self._seeds = seeds
        nrows = (ctypes.c_int * n)(*[f.shape[0] for f in fields])
        ncols = (ctypes.c_int * n)(*[f.shape[1] for f in fields])
        ptrs = (ctypes.POINTER(ctypes.c_double) * n)(*[f.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) for f in fields])
        st = (N.amb_stencil * n)(*[N.stencil_struct(s) for s in stencils])
        md = (N.amb_model * n)(*[N.model_struct(m) for m in models])
        sd = (ctypes.c_uint64 * n)(*seeds)
        self._h = ctypes.c_void_p()
        _check(L.amb_ensemble_create(n, nrows, ncols, ptrs, st, md, sd, _PRECISIONS[precision], int(graph_steps),
                                     ctypes.byref(self._h)))

    def run(self, nsteps: int) -> None:
        _check(N.lib().amb_ensemble_run(self._h, int(nsteps)))

    def field(self, replica: int) -> np.ndarray:
        out = np.empty(self._shapes[replica])
        _check(N.lib().amb_ensemble_get_field(self._h, int(replica), out.ctypes.data))
        return out

    @property
    def fields(self):
        return [self.field(r) for r in range(len(self._shapes))]

    @property
    def offsets(self) -> np.ndarray:
        """Start of each replica in the packed layout of :meth:`gather` (length n + 1)."""
        return np.concatenate([[0], np.cumsum([r * c for r, c in self._shapes])]).astype(np.int64)

    def gather(self, out=None):
        """Every replica's current field packed back to back in one FP32 device tensor
        (device-to-device; replica r at ``offsets[r]``)."""
        torch = _torch()
        n = int(self.offsets[-1])
        if out is None:
            out = torch.empty(n, dtype=torch.float32, device="cuda")
        if out.dtype != torch.float32 or out.numel() < n or not out.is_contiguous():
            raise ValueError("out must be a contiguous float32 device tensor with room for every replica")
        torch.cuda.current_stream().synchronize()
        _check(N.lib().amb_ensemble_gather(self._h, out.data_ptr()))
        return out

    def scatter(self, src) -> None:
        """Set every replica's field from a packed FP32 device tensor (the layout of
        :meth:`gather`); clears the compensation residuals."""
        torch = _torch()
        if src.dtype != torch.float32 or src.numel() < int(self.offsets[-1]) or not src.is_contiguous():
            raise ValueError("src must be a contiguous float32 device tensor in the packed layout")
        torch.cuda.current_stream().synchronize()
        _check(N.lib().amb_ensemble_scatter(self._h, src.data_ptr()))

    def _info(self):
        ts, nt, sr = ctypes.c_int64(), ctypes.c_int(), ctypes.c_int()
        _check(N.lib().amb_ensemble_info(self._h, ctypes.byref(ts), ctypes.byref(nt), ctypes.byref(sr)))
        return ts.value, nt.value, sr.value

    @property
    def timestep(self) -> int:
        return self._info()[0]

    @property
    def ntasks(self) -> int:
        return self._info()[1]

    @property
    def seeds(self):
        return list(self._seeds)

    @property
    def fused(self) -> bool:
        """Whether the step kernel runs one warp per task doing every stage (True) or a
        producer/consumer warp pair (False); creation picks the faster by measurement, and
        assigning sets it. Both give bitwise the same fields."""
        form = ctypes.c_int()
        _check(N.lib().amb_ensemble_form(self._h, -1, ctypes.byref(form)))
        return bool(form.value)

    @fused.setter
    def fused(self, value: bool) -> None:
        _check(N.lib().amb_ensemble_form(self._h, 1 if value else 0, None))

    def __len__(self):
        return len(self._shapes)

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib().amb_ensemble_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------ helpers

def steps_from_time(dt, tfinal):
    """Number of steps to reach ``tfinal`` (activemodelbplus/integrator/__init__.py:39-57).

    Raises:
        ValueError: if ``tfinal`` is not a multiple of ``dt``.
    """
    nsteps = np.asarray(np.round(np.asarray(tfinal) / dt), dtype=int)
    error = np.abs(nsteps - np.asarray(tfinal) / dt)
    if not np.all(np.isclose(error, 0)):
        raise ValueError(f"tfinal={tfinal} is not a multiple of dt={dt}!")
    return nsteps.item() if nsteps.ndim == 0 else nsteps


def step_iterator(dt, tfinal, max_updates, min_update_time, t_interrupt=None):
    """Chunk sizes for a run of ``tfinal``: about even chunks, at most
    ``max_updates`` of them, at least ``min_update_time`` apart, split at every
    interrupt time (activemodelbplus/integrator/__init__.py:60-102)."""
    min_steps = max(int(np.round(min_update_time / dt)), 1)
    nsteps = steps_from_time(dt, tfinal)
    nupdates = max(min(nsteps // min_steps, max_updates), 1)
    timestep = np.linspace(0, nsteps, nupdates + 1, dtype=int)
    if t_interrupt is not None:
        interrupts = np.atleast_1d(steps_from_time(dt, np.asarray(t_interrupt).reshape(-1)))
        timestep = np.unique(np.concatenate([timestep, interrupts]))
    step_size = np.diff(timestep)
    assert len(step_size) >= 1
    assert np.sum(step_size) == nsteps
    assert np.all(step_size >= 0)
    return step_size


def plot_field(field, fig=None, axes=None, fontsize=8):
    """Draw (or redraw) the field with matplotlib (activemodelbplus/integrator/__init__.py:14-36).
    matplotlib is imported only here."""
    import matplotlib.pyplot as plt
    from matplotlib.colors import Normalize

    if fig is not None:
        ax, im, cbar = axes
        im.set_data(field)
        im.set_norm(Normalize(field.min(), vmax=field.max()))
        return fig, axes
    fig = plt.figure()
    ax = plt.gca()
    im = ax.imshow(field)
    cbar = fig.colorbar(im, ax=ax, fraction=0.05, pad=2e-2, location="right")
    cbar.set_label(r"$\phi$", fontsize=fontsize)
    cbar.ax.tick_params(labelsize=fontsize)
    ax.set_xlabel("$x$", fontsize=fontsize)
    ax.set_ylabel("$y$", fontsize=fontsize)
    ax.set_xticks([])
    ax.set_yticks([])
    return fig, (ax, im, cbar)


def _progress(it):
    try:
        from tqdm import tqdm
    except ImportError:
        return it
    return tqdm(it)


class _ProgressPlot:
    """Live field display for run_for_time; a no-op when matplotlib/IPython are absent."""

    def __init__(self, field):
        try:
            import matplotlib.pyplot  # noqa: F401
            self.fig, self.axes = plot_field(field)
        except ImportError:
            self.fig = None

    def update(self, field):
        if self.fig is None:
            return
        plot_field(field, self.fig, self.axes)
        try:
            from IPython.display import clear_output, display
            clear_output(wait=True)
            display(self.fig)
        except ImportError:
            pass

    def close(self):
        if self.fig is not None:
            import matplotlib.pyplot as plt
            plt.close(self.fig)
