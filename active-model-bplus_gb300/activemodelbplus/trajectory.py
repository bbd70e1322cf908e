"""Sampled trajectories and their ``.npz`` file format.

The file layout is the one the reference's analysis notebook writes and reads
(examples/structureFactor.ipynb, cell 1 writes, cells 5 and 7 read): arrays
``time`` (n,) and ``field`` (n, ny, nx) float64, plus one scalar entry per
parameter of ``Model.as_dict()`` (a, b, c, kappa, lamb, zeta, temperature) and
``Stencil.as_dict()`` (dt, dx, dy). Files written here load in that notebook
unchanged, and its files load here.
"""
from __future__ import annotations

import numpy as np

_MODEL_KEYS = ("a", "b", "c", "kappa", "lamb", "zeta", "temperature")
_STENCIL_KEYS = ("dt", "dx", "dy")


class Trajectory:
    """Fields sampled at a sequence of times, with the parameters that made them.

    Attributes:
        time: (n,) float64 absolute simulation times.
        field: (n, ny, nx) float64 host array, or a device tensor when sampled with
            ``to="device"`` (native dtype of the integrator's storage).
        model, stencil: the run's :class:`Model` and :class:`Stencil`.
    """

    def __init__(self, time, field, model, stencil):
        self.time = np.asarray(time, dtype=np.float64)
        self.field = field
        self.model = model
        self.stencil = stencil
        if len(self.time) != len(field):
            raise ValueError("time and field have different lengths")

    def __len__(self) -> int:
        return len(self.time)

    def params(self) -> dict:
        """Model and stencil parameters under the notebook's keys."""
        d = dict(self.model.as_dict())
        d.update(self.stencil.as_dict())
        return d

    def host_field(self) -> np.ndarray:
        """The samples as a float64 host array."""
        f = self.field
        if not isinstance(f, np.ndarray):
            f = f.double().cpu().numpy()
        return np.asarray(f, dtype=np.float64)

    def save(self, path: str) -> None:
        """Write the notebook's ``.npz`` layout."""
        np.savez(path, time=self.time, field=self.host_field(), **self.params())

    @classmethod
    def load(cls, path: str) -> "Trajectory":
        """Read a trajectory file (written here or by the reference's notebook)."""
        from .integrator import Model, Stencil

        z = np.load(path, allow_pickle=False)
        missing = [k for k in ("time", "field") + _MODEL_KEYS + _STENCIL_KEYS if k not in z.files]
        if missing:
            raise KeyError(f"{path}: missing entries {missing}")
        m = {k: float(z[k]) for k in _MODEL_KEYS}
        model = Model(a=m["a"], b=m["b"], c=m["c"], kappa=m["kappa"], lamb=m["lamb"], zeta=m["zeta"],
                      T=m["temperature"])
        stencil = Stencil(dt=float(z["dt"]), dx=float(z["dx"]), dy=float(z["dy"]))
        return cls(z["time"], np.asarray(z["field"], dtype=np.float64), model, stencil)
