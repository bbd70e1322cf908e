"""The ``.npz`` trajectory format: the keys and shapes the reference's analysis
notebook writes (examples/structureFactor.ipynb cell 1: ``np.savez(path,
time=..., field=..., **model.as_dict(), **stencil.as_dict())``) and reads back
(cells 5 and 7: ``traj['field']``, ``traj['time']``, ``traj['dx']``,
``traj['dy']``). No GPU needed."""
import numpy as np
import pytest

from activemodelbplus.integrator import Model, Stencil
from activemodelbplus.trajectory import Trajectory


def _notebook_style_file(path, rng):
    model = Model(a=-0.25, b=0, c=0.25, kappa=1, lamb=0.5, zeta=-1, T=0.05)
    stencil = Stencil(dt=1e-2, dx=1, dy=1)
    time = [1.0, 10.0, 100.0]
    field = [rng.standard_normal((16, 24)) for _ in time]
    params = model.as_dict()
    params.update(stencil.as_dict())
    np.savez(path, time=time, field=field, **params)
    return model, stencil, np.asarray(time), np.asarray(field)


def test_load_notebook_layout(tmp_path):
    rng = np.random.default_rng(0)
    path = tmp_path / "trajectory_1.npz"
    model, stencil, time, field = _notebook_style_file(path, rng)
    tr = Trajectory.load(str(path))
    assert tr.model == model and tr.stencil == stencil
    assert np.array_equal(tr.time, time) and np.array_equal(tr.field, field)


def test_save_matches_notebook_layout(tmp_path):
    rng = np.random.default_rng(1)
    model = Model(-0.25, 0, 0.25, 1, -1, -4, 0.05)
    stencil = Stencil(1e-3, 1, 1)
    field = rng.standard_normal((2, 8, 12))
    Trajectory([0.5, 1.0], field, model, stencil).save(str(tmp_path / "t.npz"))
    z = np.load(tmp_path / "t.npz")
    assert set(z.files) == {"time", "field", "a", "b", "c", "kappa", "lamb", "zeta", "temperature", "dt", "dx",
                            "dy"}
    assert z["field"].dtype == np.float64 and z["field"].shape == (2, 8, 12)
    assert float(z["temperature"]) == 0.05 and float(z["lamb"]) == -1 and float(z["dt"]) == 1e-3
    # the reads the notebook's analysis cells make
    assert z["field"][0].shape == (8, 12) and float(z["dx"]) == 1.0
    assert np.array_equal(z["time"], [0.5, 1.0])


def test_missing_keys_and_length_mismatch(tmp_path):
    np.savez(tmp_path / "bad.npz", time=[0.0], field=np.zeros((1, 4, 4)))
    with pytest.raises(KeyError):
        Trajectory.load(str(tmp_path / "bad.npz"))
    with pytest.raises(ValueError):
        Trajectory([0.0, 1.0], np.zeros((1, 4, 4)), Model(), Stencil())
