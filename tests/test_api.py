"""API surface of Model / Stencil / helpers, following the reference's binding
tests (test/test_bindings.py:10-49) and Python wrapper
(activemodelbplus/integrator/__init__.py:39-102). No GPU needed."""
import numpy as np
import pytest

from activemodelbplus.integrator import (CudaException, Model, Stencil, step_iterator, steps_from_time)


def test_model():
    params = (1, 2, 3, 4, 5, 6, 7)
    model = Model(*params)
    copy = Model(model)
    assert params == model.as_tuple()
    assert (model.a, model.b, model.c, model.kappa, model.lamb, model.zeta, model.T) == params
    assert copy is not model
    assert copy == model
    assert copy.as_tuple() == model.as_tuple()
    assert copy.as_dict() == model.as_dict()
    copy.a += 1
    assert copy != model
    assert copy.as_tuple() != model.as_tuple()
    assert copy.as_dict() != model.as_dict()


def test_model_keywords_dict_and_repr():
    m = Model(a=-0.25, b=0, c=0.25, kappa=1, lamb=-1, zeta=-4, T=0.05)
    assert m.as_dict() == {"a": -0.25, "b": 0.0, "c": 0.25, "kappa": 1.0, "lamb": -1.0, "zeta": -4.0,
                           "temperature": 0.05}
    assert repr(m) == "<Model " + str(m.as_dict()) + ">"
    assert str(m) == str(m.as_dict())
    assert Model().as_tuple() == (0.0,) * 7
    assert Model(model=m) == m
    with pytest.raises(AttributeError):
        m.temperature = 1.0
    with pytest.raises(TypeError):
        Model(1, 2, 3, 4, 5, 6, 7, 8)


def test_stencil():
    params = (1, 2, 3)
    stencil = Stencil(*params)
    copy = Stencil(stencil)
    assert params == stencil.as_tuple()
    assert (stencil.dt, stencil.dx, stencil.dy) == params
    assert copy is not stencil
    assert copy == stencil
    assert copy.as_dict() == stencil.as_dict()
    copy.dx += 1
    assert copy.as_tuple() != stencil.as_tuple()
    assert copy.as_dict() != stencil.as_dict()
    assert repr(Stencil(dt=1e-3, dx=1, dy=1)) == "<Stencil {'dt': 0.001, 'dx': 1.0, 'dy': 1.0}>"


def test_steps_from_time():
    assert steps_from_time(1e-3, 1.0) == 1000
    assert steps_from_time(1e-2, 1e3) == 100000
    assert list(steps_from_time(0.1, np.array([0.5, 1.0]))) == [5, 10]
    with pytest.raises(ValueError):
        steps_from_time(1e-2, 0.015)


def test_step_iterator():
    s = step_iterator(1e-2, 100.0, max_updates=10, min_update_time=1)
    assert s.sum() == 10000 and len(s) == 10
    s = step_iterator(1e-2, 1.0, max_updates=100, min_update_time=10)
    assert list(s) == [100]
    s = step_iterator(0.1, 10.0, max_updates=4, min_update_time=1, t_interrupt=[0.3, 5.0])
    assert s.sum() == 100
    edges = np.cumsum(np.concatenate([[0], s]))
    assert 3 in edges and 50 in edges


def test_integrator_without_gpu_raises():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from activemodelbplus.integrator import Integrator
    with pytest.raises(CudaException):
        Integrator(np.zeros((16, 16)), Stencil(1e-3, 1, 1), Model())
