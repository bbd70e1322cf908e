"""Batched ensemble: every replica equals a standalone Integrator run of the same field,
parameters and seed (bitwise: same kernel arithmetic, decomposition-independent noise),
across graph replays, odd remainders and both graph parities."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(128, 128), (192, 192), (256, 320), (144, 112), (64, 256), (100, 200)]


def replicas():
    from activemodelbplus.integrator import Model, Stencil
    rng = np.random.default_rng(0)
    fields, stencils, models = [], [], []
    for i, shape in enumerate(SHAPES):
        phi0 = rng.uniform(-0.6, 0.6)
        fields.append(phi0 + 0.02 * rng.standard_normal(shape))
        stencils.append(Stencil(1e-3, 1.0, 1.0 if i % 2 == 0 else 1.1))
        T = 0.0 if i % 3 == 0 else rng.uniform(0, 0.1)
        models.append(Model(-0.25, 0, 0.25, 1, rng.uniform(-1, 1), rng.uniform(-4, 4), T))
    return fields, stencils, models


@pytest.mark.parametrize("precision", ["f32c", "f32"])
@pytest.mark.parametrize("fused", [False, True])
def test_ensemble_replicas_equal_single_runs(precision, fused):
    """Both kernel forms (warp pair per task, one warp per task)."""
    from activemodelbplus.integrator import Ensemble, Integrator
    fields, stencils, models = replicas()
    seeds = [100 + i for i in range(len(fields))]
    ens = Ensemble(fields, stencils, models, precision=precision, seeds=seeds, graph_steps=8)
    ens.fused = fused
    assert ens.fused == fused
    for n in (30, 7, 16):   # 3 graph replays + 6 single steps; 7 single steps (parity flips); 2 replays
        ens.run(n)
    assert ens.timestep == 53
    for r, (f, st, m) in enumerate(zip(fields, stencils, models)):
        sim = Integrator(f, st, m, precision=precision, seed=seeds[r], kernel="sliding")
        sim.run(53)
        assert np.array_equal(ens.field(r), sim.field), r
    ens.close()


def test_ensemble_rejects_narrow_replicas_and_nonfinite():
    from activemodelbplus.integrator import CudaException, Ensemble, Model, Stencil
    with pytest.raises(ValueError):
        Ensemble([np.zeros((64, 100))], Stencil(1e-3, 1, 1), Model())
    bad = np.zeros((64, 128))
    bad[3, 4] = np.nan
    ens = Ensemble([np.zeros((64, 128)), bad], Stencil(1e-3, 1, 1), Model(-0.25, 0, 0.25, 1, 0, 0, 0))
    with pytest.raises(CudaException):
        ens.run(2)


def test_config4_scale_ensemble_replicas_equal_single_runs():
    """The batched-ensemble configuration at its size: 256 replicas with sizes drawn from
    {128, 192, 256, 384, 512, 768, 1024}^2 and zeta in [-4, 4], lambda in [-1, 1], phi0 in
    [-0.6, 0.6], T in [0, 0.1] (a=-0.25, c=0.25, kappa=1, dt=1e-3), FP32-compensated, 12 steps
    (a 4-step graph replayed three times). The first replica of every size class, and a few more,
    equal standalone Integrator runs of the same field, parameters and seed bitwise."""
    from activemodelbplus.integrator import Ensemble, Integrator, Model, Stencil
    rng = np.random.default_rng(7)
    sizes = rng.choice([128, 192, 256, 384, 512, 768, 1024], size=256)
    fields, models = [], []
    for n in sizes:
        phi0 = rng.uniform(-0.6, 0.6)
        fields.append(phi0 + 0.01 * rng.standard_normal((n, n)))
        models.append(Model(-0.25, 0, 0.25, 1, rng.uniform(-1, 1), rng.uniform(-4, 4), rng.uniform(0, 0.1)))
    stencil = Stencil(1e-3, 1, 1)
    ens = Ensemble(fields, stencil, models, precision="f32c", seeds=list(range(256)), graph_steps=4)
    ens.run(12)
    picks = sorted({int(np.flatnonzero(sizes == s)[0]) for s in np.unique(sizes)} | {3, 100, 255})
    for r in picks:
        sim = Integrator(fields[r], stencil, models[r], precision="f32c", seed=r, kernel="sliding")
        sim.run(12)
        assert np.array_equal(ens.field(r), sim.field), (r, sizes[r])
    ens.close()
