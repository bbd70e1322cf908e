"""The FP64 path against the reference's own CUDA integrator, run on the same GPU from
its compiled cubin (oracle/_ref/ref_integrator.cubin, built from the reference sources by
oracle/build.py). At T = 0 both are deterministic: 1e-12 relative after the steps."""
import numpy as np
import pytest

import oracle
from oracle import Params, ReferenceGpuIntegrator

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ReferenceGpuIntegrator.available(), reason="reference cubin not built")]


@pytest.mark.parametrize("shape,model,nsteps", [
    ((256, 256), dict(a=-0.25, b=0.0, c=0.25, kappa=1.0, lamb=0.0, zeta=0.0), 2000),   # Model B spinodal
    ((128, 192), dict(a=-0.25, b=0.1, c=0.25, kappa=1.0, lamb=-1.0, zeta=-4.0), 500),  # AMB+, b != 0
    ((64, 96), dict(a=-0.2, b=0.0, c=0.3, kappa=0.8, lamb=0.5, zeta=-1.0), 300),
])
def test_fp64_path_matches_reference_cuda_integrator(shape, model, nsteps):
    from activemodelbplus.integrator import Integrator, Model, Stencil
    rng = np.random.default_rng(shape[0])
    field = -0.1 + 0.1 * rng.random(shape)
    p = Params(dt=1e-3, dx=1.0, dy=1.0, T=0.0, **model)
    ref = ReferenceGpuIntegrator(field, p, seed=1)
    ref.run(nsteps)
    want = ref.field
    ref.close()
    sim = Integrator(field, Stencil(p.dt, p.dx, p.dy), Model(p.a, p.b, p.c, p.kappa, p.lamb, p.zeta, 0.0))
    sim.run(nsteps)
    got = sim.field
    assert np.abs(got - want).max() / np.abs(want).max() < 1e-12


def test_reference_cuda_integrator_matches_golden_spinodal():
    """The reference GPU run reproduces the reference CPU scheme's stored 256^2, 10^4-step result."""
    import os
    from conftest import GOLDEN
    g = np.load(os.path.join(GOLDEN, "tjhung_spinodal_256.npz"))
    p = Params(dt=float(g["dt"]), a=-0.25, b=0.0, c=0.25, kappa=1.0)
    ref = ReferenceGpuIntegrator(g["initial"], p, seed=1)
    ref.run(int(g["nsteps"]))
    f = ref.field
    ref.close()
    assert np.abs(f[::4, ::4] - g["final_sub"]).max() / float(g["final_absmax"]) < 1e-12


def test_reference_noise_statistics_match_philox_noise():
    """T > 0: curand XORWOW and Philox give statistically equal runs (mean field and variance
    after 200 steps agree within sampling error); bitwise comparison is impossible."""
    from activemodelbplus.integrator import Integrator, Model, Stencil
    field = np.full((256, 256), -0.4)
    p = Params(dt=1e-3, dx=1.0, dy=1.0, a=-0.25, b=0.0, c=0.25, kappa=1.0, lamb=-1.0, zeta=-4.0, T=0.05)
    ref = ReferenceGpuIntegrator(field, p, seed=7)
    ref.run(200)
    a = ref.field
    ref.close()
    sim = Integrator(field, Stencil(p.dt, p.dx, p.dy), Model(p.a, p.b, p.c, p.kappa, p.lamb, p.zeta, p.T), seed=7)
    sim.run(200)
    b = sim.field
    assert abs(a.mean() - b.mean()) < 1e-9          # both conserve the mean
    assert abs(a.std() / b.std() - 1) < 0.02         # same noise amplitude
