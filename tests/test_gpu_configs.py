"""Parity at the sizes and launch shapes the measurements use, on the GPU.

* The FP32-compensated step at the bench workload (4096^2 AMB+, zeta=-1, lambda=0.5,
  T=0.05) with the launch shape the bench times (sliding kernel, default row segments, four
  warp pairs per CTA), 1000 steps, against the FP64 path with the same Philox key: the
  structure factor within 1e-4 (relative L2 over the notebook's bins,
  examples/structureFactor.ipynb), and the field's max and RMS error bounded.
* The 1024^2 noisy AMB+ configuration (zeta=-4, lambda=-1, T=0.05, phi0=-0.4): host-injected
  noise step by step against the oracle (FP64 at the reference's tight_tol, 1e-12 relative;
  FP32-compensated at 1e-6); then 10^5 Philox steps, FP32-compensated against FP64; and at
  T = 0, 10^4 FP64 steps against the reference's own CUDA integrator at 1e-12 relative
  (the long-run pins of test/test_integrator.cc:197-251 at the configuration's size).
"""
import ctypes

import numpy as np
import pytest

import oracle
from oracle import Params

pytestmark = pytest.mark.gpu


def _api():
    from activemodelbplus.integrator import Integrator, Model, Stencil
    return Integrator, Model, Stencil


def _errors(a, b, phi0):
    """max |a - b|, RMS (a - b), relative L2 of S(k) (the notebook's bins) of a against b."""
    from activemodelbplus.analysis import structure_factor
    d = a - b
    _, sa, _ = structure_factor(a, phi0=phi0)
    _, sb, _ = structure_factor(b, phi0=phi0)
    m = np.isfinite(sb)
    return (float(np.abs(d).max()), float(np.sqrt(np.mean(d * d))),
            float(np.linalg.norm(sa[m] - sb[m]) / np.linalg.norm(sb[m])))


def test_bench_workload_f32c_at_bench_launch_shape_tracks_fp64():
    """4096^2, 1000 steps: the kernel and launch shape behind the headline number against FP64.
    Bounds: S(k) relative L2 <= 1e-4 (the FP32-compensated accuracy target), max |d| < 1e-6,
    RMS < 1e-7 (the residual keeps the field within a few FP32 ulps of 0.4)."""
    Integrator, Model, Stencil = _api()
    rng = np.random.default_rng(2024)
    field = -0.4 + 0.01 * rng.standard_normal((4096, 4096))
    stencil, model = Stencil(1e-3, 1, 1), Model(-0.25, 0, 0.25, 1, 0.5, -1, 0.05)
    f64 = Integrator(field, stencil, model, precision="f64", seed=1000)
    f64.run(1000)
    ref = f64.field
    del f64
    sim = Integrator(field, stencil, model, precision="f32c", seed=1000, kernel="sliding",
                     launch={"seg_rows": 0, "pairs_per_cta": 4})
    sim.run(1000)
    got = sim.field
    emax, erms, esk = _errors(got, ref, -0.4)
    assert emax < 1e-6 and erms < 1e-7, (emax, erms)
    assert esk < 1e-4, esk


CONFIG1 = dict(dt=1e-3, dx=1.0, dy=1.0, a=-0.25, b=0.0, c=0.25, kappa=1.0, lamb=-1.0, zeta=-4.0, T=0.05)


def _config1_field():
    rng = np.random.default_rng(1)
    return -0.4 + 0.01 * rng.standard_normal((1024, 1024))


def test_config1_injected_noise_stepwise():
    """1024^2, host-supplied standard normals, 3 steps: FP64 device steps equal the oracle's at
    1e-12 relative after every step; the FP32-compensated kernels stay within 1e-6."""
    import torch
    from activemodelbplus.integrator import _native as N
    ny = nx = 1024
    p = Params(**CONFIG1)
    field = _config1_field()
    noise = np.random.default_rng(2).standard_normal((3, 2, ny, nx))
    s = N.amb_stencil(p.dt, p.dx, p.dy)
    m = N.amb_model(p.a, p.b, p.c, p.kappa, p.lamb, p.zeta, p.T)
    stream = torch.cuda.current_stream().cuda_stream
    a = torch.from_numpy(field.copy()).cuda()
    b = torch.empty_like(a)
    dn = torch.from_numpy(noise).cuda()
    ref = field
    for k in range(3):
        flag = ctypes.c_int(0)
        rc = N.lib().amb_step_f64(ctypes.byref(s), ctypes.byref(m), 0, ny, nx, a.data_ptr(), b.data_ptr(), k, 1,
                                  dn[k].data_ptr(), stream, ctypes.byref(flag))
        assert rc == 0 and flag.value == 1, N.last_error()
        a, b = b, a
        ref = oracle.run(ref, p, 1, noise="injected", injected=noise[k:k + 1], nthreads=8)
        got = a.cpu().numpy()
        assert np.abs(got - ref).max() / np.abs(ref).max() < 1e-12
    # FP32-compensated, both kernels, the same normals rounded to FP32
    noise32 = noise.astype(np.float32)
    ref32 = oracle.run(field, p, 3, noise="injected", injected=noise32.astype(np.float64), nthreads=8)
    for kernel in (N.AMB_KERNEL_TILE, N.AMB_KERNEL_SLIDING):
        fa = torch.from_numpy(field.astype(np.float32)).cuda()
        fb = torch.empty_like(fa)
        res = torch.zeros((ny, nx), dtype=torch.int16, device="cuda")
        inj = torch.from_numpy(noise32).cuda()
        cfg = N.amb_kernel_config(kernel, 0, 0, 0)
        flag = ctypes.c_int(0)
        rc = N.lib().amb_step_f32_ex(ctypes.byref(s), ctypes.byref(m), 0, ny, nx, fa.data_ptr(), fb.data_ptr(),
                                     res.data_ptr(), 0, 3, inj.data_ptr(), ctypes.byref(cfg), stream,
                                     ctypes.byref(flag))
        assert rc == 0, N.last_error()
        got = (fb if flag.value else fa).double().cpu().numpy()
        assert np.abs(got - ref32).max() < 1e-6, kernel


def test_config1_long_run_f32c_tracks_fp64():
    """1024^2, 10^5 steps (t = 100) with the same Philox key: FP32-compensated against FP64.
    Bounds: S(k) relative L2 < 1e-4; max |d| < 1e-4 and RMS < 1e-5 (rounding differences grow
    with the phase-separating dynamics over t = 100); mean conserved to FP32 roundoff."""
    Integrator, Model, Stencil = _api()
    p = CONFIG1
    field = _config1_field()
    stencil = Stencil(p["dt"], p["dx"], p["dy"])
    model = Model(p["a"], p["b"], p["c"], p["kappa"], p["lamb"], p["zeta"], p["T"])
    f64 = Integrator(field, stencil, model, precision="f64", seed=31)
    f64.run(100000)
    ref = f64.field
    sim = Integrator(field, stencil, model, precision="f32c", seed=31)
    sim.run(100000)
    got = sim.field
    emax, erms, esk = _errors(got, ref, -0.4)
    assert esk < 1e-4, esk
    assert emax < 1e-4 and erms < 1e-5, (emax, erms)
    assert abs(ref.mean() - field.mean()) < 1e-12
    assert abs(got.mean() - field.mean()) < 1e-6


@pytest.mark.skipif(not oracle.ReferenceGpuIntegrator.available(), reason="reference cubin not built")
def test_config1_t0_fp64_matches_reference_cuda_integrator():
    """1024^2 AMB+ at T = 0, 10^4 steps: the FP64 path against the reference's CUDA integrator
    (its own kernels, run from the cubin built from src/integrator.cu) at 1e-12 relative."""
    Integrator, Model, Stencil = _api()
    p = dict(CONFIG1, T=0.0)
    field = _config1_field()
    ref = oracle.ReferenceGpuIntegrator(field, Params(**p), seed=1)
    ref.run(10000)
    want = ref.field
    ref.close()
    sim = Integrator(field, Stencil(p["dt"], p["dx"], p["dy"]),
                     Model(p["a"], p["b"], p["c"], p["kappa"], p["lamb"], p["zeta"], 0.0))
    sim.run(10000)
    got = sim.field
    assert np.abs(got - want).max() / np.abs(want).max() < 1e-12
