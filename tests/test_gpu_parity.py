"""Parity of the CUDA library with the reference, on the GPU.

The reference's own test cases (test/test_tjhung.cc, test/test_integrator.cc)
re-expressed in pytest and run against the golden fixtures made by the
reference's CPU scheme and against the oracle (oracle/amb_oracle.c, itself
pinned to the reference in test_oracle.py).

Tolerances: FP64 path 1e-12 (the reference's tight_tol, absolute, elementwise;
test/test_utilities.h:7), relative to max|phi| for multi-step runs. FP32 paths
are compared with the FP64 path at the tolerances stated per test.
"""
import ctypes
import os

import numpy as np
import pytest

import oracle
from oracle import Params
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

TIGHT = 1e-12
LOOSE = 1e-6


def lib_integrator():
    from activemodelbplus import integrator
    return integrator


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


def params_of(stencil, model):
    return Params(dt=stencil.dt, dx=stencil.dx, dy=stencil.dy, a=model.a, b=model.b, c=model.c,
                  kappa=model.kappa, lamb=model.lamb, zeta=model.zeta, T=model.T)


def maxabs(a):
    return float(np.max(np.abs(a)))


# --------------------------------------------------------------- reference pins

def test_tjhung_integration_case():
    """test/test_tjhung.cc:8-40 against the stored reference outputs."""
    I = lib_integrator()
    g = golden("tjhung_onestep_64x32.npz")
    A, K, lamb, zeta, dt = (float(g[k]) for k in ("A", "K", "lamb", "zeta", "dt"))
    sim = I.Integrator(g["initial"], I.Stencil(dt, 1, 1), I.Model(-A, 0, A, K, lamb, zeta, 0))
    assert maxabs(sim.passive_chemical_potential - g["mueq"]) < TIGHT
    assert maxabs(sim.active_chemical_potential - g["muact"]) < TIGHT
    jeq = sim.passive_current
    assert maxabs(jeq[0] - g["jxeq"]) < TIGHT
    assert maxabs(jeq[1] - g["jyeq"]) < TIGHT
    jact = sim.active_current
    assert maxabs(jact[0] - g["jxact"]) < TIGHT
    assert maxabs(jact[1] - g["jyact"]) < TIGHT
    sim.run(1)
    actual_div = -(sim.field - g["initial"]) / dt
    assert maxabs(actual_div + g["dphi"]) < TIGHT * 10  # field ~1, /dt amplifies ulps by 100


def test_spinodal_256_1e4_steps_matches_reference():
    """Model B spinodal 256^2, dt=1e-3, 10^4 steps: 1e-12 relative to max|phi| against
    the reference CPU scheme's stored result."""
    I = lib_integrator()
    g = golden("tjhung_spinodal_256.npz")
    sim = I.Integrator(g["initial"], I.Stencil(float(g["dt"]), 1, 1), I.Model(-0.25, 0, 0.25, 1, 0, 0, 0))
    sim.run(int(g["nsteps"]))
    f = sim.field
    scale = float(g["final_absmax"])
    assert maxabs(f[::4, ::4] - g["final_sub"]) / scale < TIGHT
    assert abs(f.sum() - float(g["final_sum"])) < 1e-9
    assert sim.timestep == 10000


def test_active_64_matches_reference():
    I = lib_integrator()
    g = golden("tjhung_active_64.npz")
    sim = I.Integrator(g["initial"], I.Stencil(float(g["dt"]), 1, 1),
                       I.Model(-0.25, 0, 0.25, 1, float(g["lamb"]), float(g["zeta"]), 0))
    sim.run(int(g["nsteps"]))
    assert maxabs(sim.field - g["final"]) / maxabs(g["final"]) < TIGHT


# ----------------------------------------------- per-term cases (test_integrator.cc)

@pytest.mark.parametrize("case", ["bulk", "kappa", "lambda", "zeta", "all"])
def test_single_term_currents(case):
    """test/test_integrator.cc:47-195: one physics term on at a time, 32x64 random field,
    dy != dx; every getter and the one-step divergence at 1e-12."""
    I = lib_integrator()
    rng = np.random.default_rng(["bulk", "kappa", "lambda", "zeta", "all"].index(case))
    field = rng.uniform(-1, 1, (32, 64))
    dt = 1e-2
    stencil = {"zeta": I.Stencil(dt, 1, 1.25)}.get(case, I.Stencil(dt, 1, 0.75))
    model = {"bulk": I.Model(1, 2, 3, 0, 0, 0, 0), "kappa": I.Model(0, 0, 0, 1, 0, 0, 0),
             "lambda": I.Model(0, 0, 0, 0, 1, 0, 0), "zeta": I.Model(0, 0, 0, 0, 0, 1, 0),
             "all": I.Model(-0.3, 0.4, 0.25, 0.8, -1.2, 2.5, 0)}[case]
    sim = I.Integrator(field, stencil, model)
    p = params_of(stencil, model)
    t = oracle.terms(field, p)
    assert maxabs(sim.chemical_potential - (t["mu_p"] + t["mu_a"])) < TIGHT
    assert maxabs(sim.passive_chemical_potential - t["mu_p"]) < TIGHT
    for name, (ky, kx) in {"passive_current": ("jp_y", "jp_x"), "lambda_current": ("jl_y", "jl_x"),
                           "circulating_current": ("jc_y", "jc_x")}.items():
        got = getattr(sim, name)
        assert maxabs(got[0] - t[ky]) < TIGHT, name
        assert maxabs(got[1] - t[kx]) < TIGHT, name
    if case == "bulk" or case == "kappa":
        assert maxabs(np.array(sim.active_current)) < TIGHT
    if case in ("lambda", "zeta"):
        assert maxabs(np.array(sim.passive_current)) < TIGHT
    if case == "zeta":
        assert maxabs(sim.chemical_potential) < TIGHT
        assert maxabs(np.array(sim.lambda_current)) < TIGHT
    assert maxabs(np.array(sim.random_current)) == 0.0
    sim.run(1)
    actual_div = -(sim.field - field) / dt
    expected_div = oracle.divergence(field, p)
    assert maxabs(actual_div - expected_div) < TIGHT * max(1.0, maxabs(expected_div))


def test_timestep_accounting():
    """test/test_integrator.cc:253-266 (and run(n<=0) advancing the counter, src/integrator.cu:520)."""
    I = lib_integrator()
    sim = I.Integrator(np.random.default_rng(0).uniform(-1, 1, (64, 64)), I.Stencil(0.1, 1, 1), I.Model())
    assert sim.timestep == 0
    sim.run(10)
    assert sim.timestep == 10
    assert abs(sim.time - 1.0) < TIGHT
    sim.run(0)
    assert sim.timestep == 10


def test_constructor_and_copies():
    """test/test_bindings.py:51-71 and test/test_integrator.cc:9-21."""
    I = lib_integrator()
    stencil = I.Stencil(1e-2, 1, 1)
    model = I.Model(0.25, 0.5, 0.25, 1, 1, 1, 0)
    initial = np.random.random((128, 256))
    sim = I.Integrator(initial, stencil, model)
    assert (sim.field == initial).all()
    assert sim.stencil is not stencil and sim.model is not model
    assert sim.stencil == stencil and sim.model == model
    assert sim.timestep == 0
    sim.run(1)
    assert (sim.field != initial).any()
    assert sim.timestep == 1
    assert sim.time == stencil.dt


# ----------------------------------------------------------- sizes and conservation

@pytest.mark.parametrize("shape", [(1, 1), (2, 3), (5, 9), (17, 23), (33, 64), (64, 31), (100, 7)])
def test_arbitrary_grid_sizes(shape):
    """Any nrows, ncols >= 1 (the reference needs multiples of its 8x8 tile)."""
    I = lib_integrator()
    rng = np.random.default_rng(shape[0] * 1000 + shape[1])
    field = rng.uniform(-0.5, 0.5, shape)
    stencil, model = I.Stencil(1e-3, 1, 0.9), I.Model(-0.25, 0.1, 0.25, 1, -1, -4, 0)
    sim = I.Integrator(field, stencil, model)
    sim.run(20)
    ref = oracle.run(field, params_of(stencil, model), 20)
    assert maxabs(sim.field - ref) / max(maxabs(ref), 1e-300) < TIGHT


def test_mass_conservation():
    """test/test_integrator.cc:197-228: 512x256, 1000 steps, four models; trajectories differ."""
    I = lib_integrator()
    rng = np.random.default_rng(1)
    initial = 0.1 * rng.uniform(-1, 1, (256, 512))
    initial -= initial.mean()
    stencil = I.Stencil(1e-2, 1, 1.25)
    prev = None
    for m in (I.Model(-0.25, 0, 0.25, 1, 0, 0, 0), I.Model(-0.25, 0.5, 0.25, 1, 0, 0, 0),
              I.Model(-0.25, 0.5, 0.25, 1, 1, 0, 0), I.Model(-0.25, 0.5, 0.25, 1, 1, 1, 0)):
        sim = I.Integrator(initial, stencil, m)
        m0 = sim.mass()
        sim.run(1000)
        f = sim.field
        assert abs(oracle.mass(f) - m0) < LOOSE
        assert abs(sim.mass() - oracle.mass(f)) < 1e-12
        if prev is not None:
            assert maxabs(f - prev) > LOOSE
        prev = f


def test_phase_separation():
    """test/test_integrator.cc:230-251: 10^5 steps of Model B reach the binodal +-1 within 0.1."""
    I = lib_integrator()
    rng = np.random.default_rng(2)
    initial = 0.1 * rng.uniform(-1, 1, (256, 512))
    initial -= initial.mean()
    sim = I.Integrator(initial, I.Stencil(1e-2, 1, 1.25), I.Model(-0.25, 0, 0.25, 1, 0, 0, 0))
    sim.run(100000)
    f = sim.field
    assert abs(f.max() - 1) < 0.1 and abs(f.min() + 1) < 0.1


# ------------------------------------------------------------------ noise

def test_philox_normals_match_oracle():
    """The device's Philox + Box-Muller normals equal the oracle's definition to the accuracy of
    their single-precision evaluation (5e-5 absolute for |z| <= 5.8; both field precisions draw
    the same device normals, so the FP64 and FP32 random currents are identical)."""
    I = lib_integrator()
    ny, nx, seed = 48, 72, 0x1234_5678_9ABC_DEF0
    model = I.Model(-0.25, 0, 0.25, 1, 0, 0, 0.05)
    stencil = I.Stencil(1e-3, 1, 1)
    mag = np.sqrt(2 * model.T) * np.sqrt(1 / (stencil.dt * stencil.dx * stencil.dy))
    field = np.zeros((ny, nx))
    xy, xx = oracle.normals(ny, nx, seed, 3)
    currents = {}
    for precision in ("f64", "f32"):
        sim = I.Integrator(field, stencil, model, precision=precision, seed=seed)
        sim.set_field(field)
        sim._timestep = 3  # noise of step 3
        jr = sim.random_current
        assert maxabs(jr[0] / mag - xy) < 5e-5
        assert maxabs(jr[1] / mag - xx) < 5e-5
        currents[precision] = jr
    assert np.array_equal(currents["f64"][0], currents["f32"][0])


def test_philox_run_matches_oracle():
    """Full Philox-noise FP64 run at T > 0: step by step, the step kernel's in-tile noise (one
    Philox call per column quad) equals the per-site noise the diagnostics report, and with those
    normals injected the oracle reproduces the run at 1e-12."""
    I = lib_integrator()
    rng = np.random.default_rng(4)
    field = -0.4 + 0.01 * rng.standard_normal((64, 96))
    stencil, model = I.Stencil(1e-3, 1, 1), I.Model(-0.25, 0, 0.25, 1, -1, -4, 0.05)
    p = params_of(stencil, model)
    mag = np.sqrt(2 * model.T) * np.sqrt(1 / (stencil.dt * stencil.dx * stencil.dy))
    sim = I.Integrator(field, stencil, model, seed=99)
    ref = field.copy()
    for _ in range(10):
        jr = sim.random_current
        xi = np.stack([jr[0] / mag, jr[1] / mag])[None]
        sim.run(1)
        ref = oracle.run(ref, p, 1, noise="injected", injected=xi)
        assert maxabs(sim.field - ref) / maxabs(ref) < TIGHT


def test_injected_noise_stepwise():
    """T > 0 with host-supplied standard normals: the FP64 device step matches the oracle
    step by step (amb_step_f64 with injected noise)."""
    import torch
    I = lib_integrator()
    from activemodelbplus.integrator import _native as N
    rng = np.random.default_rng(6)
    ny, nx, nsteps = 80, 64, 6
    field = -0.4 + 0.01 * rng.standard_normal((ny, nx))
    noise = rng.standard_normal((nsteps, 2, ny, nx))
    stencil, model = I.Stencil(1e-3, 1, 1), I.Model(-0.25, 0, 0.25, 1, -1, -4, 0.05)
    p = params_of(stencil, model)
    a = torch.from_numpy(field.copy()).cuda()
    b = torch.empty_like(a)
    dn = torch.from_numpy(noise).cuda()
    s, m = N.stencil_struct(stencil), N.model_struct(model)
    cur = field
    for k in range(nsteps):
        flag = ctypes.c_int(0)
        rc = N.lib().amb_step_f64(ctypes.byref(s), ctypes.byref(m), 0, ny, nx, a.data_ptr(), b.data_ptr(), k, 1,
                                  dn[k].data_ptr(), torch.cuda.current_stream().cuda_stream, ctypes.byref(flag))
        assert rc == 0 and flag.value == 1
        a, b = b, a
        cur = oracle.run(cur, p, 1, noise="injected", injected=noise[k:k + 1])
        assert maxabs(a.cpu().numpy() - cur) / maxabs(cur) < TIGHT


def test_noise_statistics_device():
    """Device normals over a 512^2 field: mean 0, variance 1, Gaussian kurtosis."""
    I = lib_integrator()
    sim = I.Integrator(np.zeros((512, 512)), I.Stencil(1e-3, 1, 1), I.Model(0, 0, 0, 0, 0, 0, 0.5), seed=3)
    mag = np.sqrt(2 * 0.5) * np.sqrt(1 / 1e-3)
    for z in sim.random_current:
        z = z / mag
        assert abs(z.mean()) < 0.01 and abs(z.var() - 1) < 0.01
        assert abs(((z - z.mean()) ** 4).mean() / z.var() ** 2 - 3) < 0.05


# ------------------------------------------------------------------ precision

@pytest.mark.parametrize("T", [0.0, 0.05])
def test_fp32_paths_track_fp64(T):
    """FP32 storage vs FP64 on AMB+ (zeta=-1, lambda=0.5), 256^2, 2000 steps, same Philox
    noise. Bounds: F32C max|d| < 2e-5, F32 max|d| < 2e-4 (the F32C residual removes the
    storage rounding that dominates plain F32 at T = 0); the F32C structure factor within 1e-4
    (relative L2 over the notebook's bins) of the FP64 one."""
    from activemodelbplus.analysis import structure_factor
    I = lib_integrator()
    rng = np.random.default_rng(8)
    field = -0.4 + 0.01 * rng.standard_normal((256, 256))
    stencil, model = I.Stencil(1e-3, 1, 1), I.Model(-0.25, 0, 0.25, 1, 0.5, -1, T)
    ref = I.Integrator(field, stencil, model, seed=5)
    ref.run(2000)
    f64 = ref.field
    errs = {}
    _, s64, _ = structure_factor(f64, phi0=-0.4)
    for precision in ("f32", "f32c"):
        sim = I.Integrator(field, stencil, model, precision=precision, seed=5)
        sim.run(2000)
        errs[precision] = maxabs(sim.field - f64)
        if precision == "f32c":
            _, s32, _ = structure_factor(sim.field, phi0=-0.4)
            m = np.isfinite(s64)
            assert np.linalg.norm(s32[m] - s64[m]) / np.linalg.norm(s64[m]) < 1e-4
    assert errs["f32c"] < 2e-5
    assert errs["f32"] < 2e-4
    if T == 0.0:
        assert errs["f32c"] < errs["f32"]


# ------------------------------------------------------------------ failures

def test_nonfinite_field_raises():
    """src/integrator.cu:524-537: a non-finite field after run raises CudaException."""
    I = lib_integrator()
    f = np.zeros((32, 32))
    f[3, 5] = np.nan
    sim = I.Integrator(f, I.Stencil(1e-3, 1, 1), I.Model(-0.25, 0, 0.25, 1, 0, 0, 0))
    with pytest.raises(I.CudaException, match="numerical error"):
        sim.run(1)
    blow = I.Integrator(np.random.default_rng(0).uniform(-1, 1, (32, 32)), I.Stencil(10.0, 1, 1),
                        I.Model(-0.25, 0, 0.25, 1, 0, 0, 0), precision="f32c")
    with pytest.raises(I.CudaException):
        blow.run(50)


def test_invalid_arguments():
    I = lib_integrator()
    with pytest.raises(TypeError):
        I.Integrator(np.zeros(16), I.Stencil(1e-3, 1, 1), I.Model())
    with pytest.raises(ValueError):
        I.Integrator(np.zeros((0, 4)), I.Stencil(1e-3, 1, 1), I.Model())
    with pytest.raises(ValueError):
        I.Integrator(np.zeros((8, 8)), I.Stencil(1e-3, 1, 1), I.Model(), precision="f16")


# ------------------------------------------------------------- handle layer + resume

def test_c_handle_layer_matches_python_layer():
    """amb_integrator_* (host buffers in/out) equals the Python Integrator."""
    I = lib_integrator()
    from activemodelbplus.integrator import _native as N
    L = N.lib()
    rng = np.random.default_rng(10)
    field = np.ascontiguousarray(rng.uniform(-0.5, 0.5, (40, 56)))
    stencil, model = I.Stencil(1e-3, 1, 1), I.Model(-0.25, 0, 0.25, 1, -1, -4, 0.02)
    for prec_name, prec in (("f64", N.AMB_F64), ("f32c", N.AMB_F32C)):
        h = ctypes.c_void_p()
        s, m = N.stencil_struct(stencil), N.model_struct(model)
        assert L.amb_integrator_create(field.ctypes.data, 40, 56, ctypes.byref(s), ctypes.byref(m), prec, 77,
                                       ctypes.byref(h)) == 0
        try:
            assert L.amb_integrator_run(h, 25) == 0
            out = np.empty_like(field)
            assert L.amb_integrator_get_field(h, out.ctypes.data) == 0
            ts = ctypes.c_int64()
            L.amb_integrator_get_timestep(h, ctypes.byref(ts))
            assert ts.value == 25
            jy, jx = np.empty_like(field), np.empty_like(field)
            assert L.amb_integrator_get_current(h, N.CURRENTS["total"], jy.ctypes.data, jx.ctypes.data) == 0
            sim = I.Integrator(field, stencil, model, precision=prec_name, seed=77)
            sim.run(25)
            assert np.array_equal(out, sim.field)
            cur = sim.current
            assert np.array_equal(jy, cur[0]) and np.array_equal(jx, cur[1])
        finally:
            L.amb_integrator_destroy(h)


@pytest.mark.parametrize("precision", ["f64", "f32c"])
def test_checkpoint_resume_is_exact(precision, tmp_path):
    I = lib_integrator()
    rng = np.random.default_rng(12)
    field = -0.4 + 0.01 * rng.standard_normal((64, 64))
    stencil, model = I.Stencil(1e-3, 1, 1), I.Model(-0.25, 0, 0.25, 1, -1, -4, 0.05)
    a = I.Integrator(field, stencil, model, precision=precision, seed=21)
    a.run(100)
    b = I.Integrator(field, stencil, model, precision=precision, seed=21)
    b.run(40)
    path = str(tmp_path / "ckpt.npz")
    b.save_checkpoint(path)
    c = I.Integrator.load_checkpoint(path)
    c.run(60)
    assert c.timestep == 100
    assert np.array_equal(a.field, c.field)


def test_run_for_time_with_interrupts():
    I = lib_integrator()
    sim = I.Integrator(np.random.default_rng(3).uniform(-0.1, 0.1, (32, 32)), I.Stencil(1e-2, 1, 1),
                       I.Model(-0.25, 0, 0.25, 1, 0, 0, 0))
    seen = []
    sim.run_for_time(1.0, t_interrupt=np.array([0.0, 0.25, 0.5, 1.0]), f_interrupt=lambda s: seen.append(s.timestep),
                     max_updates=3, min_update_time=0.1)
    assert sim.timestep == 100
    assert seen == [0, 25, 50, 100]
    with pytest.raises(ValueError):
        sim.run_for_time(0.015)


# ------------------------------------------------------------------ trajectories

@pytest.mark.parametrize("precision", ["f64", "f32c"])
@pytest.mark.parametrize("to", ["host", "device"])
def test_sample_trajectory_matches_chunked_runs(precision, to, tmp_path):
    """sample_trajectory (no host wait between samples) records exactly the fields
    that run() in the same chunks produces; the file reloads unchanged."""
    I = lib_integrator()
    from activemodelbplus.trajectory import Trajectory
    f0 = -0.4 + 0.01 * np.random.default_rng(4).standard_normal((64, 128))
    st, mo = I.Stencil(1e-3, 1, 1), I.Model(-0.25, 0, 0.25, 1, -1, -4, 0.05)
    t = np.array([0.0, 0.005, 0.005, 0.02, 0.1])
    a = I.Integrator(f0, st, mo, precision=precision, seed=5)
    a.run(10)
    tr = a.sample_trajectory(t, to=to)
    b = I.Integrator(f0, st, mo, precision=precision, seed=5)
    b.run(10)
    expect = []
    for n in np.round(t / 1e-3).astype(int):
        b.run(int(n + 10 - b.timestep))
        expect.append(b.field)
    assert a.timestep == 110
    assert np.allclose(tr.time, 0.01 + t)
    assert np.array_equal(tr.host_field(), np.asarray(expect))
    tr.save(str(tmp_path / "trajectory.npz"))
    back = Trajectory.load(str(tmp_path / "trajectory.npz"))
    assert np.array_equal(back.field, tr.host_field()) and back.model == mo and back.stencil == st


def test_sample_trajectory_rejects_and_raises():
    I = lib_integrator()
    sim = I.Integrator(np.zeros((32, 32)), I.Stencil(1e-2, 1, 1), I.Model(-0.25, 0, 0.25, 1, 0, 0, 0))
    with pytest.raises(ValueError):
        sim.sample_trajectory([0.1, 0.05])
    with pytest.raises(ValueError):
        sim.sample_trajectory([0.015])
    blow = I.Integrator(np.random.default_rng(0).uniform(-1, 1, (32, 32)), I.Stencil(10.0, 1, 1),
                        I.Model(-0.25, 0, 0.25, 1, 0, 0, 0), precision="f32c")
    with pytest.raises(I.CudaException):
        blow.sample_trajectory([10.0, 500.0])


def test_run_for_time_raises_on_nonfinite():
    I = lib_integrator()
    blow = I.Integrator(np.random.default_rng(0).uniform(-1, 1, (32, 32)), I.Stencil(10.0, 1, 1),
                        I.Model(-0.25, 0, 0.25, 1, 0, 0, 0), precision="f32c")
    with pytest.raises(I.CudaException):
        blow.run_for_time(500.0, max_updates=5, min_update_time=10.0)
