"""Learned stepper on the GPU: the tcgen05 kernels against the CPU FP64 oracle
(oracle/learned.py), the exact fixed-point update, and what training gains.

Tolerances: FP32 accumulation of <= 800 bf16 products gives ~1e-6 relative error
on FP32 outputs; bf16 outputs carry one bf16 rounding (relative 2^-8); network
gradients carry the bf16 rounding of every stored activation and gradient."""
import math

import numpy as np
import pytest

import oracle.learned as OL

pytestmark = pytest.mark.gpu


def mods():
    import torch
    from activemodelbplus import learned as L
    from activemodelbplus.integrator import _native as N
    return torch, L, N


def bf16(a):
    torch = mods()[0]
    return torch.from_numpy(np.asarray(a, dtype=np.float32)).to(torch.bfloat16).cuda()


# ------------------------------------------------------------ self-test

@pytest.mark.parametrize("a_mn,b_mn", [(0, 0), (1, 1), (0, 1), (1, 0)])
@pytest.mark.parametrize("n,k", [(32, 16), (16, 64), (32, 64)])
def test_tensor_core_selftest(a_mn, b_mn, n, k):
    """One 128 x n x k GEMM through tcgen05 with the operands in the K-major and the
    MN-major core-matrix layouts: D = A B^T to FP32 accumulation accuracy."""
    torch, L, N = mods()
    rng = np.random.default_rng(n * k + a_mn * 2 + b_mn)
    A = OL.bf16_round(rng.standard_normal((128, k)))
    B = OL.bf16_round(rng.standard_normal((n, k)))
    d = torch.zeros(128, n, dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    a_dev, b_dev = bf16(A), bf16(B)  # keep both alive until the kernel has run
    rc = N.lib().amb_tc_selftest(a_dev.data_ptr(), b_dev.data_ptr(), d.data_ptr(), n, k, a_mn, b_mn,
                                 err.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == 0, N.last_error()
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    ref = A @ B.T
    assert np.abs(d.cpu().numpy() - ref).max() < 1e-4


# ------------------------------------------------------------ convolutions

def run_conv(x, w, b, *, cin, npad, cout, epilogue, gate=None, with_pre=False):
    torch, L, N = mods()
    xc = L.to_chunks(torch.from_numpy(x).float().cuda(), cin)
    img = L.weight_image(torch.from_numpy(w).float().cuda(), cin, npad)
    bias = None
    if b is not None:
        bias = torch.zeros(npad, dtype=torch.float32, device="cuda")
        bias[: len(b)] = torch.from_numpy(np.asarray(b, dtype=np.float32)).cuda()
    B, _, H, W = x.shape
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    if epilogue == N.AMB_EPI_F32:
        out = torch.empty(B, cout, H, W, dtype=torch.float32, device="cuda")
        L.conv_forward(xc, img, bias, cin=cin, npad=npad, cout=cout, epilogue=epilogue, out_f32=out, error=err)
        torch.cuda.synchronize()
        assert int(err.item()) == 0
        return out.cpu().numpy().astype(np.float64), None
    out = torch.empty(B, npad // 8, H, W, 8, dtype=torch.bfloat16, device="cuda")
    pre = torch.empty_like(out) if with_pre else None
    g = None if gate is None else L.to_chunks(torch.from_numpy(gate).float().cuda(), npad)
    L.conv_forward(xc, img, bias, cin=cin, npad=npad, epilogue=epilogue, out=out, pre=pre, gate=g, error=err)
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    o = L.from_chunks(out, npad).cpu().numpy().astype(np.float64)
    p = None if pre is None else L.from_chunks(pre, npad).cpu().numpy().astype(np.float64)
    return o, p


SHAPES = [(2, 16, 128), (1, 20, 256), (3, 7, 128), (1, 3, 384), (1, 130, 128)]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("cin_used,cin,cout,npad", [(5, 16, 32, 32), (32, 32, 32, 32), (32, 32, 2, 16),
                                                    (16, 16, 16, 16)])
def test_conv_forward_f32(shape, cin_used, cin, cout, npad):
    B, H, W = shape
    rng = np.random.default_rng(H * W + cin + npad)
    x = OL.bf16_round(rng.standard_normal((B, cin_used, H, W)))
    w = OL.bf16_round(rng.standard_normal((cout, cin_used, 5, 5)) * 0.1)
    b = rng.standard_normal(cout).astype(np.float32)
    got, _ = run_conv(x, w, b, cin=cin, npad=npad, cout=cout, epilogue=1)
    ref = OL.conv5x5(x, w, b.astype(np.float64))
    assert np.abs(got - ref).max() < 2e-5 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("shape", [(4, 64, 512), (16, 128, 128), (1, 512, 512), (3, 45, 256)])
def test_conv_forward_multirow_ctas(shape):
    """Shapes where each CTA stages many rows (up to 16) across several 128-site windows,
    as in inference on 512 x 512 fields and training on batches of 128 x 128 fields."""
    B, H, W = shape
    rng = np.random.default_rng(B * H + W)
    x = OL.bf16_round(rng.standard_normal((B, 32, H, W)))
    w = OL.bf16_round(rng.standard_normal((32, 32, 5, 5)) * 0.05)
    b = rng.standard_normal(32).astype(np.float32)
    got, _ = run_conv(x, w, b, cin=32, npad=32, cout=32, epilogue=1)
    ref = OL.conv5x5(x, w, b.astype(np.float64))
    assert np.abs(got - ref).max() < 2e-5 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("shape", SHAPES[:3])
def test_conv_forward_gelu(shape):
    B, H, W = shape
    rng = np.random.default_rng(5)
    x = OL.bf16_round(rng.standard_normal((B, 32, H, W)))
    w = OL.bf16_round(rng.standard_normal((32, 32, 5, 5)) * 0.05)
    b = rng.standard_normal(32).astype(np.float32) * 0.1
    out, pre = run_conv(x, w, b, cin=32, npad=32, cout=32, epilogue=0, with_pre=True)
    z = OL.conv5x5(x, w, b.astype(np.float64))
    assert np.abs(pre - z).max() <= 2.0 ** -8 * np.abs(z).max() + 1e-6
    a = OL.gelu(z)
    assert np.abs(out - a).max() <= 2.0 ** -8 * np.abs(a).max() + 1e-5


@pytest.mark.parametrize("cin_fwd,npad_fwd,cout_used", [(32, 32, 32), (32, 16, 2)])
def test_conv_data_gradient(cin_fwd, npad_fwd, cout_used):
    """dgrad through the GELU of the layer below: conv of dz with the flipped, channel-swapped
    image, times gelu'(gate), against FP64 autograd."""
    torch, L, N = mods()
    rng = np.random.default_rng(cout_used)
    B, H, W = 2, 12, 128
    w = rng.standard_normal((cout_used, 32, 5, 5)) * 0.05
    dz = OL.bf16_round(rng.standard_normal((B, cout_used, H, W)))
    gate = OL.bf16_round(rng.standard_normal((B, 32, H, W)))
    wt = torch.from_numpy(w).float().cuda()
    img = L.dgrad_image(wt, cin_fwd, npad_fwd)
    dzc = L.to_chunks(torch.from_numpy(dz).float().cuda(), npad_fwd)
    gc = L.to_chunks(torch.from_numpy(gate).float().cuda(), cin_fwd)
    out = torch.empty(B, cin_fwd // 8, H, W, 8, dtype=torch.bfloat16, device="cuda")
    L.conv_forward(dzc, img, None, cin=npad_fwd, npad=cin_fwd, epilogue=N.AMB_EPI_GELU_BWD, out=out, gate=gc)
    got = L.from_chunks(out, 32).cpu().numpy().astype(np.float64)
    dx, _ = OL.conv5x5_grads(np.zeros((B, 32, H, W)), OL.bf16_round(w), dz)
    ref = dx * OL.gelu_grad(gate)
    assert np.abs(got - ref).max() <= 2.0 ** -7 * np.abs(ref).max() + 1e-6


@pytest.mark.parametrize("shape", [(2, 16, 128), (1, 13, 256), (1, 9, 384)])
@pytest.mark.parametrize("cin_used,cin,cout,npad", [(32, 32, 32, 32), (5, 16, 32, 32), (32, 32, 2, 16)])
def test_conv_weight_gradient(shape, cin_used, cin, cout, npad):
    torch, L, N = mods()
    B, H, W = shape
    rng = np.random.default_rng(H + cin + npad)
    x = OL.bf16_round(rng.standard_normal((B, cin_used, H, W)))
    dz = OL.bf16_round(rng.standard_normal((B, cout, H, W)))
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    dw = L.conv_wgrad(L.to_chunks(torch.from_numpy(x).float().cuda(), cin),
                      L.to_chunks(torch.from_numpy(dz).float().cuda(), npad), cin=cin, npad=npad, error=err)
    got = L.wgrad_to_weights(dw, cout, cin_used).cpu().numpy().astype(np.float64)
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    _, ref = OL.conv5x5_grads(x, np.zeros((cout, cin_used, 5, 5)), dz)
    assert np.abs(got - ref).max() < 2e-5 * max(1.0, np.abs(ref).max())


def test_wgrad_is_deterministic():
    torch, L, N = mods()
    rng = np.random.default_rng(3)
    x = L.to_chunks(torch.from_numpy(rng.standard_normal((4, 32, 32, 128))).float().cuda(), 32)
    dz = L.to_chunks(torch.from_numpy(rng.standard_normal((4, 32, 32, 128))).float().cuda(), 32)
    a = L.conv_wgrad(x, dz, cin=32, npad=32)
    b = L.conv_wgrad(x, dz, cin=32, npad=32)
    assert torch.equal(a, b)


# ------------------------------------------------------------ network

def test_network_forward_and_gradients_match_oracle():
    """Whole flux network, forward + backward on the device kernels vs FP64 autograd with
    the same bf16 rounding points: flux to 5e-3 relative, gradients to 3e-2 relative (L2).
    (FP32 accumulation differs from FP64 by ~1e-5 relative per layer; where that moves a value
    across a bf16 rounding boundary the stored activation differs by 2^-8 relative, and such
    flips compound over six layers to ~1e-3.)"""
    torch, L, N = mods()
    net = L.FluxNet(seed=1)
    for w in net.weights:
        w.mul_(1.5)
    net.refresh()
    rng = np.random.default_rng(4)
    B, H, W = 2, 16, 128
    phi = (-0.3 + 0.5 * rng.standard_normal((B, H, W))).astype(np.float32)
    params = np.array([[-2.0, 0.5, 0.05], [1.0, -0.7, 0.0]], dtype=np.float32)
    x = L.network_input(torch.from_numpy(phi).cuda(), torch.from_numpy(params).cuda())
    xin = OL.network_input(phi, params)
    assert np.array_equal(L.from_chunks(x, 5).cpu().numpy().astype(np.float64), OL.bf16_round(xin))
    flux = net.forward(x, train=True)
    dflux = rng.standard_normal((B, 2, H, W)).astype(np.float32)
    gw, gb = net.backward(torch.from_numpy(dflux).cuda())
    net.check_error()
    ws = [w.cpu().numpy().astype(np.float64) for w in net.weights]
    bs = [b.cpu().numpy().astype(np.float64) for b in net.biases]
    rflux, rgw, rgb = OL.fluxnet(xin, ws, bs, dflux.astype(np.float64))
    f = flux.cpu().numpy()
    assert np.linalg.norm(f - rflux) <= 5e-3 * np.linalg.norm(rflux)
    for l in range(6):
        g = gw[l].cpu().numpy()
        assert np.linalg.norm(g - rgw[l]) <= 3e-2 * np.linalg.norm(rgw[l]), l
        gbl = gb[l].cpu().numpy()[: len(rgb[l])]
        assert np.linalg.norm(gbl - rgb[l]) <= 3e-2 * np.linalg.norm(rgb[l]), l


# ------------------------------------------------------------ fixed-point update

@pytest.mark.parametrize("T,with_extra", [(0.0, False), (0.05, False), (0.0, True), (0.05, True)])
def test_update_is_exact_and_conservative(T, with_extra):
    """The fixed-point update against the float32 restatement in the oracle: bit-exact, and
    the integer mass is unchanged."""
    torch, L, N = mods()
    rng = np.random.default_rng(6)
    H, W = 48, 128
    phi_q = np.rint(rng.uniform(-0.8, 0.8, (H, W)) * OL.FIX).astype(np.int32)
    flux = (0.3 * rng.standard_normal((2, H, W))).astype(np.float32)
    extra = (0.2 * rng.standard_normal((2, H, W))).astype(np.float32) if with_extra else None
    q = torch.from_numpy(phi_q).cuda()
    f = torch.empty(H, W, dtype=torch.float32, device="cuda")
    xi = torch.empty(2, H, W, dtype=torch.float32, device="cuda")
    step = torch.tensor([7], dtype=torch.int64, device="cuda")
    flag = torch.zeros(1, dtype=torch.int32, device="cuda")
    dtk = 0.05
    flux_dev = torch.from_numpy(flux).cuda()
    extra_dev = torch.from_numpy(extra).cuda() if with_extra else None
    lib, strm = N.lib(), torch.cuda.current_stream().cuda_stream
    mag = math.sqrt(2 * T) * math.sqrt(1 / (dtk * 1.0 * 1.0))
    if T > 0:
        assert lib.amb_learned_noise(H, W, 99, step.data_ptr(), xi.data_ptr(), strm) == 0, N.last_error()
    rc = lib.amb_learned_update(flux_dev.data_ptr(), extra_dev.data_ptr() if with_extra else None, H, W, dtk, 1.0,
                                1.0, xi.data_ptr() if T > 0 else None, mag, q.data_ptr(), f.data_ptr(), 3.0,
                                flag.data_ptr(), step.data_ptr(), strm)
    assert rc == 0, N.last_error()
    got = q.cpu().numpy().astype(np.int64)
    if T > 0:
        ref = OL.face_update(phi_q, flux, dtk, xi=xi.cpu().numpy(), noise_mag=mag, extra=extra)
        import oracle
        xy, xx = oracle.normals(H, W, 99, 7)  # the same Philox-keyed normals, evaluated in double
        assert np.abs(xi.cpu().numpy() - np.stack([xy, xx])).max() < 5e-5
    else:
        ref = OL.face_update(phi_q, flux, dtk, extra=extra)
    assert np.array_equal(got, ref)
    assert got.sum() == phi_q.astype(np.int64).sum()
    assert np.array_equal(f.cpu().numpy(), (got / OL.FIX).astype(np.float32))
    assert int(flag.item()) == 0
    assert int(step.item()) == 8  # the next macro step's noise key


# ------------------------------------------------------------ stepper and training gain

def test_stepper_conserves_and_falls_back():
    """A network whose flux is far off fails the residual check, so every span is redone by
    the plain integrator; the fixed-point mass is unchanged by learned macro steps."""
    torch, L, N = mods()
    from activemodelbplus.integrator import Model, Stencil
    rng = np.random.default_rng(7)
    field = -0.4 + 0.01 * rng.standard_normal((64, 128))
    net = L.FluxNet(seed=3)
    net.weights[-1].mul_(100.0)  # a wildly wrong flux on top of the exact linear part
    net.refresh()
    st = L.LearnedStepper(net, field, Stencil(1e-3, 1, 1), Model(-0.25, 0, 0.25, 1, -1, -4, 0.0), K=50,
                          check_every=4, tol=0.05)
    m0 = st.mass_q()
    st.advance(8)
    assert st.fallback_spans == 2 and st.learned_steps == 0
    assert st.macro_steps == 8 and np.isfinite(st.field).all()
    st.tol = 1e9  # accept everything: pure learned steps, exact conservation
    m1 = st.mass_q()
    st.advance(8)
    assert st.learned_steps == 8
    assert st.mass_q() == m1
    assert abs(m1 - m0) < 64 * 128  # plain FP32 spans conserve to rounding


def test_drift_inside_a_long_span_is_rolled_back():
    """The residual check is a spot check of each span's last macro step, and a span is kept or
    redone as a whole. Here the shipped network runs until the adaptive interval has grown to its
    longest (8 macro steps); then its flux is corrupted. The next span's end check fails, the
    whole span is redone by the plain integrator (none of its learned steps survives), and the
    interval returns to the shortest."""
    import os
    torch, L, N = mods()
    from activemodelbplus.integrator import Model, Stencil
    here = os.path.dirname(L.__file__)
    net = L.FluxNet.load(os.path.join(here, "weights", "fluxnet_k50.npz"))
    field = -0.4 + 0.01 * np.random.default_rng(9).standard_normal((128, 256))
    st = L.LearnedStepper(net, field, Stencil(1e-3, 1, 1), Model(-0.25, 0, 0.25, 1, -1, -4, 0.05), K=50,
                          check_every=2, max_check_every=8, tol=1.0, residual_sigma=2.0, use_graph=False)
    st.advance(2 + 4 + 8)  # accepted spans of 2, 4 and 8 macro steps: the interval is now 8
    assert st.fallback_spans == 0 and st.learned_steps == 14 and st.interval == 8
    learned_before, state = st.learned_steps, st.phi_q.clone()
    net.weights[-1].mul_(50.0)  # the flux drifts far off from here on
    net.refresh()
    st.advance(8)
    assert st.fallback_spans == 1 and st.learned_steps == learned_before  # the span was redone
    assert st.interval == 2
    assert not torch.equal(st.phi_q, state) and np.isfinite(st.field).all()


def test_run_for_time_finishes_a_remainder_with_plain_steps():
    """t = 3 K dt + 7 dt: three macro steps, then seven Euler steps of the plain integrator; the
    clock reads t, and a t that is not a multiple of dt is refused."""
    torch, L, N = mods()
    from activemodelbplus.integrator import Model, Stencil
    field = -0.4 + 0.01 * np.random.default_rng(4).standard_normal((64, 128))
    net = L.FluxNet(seed=1)
    st = L.LearnedStepper(net, field, Stencil(1e-3, 1, 1), Model(-0.25, 0, 0.25, 1, -1, -4, 0.05), K=50,
                          check_every=10 ** 6, tol=1e9, use_graph=False)
    st.run_for_time(0.157)
    assert st.macro_steps == 3 and st.extra_steps == 7
    assert math.isclose(st.time, 0.157, rel_tol=1e-12)
    assert np.isfinite(st.field).all()
    with pytest.raises(ValueError):
        st.run_for_time(0.0005)


def test_learned_end_state_matches_plain_at_t1000():
    """The shipped K = 50 network against the plain FP32 integrator on the learned-stepper
    workload (512^2 AMB+, zeta=-4, lambda=-1, T=0.05, phi = -0.4 + 0.01 N(0,1) from numpy seed
    0, to t = 10^3), ten noise seeds per arm (the comparison `bench.py --learned` reports): the
    S(k) peak position of the learned mean (sub-bin estimate over the notebook's bins) within
    2 % of the plain mean, the droplet count within 5 %, the fixed-point mass exact in every
    run, no fallback span, and the learned runs faster. Both arms are deterministic (fixed
    Philox keys, fixed-order kernels), so the errors are those of the committed record."""
    import os
    torch, L, N = mods()
    from activemodelbplus.integrator import Model, Stencil
    here = os.path.dirname(L.__file__)
    net = L.FluxNet.load(os.path.join(here, "weights", "fluxnet_k50.npz"))
    field = -0.4 + 0.01 * np.random.default_rng(0).standard_normal((512, 512))
    res = L.compare_with_plain(net, field, Stencil(1e-3, 1, 1), Model(-0.25, 0, 0.25, 1, -1, -4, 0.05),
                               t_end=1000.0, seed=0, learned_runs=10)
    print({k: res[k] for k in ("k_peak_rel_err", "k_peak_rel_err_se", "droplets_rel_err",
                               "droplets_rel_err_se", "speedup")})
    assert abs(res["k_peak_rel_err"]) < 0.02, res["k_peak_rel_err"]
    assert abs(res["droplets_rel_err"]) < 0.05, res["droplets_rel_err"]
    assert res["learned_mass_q_drift_max"] == 0 and res["learned_fallback_spans"] == 0
    assert res["speedup"] > 1.0


def test_linear_macro_step_matches_the_propagator():
    """With a zero network flux and T = 0, a learned macro step is the linear part alone: the
    field becomes irfft2(a(k)^K phi_hat) up to the fixed-point rounding (2^-24 per face)."""
    torch, L, N = mods()
    from activemodelbplus.integrator import Model, Stencil
    H, W, K = 64, 256, 50
    st_, m = Stencil(1e-3, 1, 1), Model(-0.25, 0, 0.25, 1, 0, 0, 0.0)
    field = 0.3 * np.random.default_rng(8).standard_normal((H, W))
    net = L.FluxNet(seed=0)
    net.weights[-1].zero_()
    net.biases[-1].zero_()
    s = L.LearnedStepper(net, field, st_, m, K=K, check_every=1, tol=1e9, use_graph=False)
    start = s.field
    s._apply(noisy=False)
    a = (1 - st_.dt * L.linear_rate((H, W), st_, m)) ** K
    ref = np.fft.irfft2(np.fft.rfft2(start) * a, s=(H, W))
    assert np.abs(s.field - ref).max() < 1e-5
    assert s.mass_q() == int(np.rint(start * L.FIX).astype(np.int64).sum())


def test_training_gains_over_untrained():
    """A short training run on plain-integrator pairs: the trained flux predicts the
    deterministic 50-step increment far better than the untrained network."""
    torch, L, N = mods()
    K, dt = 50, 1e-3
    phi, delta, params, models = L.generate_pairs(48, 128, K, [2000, 6000, 12000], seed=11)
    tr = (phi[:, :40], delta[:, :40], params[:40])
    te = (phi[:, 40:], delta[:, 40:], params[40:])
    net = L.FluxNet(seed=0)
    before = L.evaluate(net, *te, K=K, dt=dt)
    L.train(net, *tr, K=K, dt=dt, iters=400, batch=8, lr=2e-3)
    after = L.evaluate(net, *te, K=K, dt=dt)
    assert after < 0.5 * before, (before, after)


def _rollout_stats(net, field, stencil, model, t_end, seeds):
    """Mean S(k) mean wavenumber and droplet count of learned rollouts (no residual checks:
    every macro step is the network's) over noise seeds."""
    from activemodelbplus import learned as L
    from activemodelbplus.analysis import count_droplets, mean_wavenumber, structure_factor
    ks, ds = [], []
    for sd in seeds:
        st = L.LearnedStepper(net, field, stencil, model, K=50, seed=sd, check_every=10 ** 6, tol=1e9)
        st.run_for_time(t_end)
        f = st.field  # fixed point: always finite (a diverging rollout saturates at the bound)
        k, S, _ = structure_factor(f, phi0=float(field.mean()))
        ks.append(mean_wavenumber(k, S))
        ds.append(count_droplets(f, float(field.mean())))
    return float(np.mean(ks)), float(np.mean(ds))


def test_trained_rollout_beats_the_linear_part_alone():
    """The method without the network is the exact linear K-step propagator alone (the
    network's flux set to zero). Rolled out to t = 200 on 256^2 AMB+ (zeta=-4, lambda=-1,
    T=0.05) without residual checks, the shipped network's end states match the plain FP32
    integrator's S(k) mean wavenumber within 5 % and are at least three times closer than the
    linear-part-only macro steps in both the mean wavenumber and the droplet count. (At this
    early, fast-coarsening time the network's droplet count runs ~25 % below the plain one;
    the statistical comparison at t = 10^3 is bench.py --learned.)"""
    import os
    torch, L, N = mods()
    from activemodelbplus.analysis import count_droplets, mean_wavenumber, structure_factor
    from activemodelbplus.integrator import Integrator, Model, Stencil
    here = os.path.dirname(L.__file__)
    net = L.FluxNet.load(os.path.join(here, "weights", "fluxnet_k50.npz"))
    zero = L.FluxNet.load(os.path.join(here, "weights", "fluxnet_k50.npz"))
    for w in zero.weights[-1:]:
        w.zero_()
    for b in zero.biases[-1:]:
        b.zero_()
    zero.refresh()
    field = -0.4 + 0.01 * np.random.default_rng(5).standard_normal((256, 256))
    stencil, model = Stencil(1e-3, 1, 1), Model(-0.25, 0, 0.25, 1, -1, -4, 0.05)
    t_end = 200.0
    pk, pd = [], []
    for sd in (1, 2):
        sim = Integrator(field, stencil, model, precision="f32", seed=sd)
        sim.run(int(round(t_end / stencil.dt)))
        f = sim.field
        k, S, _ = structure_factor(f, phi0=float(field.mean()))
        pk.append(mean_wavenumber(k, S))
        pd.append(count_droplets(f, float(field.mean())))
    plain_k, plain_d = float(np.mean(pk)), float(np.mean(pd))
    net_k, net_d = _rollout_stats(net, field, stencil, model, t_end, (0, 1))
    lin_k, lin_d = _rollout_stats(zero, field, stencil, model, t_end, (0, 1))
    err_net = abs(net_k - plain_k) / plain_k
    err_lin = abs(lin_k - plain_k) / plain_k
    derr_net = abs(net_d - plain_d) / plain_d
    derr_lin = abs(lin_d - plain_d) / plain_d
    print(f"k_avg plain {plain_k:.4f} net {net_k:.4f} linear-only {lin_k:.4f}; "
          f"droplets plain {plain_d:.1f} net {net_d:.1f} linear-only {lin_d:.1f}")
    assert err_net < 0.05, err_net
    assert err_lin > 3 * err_net and derr_lin > 3 * derr_net, (err_net, err_lin, derr_net, derr_lin)


def test_filtered_macro_noise_matches_k_plain_steps():
    """At a uniform bulk state (phi = 1, where the deterministic flux vanishes) and small T,
    the noise of one filtered macro step has the same radially binned power spectrum as K
    plain steps (within 12% per bin over 8 seeds), while the unfiltered draw overstates the
    high-wavenumber power several-fold."""
    torch, L, N = mods()
    from activemodelbplus.integrator import Integrator, Model, Stencil
    H = W = 128
    K = 50
    st = Stencil(1e-3, 1, 1)
    m = Model(-0.25, 0, 0.25, 1, 0, 0, 1e-4)
    net = L.FluxNet(seed=0)
    net.weights[-1].zero_()
    net.biases[-1].zero_()
    kk = np.hypot(*np.meshgrid(np.fft.fftfreq(H), np.fft.fftfreq(W), indexing="ij")).ravel()
    bins = np.digitize(kk, np.linspace(0, 0.71, 15))

    def spectrum(d):
        p = np.abs(np.fft.fft2(d)).ravel() ** 2
        return np.array([p[bins == b].mean() for b in range(1, 15)])

    sp_plain, sp_f, sp_s, sp_u = 0, 0, 0, 0
    for seed in range(8):
        sim = Integrator(np.ones((H, W)), st, m, precision="f64", seed=100 + seed)
        sim.run(K)
        sp_plain = sp_plain + spectrum(sim.field - 1.0)
        # filtered noise drawn as a spectrum (default), filtered noise drawn per site, unfiltered
        for filt, spec in ((True, True), (True, False), (False, True)):
            s = L.LearnedStepper(net, np.ones((H, W)), st, m, K=K, seed=200 + seed, check_every=1, tol=1e9,
                                 filter_noise=filt, spectral_noise=spec, use_graph=False)
            s.advance(1)
            d = s.field - 1.0
            if filt and spec:
                sp_f = sp_f + spectrum(d)
            elif filt:
                sp_s = sp_s + spectrum(d)
            else:
                sp_u = sp_u + spectrum(d)
    for sp in (sp_f, sp_s):
        ratio = sp / sp_plain
        assert np.all(np.abs(ratio - 1) < 0.12), ratio
    assert (sp_u / sp_plain).max() > 3, sp_u / sp_plain


def test_stepper_graph_replay_equals_eager():
    """The CUDA-graph replay of a learned macro step (with filtered noise) gives bitwise the
    state of the eager path."""
    torch, L, N = mods()
    from activemodelbplus.integrator import Model, Stencil
    field = -0.4 + 0.05 * np.random.default_rng(9).standard_normal((64, 256))
    net = L.FluxNet(seed=5)
    for w in net.weights:
        w.mul_(0.1)
    net.refresh()
    m = Model(-0.25, 0, 0.25, 1, -1, -4, 0.05)
    out = []
    for graph in (True, False):
        s = L.LearnedStepper(net, field, Stencil(1e-3, 1, 1), m, K=50, seed=3, check_every=6, tol=1e9,
                             use_graph=graph)
        s.advance(12)
        assert s.learned_steps == 12
        out.append(s.phi_q.cpu().numpy())
    assert np.array_equal(out[0], out[1])


def test_spectral_combine_kernel():
    """amb_learned_spectral_combine against torch complex arithmetic (FP32 rounding)."""
    torch, L, N = mods()
    g = torch.Generator(device="cpu").manual_seed(2)
    H, W = 64, 256
    shape = (H, W // 2 + 1)
    rnd = lambda *s_: torch.randn(*s_, generator=g, dtype=torch.complex64).cuda()
    phi, xi, my, mx, ny_, nx_ = rnd(*shape), rnd(2, *shape), rnd(*shape), rnd(*shape), rnd(*shape), rnd(*shape)
    # also a transposed (column-major) spectrum, as torch.fft may return, made contiguous by the caller
    assert torch.fft.rfft2(torch.randn(H, W, device="cuda")).contiguous().is_contiguous()
    for x_in in (xi, None):
        out = torch.empty(2, *shape, dtype=torch.complex64, device="cuda")
        rc = N.lib().amb_learned_spectral_combine(phi.data_ptr(), x_in.data_ptr() if x_in is not None else None,
                                                  my.data_ptr(), mx.data_ptr(), ny_.data_ptr(), nx_.data_ptr(), 0.7,
                                                  phi.numel(), out[0].data_ptr(), out[1].data_ptr(),
                                                  torch.cuda.current_stream().cuda_stream)
        assert rc == 0, N.last_error()
        ey, ex = phi * my, phi * mx
        if x_in is not None:
            ey, ex = ey + 0.7 * x_in[0] * ny_, ex + 0.7 * x_in[1] * nx_
        assert float((out[0] - ey).abs().max()) < 1e-5 and float((out[1] - ex).abs().max()) < 1e-5


def test_spectral_noise_is_the_spectrum_of_real_white_noise():
    """amb_learned_noise_spectral: Hermitian-consistent (a real inverse FFT and back returns it),
    unit variance per site in real space, flat mean power over modes, and keyed by the step."""
    torch, L, N = mods()
    H, W = 96, 128
    nk = W // 2 + 1
    step = torch.tensor([3], dtype=torch.int64, device="cuda")
    out = torch.empty(2, H, nk, dtype=torch.complex64, device="cuda")
    strm = torch.cuda.current_stream().cuda_stream
    assert N.lib().amb_learned_noise_spectral(H, W, 11, step.data_ptr(), out.data_ptr(), nk, 1, strm) == 0
    real = torch.fft.irfft2(out, s=(H, W))
    back = torch.fft.rfft2(real)
    assert float((back - out).abs().max()) < 1e-3 * float(out.abs().max())
    v = float(real.var())
    assert abs(v - 1.0) < 0.05, v
    p = (out.abs() ** 2).mean(dim=(0,)).cpu().numpy()
    assert abs(p[1:-1, 1:-1].mean() / (H * W) - 1) < 0.05
    out2 = torch.empty_like(out)
    step.fill_(4)
    assert N.lib().amb_learned_noise_spectral(H, W, 11, step.data_ptr(), out2.data_ptr(), nk, 1, strm) == 0
    assert not torch.equal(out, out2)


def test_spectral_combine_with_drawn_noise_matches_the_two_kernel_form():
    """amb_learned_spectral_combine_noise equals amb_learned_noise_spectral followed by
    amb_learned_spectral_combine (same draw, same arithmetic), in row- and column-major
    spectrum layouts; a layout that is not dense is rejected."""
    torch, L, N = mods()
    g = torch.Generator(device="cpu").manual_seed(5)
    H, W = 48, 256
    nk = W // 2 + 1
    strm = torch.cuda.current_stream().cuda_stream
    step = torch.tensor([17], dtype=torch.int64, device="cuda")
    for layout in ((nk, 1), (1, H)):
        n = H * nk
        mk = lambda lead=(): torch.empty_strided(lead + (H, nk), ((n,) if lead else ()) + layout,
                                                 dtype=torch.complex64, device="cuda")
        arrs = []
        for _ in range(5):
            a = mk()
            a.copy_(torch.randn(H, nk, generator=g, dtype=torch.complex64))
            arrs.append(a)
        phi, my, mx, ny_, nx_ = arrs
        xi, ref, got = mk((2,)), mk((2,)), mk((2,))
        assert N.lib().amb_learned_noise_spectral(H, W, 9, step.data_ptr(), xi.data_ptr(), layout[0], layout[1],
                                                  strm) == 0
        assert N.lib().amb_learned_spectral_combine(phi.data_ptr(), xi.data_ptr(), my.data_ptr(), mx.data_ptr(),
                                                    ny_.data_ptr(), nx_.data_ptr(), 0.3, n, ref[0].data_ptr(),
                                                    ref[1].data_ptr(), strm) == 0
        assert N.lib().amb_learned_spectral_combine_noise(phi.data_ptr(), my.data_ptr(), mx.data_ptr(),
                                                          ny_.data_ptr(), nx_.data_ptr(), 0.3, H, W, layout[0],
                                                          layout[1], 9, step.data_ptr(), got[0].data_ptr(),
                                                          got[1].data_ptr(), strm) == 0, N.last_error()
        scale = float(ref.abs().max())
        assert float((got - ref).abs().max()) <= 1e-6 * scale
    assert N.lib().amb_learned_spectral_combine_noise(phi.data_ptr(), my.data_ptr(), mx.data_ptr(), ny_.data_ptr(),
                                                      nx_.data_ptr(), 0.3, H, W, 2 * nk, 1, 9, step.data_ptr(),
                                                      got[0].data_ptr(), got[1].data_ptr(), strm) != 0


def test_update_writes_the_next_network_input():
    """amb_learned_update_input leaves in the stepper's input buffer exactly what
    amb_learned_input makes from the updated field (eager and graph-replayed macro steps,
    and after a fallback span)."""
    torch, L, N = mods()
    from activemodelbplus.integrator import Model, Stencil
    field = -0.4 + 0.05 * np.random.default_rng(4).standard_normal((64, 256))
    net = L.FluxNet(seed=6)
    for w in net.weights:
        w.mul_(0.1)
    net.refresh()
    m = Model(-0.25, 0, 0.25, 1, -1, -4, 0.05)
    for graph in (False, True):
        s = L.LearnedStepper(net, field, Stencil(1e-3, 1, 1), m, K=50, seed=2, check_every=3, tol=1e9,
                             use_graph=graph)
        s.advance(5)
        ref = L.network_input(s.phi_f.unsqueeze(0), s.params)
        assert torch.equal(s._x.view(torch.int16), ref.view(torch.int16))
    s.tol = -1.0  # every check fails: the span is redone by the plain integrator
    s.advance(3)
    assert s.fallback_spans >= 1
    ref = L.network_input(s.phi_f.unsqueeze(0), s.params)
    assert torch.equal(s._x.view(torch.int16), ref.view(torch.int16))


def test_learned_fft_plans_match_torch_fft():
    """amb_learned_fft_forward equals torch's rfft2; amb_learned_fft_inverse2 is the
    unnormalised inverse of two spectra at once (FP32 rounding)."""
    import ctypes
    torch, L, N = mods()
    H, W = 96, 256
    lib = N.lib()
    h = ctypes.c_void_p()
    assert lib.amb_learned_fft_create(H, W, ctypes.byref(h)) == 0, N.last_error()
    try:
        strm = torch.cuda.current_stream().cuda_stream
        g = torch.Generator(device="cpu").manual_seed(3)
        phi = torch.randn(H, W, generator=g).cuda()
        spec = torch.empty(H, W // 2 + 1, dtype=torch.complex64, device="cuda")
        assert lib.amb_learned_fft_forward(h, phi.data_ptr(), spec.data_ptr(), strm) == 0
        ref = torch.fft.rfft2(phi)
        assert float((spec - ref).abs().max()) < 1e-4 * float(ref.abs().max())
        two = torch.randn(2, H, W, generator=g).cuda()
        spectra = torch.fft.rfft2(two).contiguous()
        out = torch.empty(2, H, W, device="cuda")
        assert lib.amb_learned_fft_inverse2(h, spectra.data_ptr(), out.data_ptr(), strm) == 0
        assert float((out / (H * W) - two).abs().max()) < 1e-5
    finally:
        lib.amb_learned_fft_destroy(h)
    assert lib.amb_learned_fft_create(1, W, ctypes.byref(h)) != 0
