"""Learned stepper, host side, no GPU: the operand layouts the tensor-core kernels
read (chunk planes, B-operand weight images, the flipped data-gradient image,
the weight-gradient output order) checked by emulating the kernels' index
arithmetic in numpy against the FP64 oracle; and the fixed-point face update's
exact conservation."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import oracle.learned as OL
from activemodelbplus import learned as L


def emulate_conv(xc, img, npad):
    """What amb_conv5x5_forward computes, from the same buffers: input row i shifted by
    x tap kx (A operand, K-major over the channel chunks) times image[kx][chunk][s][co][e]
    (B operand, N = (s, co)) adds slice s to output row i - 4 + s, i.e. y tap ky = 4 - s."""
    xc = xc.float().numpy().astype(np.float64)      # [B, q, H, W, 8]
    im = img.float().numpy().astype(np.float64)     # [5 kx, q, 5 s, npad, 8]
    B, q, H, W, _ = xc.shape
    out = np.zeros((B, npad, H, W))
    for ky in range(5):
        for kx in range(5):
            xs = np.roll(xc, shift=(-(ky - 2), -(kx - 2)), axis=(2, 3))  # xs[r, c] = x[r+ky-2, c+kx-2]
            out += np.einsum("bqhwe,qne->bnhw", xs, im[kx][:, 4 - ky])
    return out


def emulate_row_slices(nout):
    """The forward kernel's MMA schedule for one CTA of nout output rows: input row i
    (0 <= i < nout + 4) issues slices s_lo..s_hi, slice s feeding output row i - 4 + s with
    y tap 4 - s. Returns the (output row, y tap) pairs covered."""
    seen = []
    for i in range(nout + 4):
        s_lo = 4 - i if i < 4 else 0
        s_hi = min(nout + 3 - i, 4)
        for s in range(s_lo, s_hi + 1):
            seen.append((i - 4 + s, 4 - s))
    return seen


def emulate_wgrad(xc, dzc):
    """What amb_conv5x5_wgrad computes: dw[tap][ci][co] = sum_sites x[ci][site + tap] dz[co][site]."""
    x = L.from_chunks(xc, xc.shape[1] * 8).numpy().astype(np.float64)
    dz = L.from_chunks(dzc, dzc.shape[1] * 8).numpy().astype(np.float64)
    dw = np.zeros((25, x.shape[1], dz.shape[1]))
    for ky in range(5):
        for kx in range(5):
            xs = np.roll(x, shift=(-(ky - 2), -(kx - 2)), axis=(2, 3))
            dw[ky * 5 + kx] = np.einsum("bihw,bohw->io", xs, dz)
    return torch.from_numpy(dw)


def _rand(shape, seed):
    return torch.from_numpy(np.random.default_rng(seed).standard_normal(shape))


def test_bf16_round_matches_torch():
    v = np.random.default_rng(0).standard_normal(1000) * 10.0 ** np.random.default_rng(1).integers(-5, 5, 1000)
    assert np.array_equal(OL.bf16_round(v), torch.from_numpy(v).float().to(torch.bfloat16).double().numpy())


def test_chunk_layout_round_trip():
    x = _rand((2, 5, 6, 8), 1).float()
    xc = L.to_chunks(x, 16)
    assert tuple(xc.shape) == (2, 2, 6, 8, 8) and xc.dtype == torch.bfloat16
    back = L.from_chunks(xc, 5)
    assert torch.equal(back, x.to(torch.bfloat16).float())
    assert torch.all(L.from_chunks(xc, 16)[:, 5:] == 0)


@pytest.mark.parametrize("cin_used,cin,cout,npad", [(5, 16, 32, 32), (32, 32, 32, 32), (32, 32, 2, 16), (12, 16, 7, 16)])
def test_forward_image_layout(cin_used, cin, cout, npad):
    x = _rand((2, cin_used, 7, 9), 2).float()
    w = _rand((cout, cin_used, 5, 5), 3).float()
    got = emulate_conv(L.to_chunks(x, cin), L.weight_image(w, cin, npad), npad)
    ref = OL.conv5x5(OL.bf16_round(x.numpy()), OL.bf16_round(w.numpy()))
    assert np.abs(got[:, :cout] - ref).max() < 1e-9 * max(1.0, np.abs(ref).max())
    assert np.all(got[:, cout:] == 0)


@pytest.mark.parametrize("cin,npad,cout_used", [(32, 32, 32), (32, 16, 2), (16, 32, 32)])
def test_dgrad_image_is_the_data_gradient(cin, npad, cout_used):
    """Data gradient = forward convolution of the output gradient with the flipped,
    channel-swapped image."""
    cin_used = 5 if cin == 16 else cin
    w = _rand((cout_used, cin_used, 5, 5), 4).float()
    x = _rand((2, cin_used, 6, 7), 5)
    dz = _rand((2, cout_used, 6, 7), 6).float()
    wr, dzr = OL.bf16_round(w.numpy()), OL.bf16_round(dz.numpy())
    dx_ref, _ = OL.conv5x5_grads(x.numpy(), wr, dzr)
    got = emulate_conv(L.to_chunks(dz, npad), L.dgrad_image(w, cin, npad), cin)
    assert np.abs(got[:, :cin_used] - dx_ref).max() < 1e-9 * max(1.0, np.abs(dx_ref).max())


@pytest.mark.parametrize("cin,cin_used,npad,cout", [(32, 32, 32, 32), (16, 5, 32, 32), (32, 32, 16, 2)])
def test_wgrad_output_order(cin, cin_used, npad, cout):
    x = _rand((2, cin_used, 6, 7), 7).float()
    dz = _rand((2, cout, 6, 7), 8).float()
    dw = emulate_wgrad(L.to_chunks(x, cin), L.to_chunks(dz, npad))
    got = L.wgrad_to_weights(dw, cout, cin_used).numpy()
    _, dw_ref = OL.conv5x5_grads(OL.bf16_round(x.numpy()), np.zeros((cout, cin_used, 5, 5)),
                                 OL.bf16_round(dz.numpy()))
    assert np.abs(got - dw_ref).max() < 1e-9 * max(1.0, np.abs(dw_ref).max())


@pytest.mark.parametrize("nout", [1, 2, 3, 4, 5, 7, 16])
def test_forward_slices_cover_every_tap_once(nout):
    seen = emulate_row_slices(nout)
    assert sorted(seen) == [(o, ky) for o in range(nout) for ky in range(5)]


def test_d8_face_sums_reproduce_the_central_difference():
    f = np.random.default_rng(9).standard_normal(64)
    w = OL.d8_face_weights()
    F = sum(w[i] * np.roll(f, -e) for i, e in enumerate(range(-3, 5)))  # F(j + 1/2)
    d8 = sum(c * (np.roll(f, -d) - np.roll(f, d)) for d, c in zip(range(1, 5), OL.D8))
    assert np.abs((F - np.roll(F, 1)) - d8).max() < 1e-14


def test_face_update_conserves_exactly():
    rng = np.random.default_rng(10)
    phi_q = np.rint(rng.uniform(-1, 1, (24, 40)) * OL.FIX).astype(np.int64)
    flux = rng.standard_normal((2, 24, 40)).astype(np.float32)
    xi = rng.standard_normal((2, 24, 40)).astype(np.float32)
    for kw in ({}, {"xi": xi, "noise_mag": 3.0}, {"extra": 0.5 * flux[::-1].copy()}):
        new = OL.face_update(phi_q, flux, 0.05, **kw)
        assert new.sum() == phi_q.sum()
        assert not np.array_equal(new, phi_q)


def test_network_oracle_gradients_match_finite_differences():
    """The FP64 network oracle's backward (no bf16 rounding) against central differences."""
    rng = np.random.default_rng(11)
    x = rng.standard_normal((1, 5, 6, 6))
    ws = [rng.standard_normal((4, 5, 5, 5)) * 0.1, rng.standard_normal((2, 4, 5, 5)) * 0.1]
    bs = [rng.standard_normal(4) * 0.1, rng.standard_normal(2) * 0.1]
    dflux = rng.standard_normal((1, 2, 6, 6))
    _, gw, gb = OL.fluxnet(x, ws, bs, dflux, bf16_activations=False)
    eps = 1e-6
    for l, (i, j, ky, kx) in ((0, (1, 2, 3, 4)), (1, (0, 3, 2, 2))):
        wp = [w.copy() for w in ws]
        wm = [w.copy() for w in ws]
        wp[l][i, j, ky, kx] += eps
        wm[l][i, j, ky, kx] -= eps
        fp = (OL.fluxnet(x, wp, bs, bf16_activations=False) * dflux).sum()
        fm = (OL.fluxnet(x, wm, bs, bf16_activations=False) * dflux).sum()
        assert abs((fp - fm) / (2 * eps) - gw[l][i, j, ky, kx]) < 1e-6
    bp = [b.copy() for b in bs]
    bp[0][1] += eps
    bm = [b.copy() for b in bs]
    bm[0][1] -= eps
    fd = ((OL.fluxnet(x, ws, bp, bf16_activations=False) - OL.fluxnet(x, ws, bm, bf16_activations=False))
          * dflux).sum() / (2 * eps)
    assert abs(fd - gb[0][1]) < 1e-6


@pytest.mark.parametrize("mode", [(0, 3), (5, 0), (7, 11), (31, 31), (20, 64)])
def test_linear_rate_matches_one_oracle_step(mode):
    """A small mode about the bulk state phi = 1 decays in one step of the reference scheme
    (the CPU oracle, lambda = zeta = T = 0) by exactly 1 - dt w(k) to first order."""
    import oracle
    from activemodelbplus.integrator import Model, Stencil
    H, W = 64, 128
    ky, kx = mode
    eps = 1e-6
    r, c = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    pert = np.cos(2 * np.pi * (ky * r / H + kx * c / W))
    p = oracle.Params(dt=1e-3, dx=1.0, dy=1.0, a=-0.25, b=0.0, c=0.25, kappa=1.0, lamb=0.0, zeta=0.0, T=0.0)
    after = oracle.run(1.0 + eps * pert, p, 1)
    ratio = ((after - 1.0) * pert).sum() / (eps * (pert * pert).sum())
    w = L.linear_rate((H, W), Stencil(1e-3, 1, 1), Model(-0.25, 0, 0.25, 1, 0, 0, 0))
    assert abs(ratio - (1 - 1e-3 * w[ky, kx])) < 1e-6


def test_linear_part_flux_reproduces_the_k_step_propagator():
    from activemodelbplus.integrator import Model, Stencil
    H, W, K = 32, 48, 50
    st, m = Stencil(1e-3, 1, 1), Model(-0.25, 0, 0.25, 1, 0, 0, 0)
    lin = L.LinearPart((H, W), st, m, K, device="cpu")
    phi = torch.from_numpy(np.random.default_rng(3).standard_normal((2, H, W))).float()
    g = lin.flux(phi)
    new = phi - K * st.dt * L.divergence(g, 1.0, 1.0)
    a = torch.from_numpy((1 - st.dt * L.linear_rate((H, W), st, m)) ** K).float()
    ref = torch.fft.irfft2(torch.fft.rfft2(phi) * a, s=(H, W))
    assert float((new - ref).abs().max()) < 1e-5
    assert abs(float(new.sum() - phi.sum())) < 1e-3


def test_spectral_noise_flux_equals_face_sums_of_the_filtered_draw():
    """LinearPart's noise filters (one spectral pass, as LinearPart.extra combines them on the
    GPU) equal the order-8 face sums of the noise_filter-shaped draw, component by component."""
    from activemodelbplus.integrator import Model, Stencil
    H, W, K = 32, 64, 50
    st, m = Stencil(1e-3, 1, 1), Model(-0.25, 0, 0.25, 1, 0, 0, 0.05)
    lin = L.LinearPart((H, W), st, m, K, device="cpu", with_linear=False)
    xi = torch.from_numpy(np.random.default_rng(4).standard_normal((2, H, W))).float()
    sxi = torch.fft.rfft2(xi) * 3.0
    out = torch.stack([torch.fft.irfft2(sxi[0] * lin.ny_, s=(H, W)), torch.fft.irfft2(sxi[1] * lin.nx_, s=(H, W))])
    g = L.noise_filter((H, W), st, m, K)
    shaped = torch.fft.irfft2(torch.fft.rfft2(xi) * g, s=(H, W)).numpy().astype(np.float64)
    w = OL.d8_face_weights()
    fy = sum(w[i] * np.roll(shaped[0], -e, axis=0) for i, e in enumerate(range(-3, 5))) * 3.0
    fx = sum(w[i] * np.roll(shaped[1], -e, axis=1) for i, e in enumerate(range(-3, 5))) * 3.0
    assert np.abs(out[0].numpy() - fy).max() < 1e-4
    assert np.abs(out[1].numpy() - fx).max() < 1e-4


def test_forward_staging_covers_each_window_once():
    """The forward convolution stages each 132-site window (columns c0-2 .. c0+129, periodic)
    as one in-range bulk copy plus per-site copies of the wrapped sites: an emulation of that
    index arithmetic (csrc/amb_conv.cu, conv_fwd_kernel, warp 0) reproduces the periodic window
    exactly, writes every window site once and reads only columns of the row."""
    k_tile, k_sites = 128, 132
    for ncols in (128, 256, 512, 1024):
        for c0 in range(0, ncols, k_tile):
            left = 2 if c0 == 0 else 0
            right = 2 if c0 + k_tile == ncols else 0
            lo, run = c0 - 2 + left, k_sites - left - right
            window = [None] * k_sites
            assert 0 <= lo and lo + run <= ncols
            for s in range(run):  # the bulk copy
                assert window[left + s] is None
                window[left + s] = lo + s
            for s in range(left + right):  # the wrapped sites
                at_left = s < left
                wsite = s if at_left else k_sites - right + (s - left)
                gcol = ncols - 2 + s if at_left else s - left
                assert 0 <= gcol < ncols and window[wsite] is None
                window[wsite] = gcol
            assert window == [(c0 - 2 + j) % ncols for j in range(k_sites)], (ncols, c0)


def test_spectral_combine_noise_index_map():
    """spectral_combine_noise_kernel recovers each rfft2 mode (r, k) from its memory index i for
    a row-major (ks = 1, rs = W/2+1) or column-major (rs = 1, ks = H) spectrum (csrc/amb_conv.cu):
    an emulation visits every mode exactly once, and the Hermitian partner used for the k = 0
    and Nyquist columns (r -> H - r above H/2) stays a valid row."""
    for H, W in ((8, 16), (6, 10), (5, 8), (96, 128)):
        nk = W // 2 + 1
        for rs, ks in ((nk, 1), (1, H)):
            seen = set()
            for i in range(H * nk):
                if ks == 1:
                    r, k = i // rs, i - (i // rs) * rs
                else:
                    k, r = i // ks, i - (i // ks) * ks
                assert 0 <= r < H and 0 <= k < nk
                assert r * rs + k * ks == i
                seen.add((r, k))
                herm = k == 0 or (W % 2 == 0 and k == W // 2)
                if herm and r > H // 2:
                    assert 0 < H - r < H
            assert len(seen) == H * nk


def test_adaptive_check_interval_rules():
    """The learned stepper's check cadence: doubles to the cap while residuals stay below tol/4,
    holds between tol/4 and tol/2, resets after a larger residual, a NaN or a failed check."""
    from activemodelbplus.learned import next_check_interval as nxt
    tol, base, cap = 0.5, 40, 320
    seq, iv = [], base
    for _ in range(5):
        iv = nxt(iv, 0.04, True, tol, base, cap)
        seq.append(iv)
    assert seq == [80, 160, 320, 320, 320]
    assert nxt(160, 0.2, True, tol, base, cap) == 160          # between tol/4 and tol/2: hold
    assert nxt(160, 0.3, True, tol, base, cap) == base         # above tol/2: reset
    assert nxt(160, 0.01, False, tol, base, cap) == base       # failed check: reset
    assert nxt(160, float("nan"), True, tol, base, cap) == base
    assert nxt(40, 0.0, True, tol, 40, 40) == 40               # fixed cadence when the cap is the base


def test_peak_wavenumber_recovers_a_sub_bin_maximum():
    """The sub-bin peak estimate on the notebook's bins: a smooth peak placed between bin
    centres is recovered to a small fraction of a bin, with and without 5 % bin noise; a peak at
    the first bin falls back to that bin."""
    from activemodelbplus.analysis import default_edges, peak_wavenumber
    e = default_edges()
    k = 0.5 * (e[1:] + e[:-1])
    w = k[1] - k[0]
    rng = np.random.default_rng(0)
    for k0 in (0.3137, 0.30, 0.4521):
        S = np.exp(-0.5 * ((k - k0) / 0.06) ** 2)
        assert abs(peak_wavenumber(k, S) - k0) < 0.05 * w
        noisy = S * (1 + 0.05 * rng.standard_normal(S.shape))
        assert abs(peak_wavenumber(k, noisy) - k0) < 0.5 * w
    S = np.exp(-k / 0.1)
    assert peak_wavenumber(k, S) == k[0]
