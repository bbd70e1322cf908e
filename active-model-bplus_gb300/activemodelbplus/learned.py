"""Learned coarse stepper (no reference counterpart).

A periodic convolutional network maps (phi, zeta, lambda, T) to a face flux F
that, added to the exact flux of the scheme's stiff linear part (``LinearPart``,
the K-step propagator of the scheme linearised about the bulk, applied with FFTs),
advances the field by K explicit-Euler steps at once:

    phi(t + K dt) = phi(t) - K dt * div F  (+ the K-step noise flux when T > 0)

Because the update is a difference of face fluxes, applied in int32 fixed point
(phi * 2^24) with each face rounded once, the sum of the field is conserved
exactly. The network is 6 circular 5x5 convolutions, 32 channels, GELU (tanh form), BF16
weights and activations with FP32 accumulation; its forward and both backward
passes run on this package's own tcgen05 implicit-GEMM kernels
(``amb_conv5x5_forward`` / ``amb_conv5x5_wgrad``). Training targets are the
deterministic K-step increments of the plain integrator started from states of
noisy trajectories; the noise of a macro step is one Philox draw, made directly
as its Fourier spectrum and shaped per mode by the K-step accumulation of the
linearised plain scheme (``noise_filter``). The plain integrator is the fallback:
at the end of each span of macro steps one step is compared with K plain
deterministic steps from the same state, and if the residual exceeds ``tol`` (or
the field left its bounds) the span is redone with the plain integrator. Spans
start at ``check_every`` macro steps and double, up to ``max_check_every``, while
the residuals stay below tol/4.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from .integrator import _native as N
from .integrator import CudaException, Ensemble, Integrator, Model, Stencil, _check

CIN0 = 16      # input channels as stored (5 used: phi hi, phi lo, zeta/4, lambda, 10 T)
CIN0_USED = 5
HIDDEN = 32
NOUT = 2       # flux components (y face, x face)
NOUT_PAD = 16
NLAYERS = 6
FIX = float(1 << 24)


def _torch():
    import torch
    return torch


def _stream() -> int:
    return _torch().cuda.current_stream().cuda_stream


def _ptr(t):
    return None if t is None else t.data_ptr()


# ------------------------------------------------------------------ layouts

def to_chunks(x, cpad: int):
    """[B, C, H, W] float -> bf16 chunk planes [B, cpad/8, H, W, 8] (channels >= C zero)."""
    torch = _torch()
    B, C, H, W = x.shape
    if C < cpad:
        x = torch.nn.functional.pad(x, (0, 0, 0, 0, 0, cpad - C))
    return x.reshape(B, cpad // 8, 8, H, W).permute(0, 1, 3, 4, 2).contiguous().to(torch.bfloat16)


def from_chunks(xc, c: int):
    """bf16 chunk planes [B, q, H, W, 8] -> float32 [B, c, H, W]."""
    B, q, H, W, _ = xc.shape
    return xc.permute(0, 1, 4, 2, 3).reshape(B, q * 8, H, W)[:, :c].float()


def weight_image(w, cin_pad: int, npad: int):
    """Convolution weights [cout, cin, 5, 5] (ky, kx) -> the kernels' bf16 B-operand image
    [5 kx][cin_pad/8][5 (4 - ky)][npad][8] (zero padded): for each x tap and channel chunk,
    the five y taps stacked along N in reverse order."""
    torch = _torch()
    cout, cin = w.shape[:2]
    wp = torch.zeros(npad, cin_pad, 5, 5, dtype=torch.float32, device=w.device)
    wp[:cout, :cin] = w
    img = wp.reshape(npad, cin_pad // 8, 8, 5, 5).flip(3).permute(4, 1, 3, 0, 2).contiguous()
    return img.to(torch.bfloat16)


def dgrad_image(w, cin_pad: int, npad: int):
    """B-operand image of the data gradient of a convolution with weights w [cout, cin, 5, 5]:
    the forward convolution with the kernel flipped and the channel roles swapped. The
    result convolves an npad-channel gradient into cin_pad channels."""
    return weight_image(w.flip(2, 3).transpose(0, 1), npad, cin_pad)


def wgrad_to_weights(dw, cout: int, cin: int):
    """Kernel output [25][cin_pad][npad] -> [cout, cin, 5, 5]."""
    cin_pad, npad = dw.shape[1], dw.shape[2]
    return dw.reshape(5, 5, cin_pad, npad).permute(3, 2, 0, 1)[:cout, :cin].contiguous()


# --------------------------------------------------------------- kernels

def conv_forward(x, wimg, bias, *, cin: int, npad: int, epilogue: int, cout: int | None = None, out=None,
                 pre=None, gate=None, out_f32=None, error=None):
    """One circular 5x5 convolution on the tensor cores (``amb_conv5x5_forward``)."""
    B, q, H, W, e = x.shape
    if q * 8 != cin or e != 8:
        raise ValueError("input is not in chunk-plane layout with cin channels")
    _check(N.lib().amb_conv5x5_forward(_ptr(x), B, H, W, cin, _ptr(wimg), _ptr(bias), npad,
                                       npad if cout is None else cout, epilogue, _ptr(out), _ptr(pre), _ptr(gate),
                                       _ptr(out_f32), _ptr(error), _stream()))


class _Scratch:
    def __init__(self):
        self.buf = None

    def get(self, nbytes: int, device):
        torch = _torch()
        n = (nbytes + 3) // 4
        if self.buf is None or self.buf.numel() < n:
            self.buf = torch.empty(max(n, 1), dtype=torch.float32, device=device)
        return self.buf


_WGRAD_SCRATCH = _Scratch()


def conv_wgrad(x, dz, *, cin: int, npad: int, error=None):
    """Weight gradient [25][cin][npad] FP32 (``amb_conv5x5_wgrad``)."""
    torch = _torch()
    B, _, H, W, _ = x.shape
    lib = N.lib()
    nbytes = lib.amb_conv5x5_wgrad_scratch_bytes(B, H, W, cin, npad)
    scratch = _WGRAD_SCRATCH.get(nbytes, x.device)
    dw = torch.empty(25, cin, npad, dtype=torch.float32, device=x.device)
    _check(lib.amb_conv5x5_wgrad(_ptr(x), _ptr(dz), B, H, W, cin, npad, _ptr(dw), _ptr(scratch),
                                 scratch.numel() * 4, _ptr(error), _stream()))
    return dw


def network_input(phi, params):
    """phi [B, H, W] FP32, params [B, 3] (zeta, lambda, T) -> bf16 chunk planes [B, 2, H, W, 8]."""
    torch = _torch()
    B, H, W = phi.shape
    x = torch.empty(B, 2, H, W, 8, dtype=torch.bfloat16, device=phi.device)
    _check(N.lib().amb_learned_input(_ptr(phi), _ptr(params), B, H, W, _ptr(x), _stream()))
    return x


def divergence(flux, dx: float, dy: float):
    """Face divergence (F_x(r,c) - F_x(r,c-1))/dx + (F_y(r,c) - F_y(r-1,c))/dy of flux [B, 2, H, W]."""
    torch = _torch()
    fy, fx = flux[:, 0], flux[:, 1]
    return (fx - torch.roll(fx, 1, dims=-1)) / dx + (fy - torch.roll(fy, 1, dims=-2)) / dy


# --------------------------------------------------------------- network

class FluxNet:
    """``layers`` circular 5x5 convolutions (default 6: 5 -> 32 -> 32 -> 32 -> 32 -> 32 -> 2),
    GELU between layers, BF16 weights/activations, FP32 accumulation and FP32 master weights."""

    def __init__(self, device=None, seed: int = 0, layers: int = NLAYERS):
        torch = _torch()
        device = torch.device("cuda") if device is None else torch.device(device)
        g = torch.Generator().manual_seed(int(seed))
        if int(layers) < 2:
            raise ValueError("a FluxNet has at least two layers")
        self.device = device
        self.nlayers = nl = int(layers)
        self.cin = [CIN0] + [HIDDEN] * (nl - 1)
        self.cin_used = [CIN0_USED] + [HIDDEN] * (nl - 1)
        self.cout = [HIDDEN] * (nl - 1) + [NOUT]
        self.npad = [HIDDEN] * (nl - 1) + [NOUT_PAD]
        self.weights, self.biases = [], []
        for l in range(nl):
            fan_in = 25 * self.cin_used[l]
            std = math.sqrt(2.0 / fan_in) if l < nl - 1 else 0.1 / math.sqrt(fan_in)
            self.weights.append((torch.randn(self.cout[l], self.cin_used[l], 5, 5, generator=g) * std).to(device))
            self.biases.append(torch.zeros(self.npad[l], device=device))
        self.error = torch.zeros(1, dtype=torch.int32, device=device)
        self.linear_split = True  # the network predicts the flux beyond the exact linear part
        self._images = None
        self._dimages = None
        self._saved = None

    # -- parameters
    def parameters(self):
        return self.weights + self.biases

    def refresh(self) -> None:
        """Rebuild the bf16 operand images after the FP32 weights changed."""
        self._images = [weight_image(w, self.cin[l], self.npad[l]) for l, w in enumerate(self.weights)]
        self._dimages = [None] + [dgrad_image(self.weights[l], self.cin[l], self.npad[l])
                                  for l in range(1, self.nlayers)]

    def state_dict(self) -> dict:
        d = {}
        for l in range(self.nlayers):
            d[f"w{l}"] = self.weights[l].cpu().numpy()
            d[f"b{l}"] = self.biases[l].cpu().numpy()
        d["linear_split"] = np.asarray(int(self.linear_split))
        return d

    def load_state_dict(self, d) -> None:
        torch = _torch()
        for l in range(self.nlayers):
            self.weights[l] = torch.as_tensor(np.asarray(d[f"w{l}"]), dtype=torch.float32).to(self.device)
            self.biases[l] = torch.as_tensor(np.asarray(d[f"b{l}"]), dtype=torch.float32).to(self.device)
        self.linear_split = bool(int(np.asarray(d["linear_split"]))) if "linear_split" in d else False
        self._images = None

    def save(self, path: str, **meta) -> None:
        np.savez(path, **self.state_dict(), **{k: np.asarray(v) for k, v in meta.items()})

    @classmethod
    def load(cls, path: str, device=None) -> "FluxNet":
        z = np.load(path, allow_pickle=False)
        layers = sum(1 for k in z.files if k[:1] == "w" and k[1:].isdigit())
        net = cls(device=device, layers=layers)
        net.load_state_dict({k: z[k] for k in z.files})
        net.K = int(z["K"]) if "K" in z.files else 50
        return net

    # -- passes
    def forward(self, x, *, train: bool = False):
        """x: network input chunk planes [B, 2, H, W, 8] -> flux [B, 2, H, W] FP32."""
        torch = _torch()
        if self._images is None:
            self.refresh()
        B, _, H, W, _ = x.shape
        a = x
        inputs, pres = [], []
        for l in range(self.nlayers - 1):
            out = torch.empty(B, self.npad[l] // 8, H, W, 8, dtype=torch.bfloat16, device=x.device)
            pre = torch.empty_like(out) if train else None
            conv_forward(a, self._images[l], self.biases[l], cin=self.cin[l], npad=self.npad[l],
                         epilogue=N.AMB_EPI_GELU, out=out, pre=pre, error=self.error)
            if train:
                inputs.append(a)
                pres.append(pre)
            a = out
        flux = torch.empty(B, NOUT, H, W, dtype=torch.float32, device=x.device)
        conv_forward(a, self._images[-1], self.biases[-1], cin=self.cin[-1], npad=self.npad[-1], cout=NOUT,
                     epilogue=N.AMB_EPI_F32, out_f32=flux, error=self.error)
        if train:
            inputs.append(a)
            self._saved = (inputs, pres)
        return flux

    def backward(self, dflux):
        """Gradients of the weights and biases for dL/dflux (after ``forward(train=True)``)."""
        torch = _torch()
        if self._saved is None:
            raise RuntimeError("backward() needs a preceding forward(train=True)")
        inputs, pres = self._saved
        gw, gb = [None] * self.nlayers, [None] * self.nlayers
        dz = to_chunks(dflux, NOUT_PAD)
        L = self.nlayers - 1
        gw[L] = wgrad_to_weights(conv_wgrad(inputs[L], dz, cin=self.cin[L], npad=self.npad[L], error=self.error),
                                 self.cout[L], self.cin_used[L])
        gb[L] = torch.nn.functional.pad(dflux.sum(dim=(0, 2, 3)), (0, NOUT_PAD - NOUT))
        B, _, H, W, _ = dz.shape
        for l in range(L, 0, -1):
            prev = torch.empty(B, self.cin[l] // 8, H, W, 8, dtype=torch.bfloat16, device=dz.device)
            conv_forward(dz, self._dimages[l], None, cin=self.npad[l], npad=self.cin[l],
                         epilogue=N.AMB_EPI_GELU_BWD, out=prev, gate=pres[l - 1], error=self.error)
            dz = prev
            k = l - 1
            gw[k] = wgrad_to_weights(conv_wgrad(inputs[k], dz, cin=self.cin[k], npad=self.npad[k],
                                                error=self.error), self.cout[k], self.cin_used[k])
            gb[k] = from_chunks(dz, self.npad[k]).sum(dim=(0, 2, 3))
        self._saved = None
        return gw, gb

    def check_error(self) -> None:
        """Raise if a kernel gave up waiting on its own pipeline since the last check."""
        code = int(self.error.item())
        if code:
            self.error.zero_()
            raise CudaException(f"a convolution kernel stopped early (code {code})")


# ------------------------------------------------------------- training

def model_params_tensor(models, device):
    torch = _torch()
    return torch.tensor([[m.zeta, m.lamb, m.T] for m in models], dtype=torch.float32, device=device)


def generate_pairs(n_traj: int, size: int, K, sample_steps, *, dt: float = 1e-3, seed: int = 0,
                   graph_steps: int = 50):
    """Training pairs from the plain integrator.

    ``n_traj`` noisy trajectories of size x size with parameters drawn uniformly from
    zeta in [-4, 4], lambda in [-1, 1], phi0 in [-0.6, 0.6], T in [0, 0.1] (a = -0.25,
    b = 0, c = 0.25, kappa = 1) and initial fields phi0 + 0.01 N(0, 1), advanced as one
    batched ensemble. At each sample step the states are copied into a second, noiseless
    ensemble with the same (zeta, lambda) that runs K steps: the pair is (state, its
    deterministic K-step increment). Returns device tensors phi [S, n, H, W],
    delta [S, n, H, W] and params [n, 3], and the model list. K may be a list of
    increasing step counts; delta is then a dict {K: [S, n, H, W]} (one noiseless run
    per sample, read at each K).
    """
    torch = _torch()
    rng = np.random.default_rng(seed)
    zeta = rng.uniform(-4, 4, n_traj)
    lamb = rng.uniform(-1, 1, n_traj)
    phi0 = rng.uniform(-0.6, 0.6, n_traj)
    temp = rng.uniform(0, 0.1, n_traj)
    models = [Model(a=-0.25, b=0, c=0.25, kappa=1, lamb=float(l), zeta=float(z), T=float(t))
              for z, l, t in zip(zeta, lamb, temp)]
    quiet = [Model(a=-0.25, b=0, c=0.25, kappa=1, lamb=float(l), zeta=float(z), T=0.0) for z, l in zip(zeta, lamb)]
    fields = [p0 + 0.01 * rng.standard_normal((size, size)) for p0 in phi0]
    stencil = Stencil(dt=dt, dx=1, dy=1)
    seeds = rng.integers(0, 2**63, n_traj)
    noisy = Ensemble(fields, stencil, models, precision="f32c", seeds=seeds, graph_steps=graph_steps)
    det = Ensemble(fields, stencil, quiet, precision="f32c", seeds=seeds, graph_steps=graph_steps)
    S = len(sample_steps)
    Ks = sorted(int(k) for k in (K if isinstance(K, (list, tuple)) else [K]))
    phi = torch.empty(S, n_traj, size, size, dtype=torch.float32, device="cuda")
    deltas = {k: torch.empty_like(phi) for k in Ks}
    done = 0
    for s, st in enumerate(sample_steps):
        noisy.run(int(st) - done)
        done = int(st)
        x = noisy.gather(phi[s].reshape(-1))
        det.scatter(x)
        ran = 0
        for k in Ks:
            det.run(k - ran)
            ran = k
            det.gather(deltas[k][s].reshape(-1))
            deltas[k][s].sub_(phi[s])
    noisy.close()
    det.close()
    delta = deltas if isinstance(K, (list, tuple)) else deltas[Ks[0]]
    return phi, delta, model_params_tensor(models, "cuda"), models


def lowpass_weights(shape, sigma: float, device=None):
    """Gaussian low-pass exp(-sigma^2 |k|^2 / 2) per rfft2 mode (k in radians per site)."""
    torch = _torch()
    ny, nx = shape
    ky = 2 * np.pi * np.fft.fftfreq(ny)[:, None]
    kx = 2 * np.pi * np.fft.rfftfreq(nx)[None, :]
    w = np.exp(-0.5 * sigma * sigma * (kx * kx + ky * ky)).astype(np.float32)
    return torch.from_numpy(w).to(device if device is not None else "cuda")


def lowpass(x, w):
    """Apply rfft2-layout weights w to the last two dimensions of x (cuFFT through torch)."""
    torch = _torch()
    return torch.fft.irfft2(torch.fft.rfft2(x) * w, s=x.shape[-2:])


def train(net: FluxNet, phi, delta, params, *, K: int, dt: float, iters: int, batch: int = 16, lr: float = 2e-3,
          seed: int = 0, log_every: int = 0, lowpass_sigma: float = 0.0, highpass_weight: float = 1.0,
          linear: LinearPart | None = None):
    """Fit the flux so that -K dt div F matches the deterministic K-step increments.

    phi, delta: [S, n, H, W]; params: [n, 3]. Adam on the FP32 master weights; the
    gradients come from the network's own backward kernels. With lowpass_sigma > 0 the
    loss is the relative mean-square error of the Gaussian-low-passed increments (the
    slow, large-scale dynamics that set domain sizes) plus highpass_weight times the plain
    relative MSE; otherwise the plain relative MSE. With ``linear`` (and net.linear_split)
    the predicted increment is that of the network's flux plus the exact linear part's.
    Returns the loss history.
    """
    torch = _torch()
    S, n, H, W = phi.shape
    g = torch.Generator(device="cpu").manual_seed(int(seed))
    params_list = net.parameters()
    for p in params_list:
        p.requires_grad_(False)
    opt = torch.optim.Adam(params_list, lr=lr)
    sched = torch.optim.lr_scheduler.CosineAnnealingLR(opt, T_max=max(1, iters), eta_min=lr * 0.05)
    dtk = K * dt
    scale = float(delta.square().mean().item()) + 1e-30
    wlp = lowpass_weights((H, W), lowpass_sigma, phi.device) if lowpass_sigma > 0 else None
    scale_lp = 1.0
    if wlp is not None:
        scale_lp = sum(float(lowpass(delta[k], wlp).square().mean().item()) for k in range(S)) / S + 1e-30
    hist = []
    for it in range(iters):
        si = torch.randint(0, S, (batch,), generator=g).to(phi.device)
        ni = torch.randint(0, n, (batch,), generator=g).to(phi.device)
        x = network_input(phi[si, ni].contiguous(), params[ni].contiguous())
        flux = net.forward(x, train=True)
        f = flux.detach().requires_grad_(True)
        total = f if linear is None else f + linear.flux(phi[si, ni])
        r = -dtk * divergence(total, 1.0, 1.0) - delta[si, ni]
        if wlp is None:
            loss = r.square().mean() / scale
        else:
            loss = lowpass(r, wlp).square().mean() / scale_lp + highpass_weight * r.square().mean() / scale
        loss.backward()
        gw, gb = net.backward(f.grad)
        for p, gr in zip(params_list, gw + gb):
            p.grad = gr
        opt.step()
        sched.step()
        net.refresh()
        if log_every and (it % log_every == 0 or it == iters - 1):
            hist.append((it, float(loss.item())))
    net.check_error()
    return hist


def evaluate(net: FluxNet, phi, delta, params, *, K: int, dt: float, batch: int = 16, lowpass_sigma: float = 0.0,
             linear: LinearPart | None = None):
    """Relative mean-square error of the predicted K-step increments over a pair set
    (of their Gaussian low-passed versions when lowpass_sigma > 0)."""
    S, n, H, W = phi.shape
    wlp = lowpass_weights((H, W), lowpass_sigma, phi.device) if lowpass_sigma > 0 else None
    num, den = 0.0, 0.0
    flat_phi = phi.reshape(S * n, H, W)
    flat_delta = delta.reshape(S * n, H, W)
    flat_params = params.repeat(S, 1)
    for i in range(0, S * n, batch):
        x = network_input(flat_phi[i:i + batch].contiguous(), flat_params[i:i + batch].contiguous())
        flux = net.forward(x)
        if linear is not None:
            flux = flux + linear.flux(flat_phi[i:i + batch])
        pred = -K * dt * divergence(flux, 1.0, 1.0)
        ref = flat_delta[i:i + batch]
        if wlp is not None:
            pred, ref = lowpass(pred, wlp), lowpass(ref, wlp)
        num += float((pred - ref).square().sum().item())
        den += float(ref.square().sum().item())
    return num / max(den, 1e-30)


# -------------------------------------------------------------- stepper

def bulk_curvature(model) -> float:
    """f''(phi) in the bulk phases: -2a for the symmetric double well a < 0 < c (b = 0), else a."""
    m = Model(model)
    return -2.0 * m.a if (m.a < 0 and m.c > 0) else m.a


def linear_rate(shape, stencil, model, curvature: float | None = None) -> np.ndarray:
    """Decay rate w(k) (rfft2 layout [ny, nx//2 + 1]) of the plain scheme linearised about a
    uniform state with free-energy curvature f'': w = (s_x^2 + s_y^2)(f'' - kappa L(k)), with s
    the symbol of the order-8 first derivative and L that of the Tjhung Laplacian."""
    ny, nx = shape
    st, m = Stencil(stencil), Model(model)
    f2 = bulk_curvature(m) if curvature is None else curvature
    ty = 2 * np.pi * np.fft.fftfreq(ny)[:, None]
    tx = 2 * np.pi * np.fft.rfftfreq(nx)[None, :]
    c = (4.0 / 5.0, -1.0 / 5.0, 4.0 / 105.0, -1.0 / 280.0)
    sx = (2.0 / st.dx) * sum(cd * np.sin((d + 1) * tx) for d, cd in enumerate(c))
    sy = (2.0 / st.dy) * sum(cd * np.sin((d + 1) * ty) for d, cd in enumerate(c))
    lap = ((1.5 - 0.5 * np.cos(ty)) * (2 * np.cos(tx) - 2) / st.dx ** 2 +
           (1.5 - 0.5 * np.cos(tx)) * (2 * np.cos(ty) - 2) / st.dy ** 2)
    return (sx ** 2 + sy ** 2) * (f2 - m.kappa * lap)


def noise_filter(shape, stencil, model, K: int, curvature: float | None = None):
    """Per-mode amplitude factor g(k) (rfft2 layout) that turns one draw of the K-step noise
    flux into the noise the linearised plain scheme accumulates over K steps: one step maps
    a mode by a(k) = 1 - dt w(k), so K steps of independent noise add sum_j a^(2j) =
    (1 - a^(2K)) / (1 - a^2) times the one-step variance, where a single macro draw adds K
    times it: g^2 = (1 - a^(2K)) / (K (1 - a^2))."""
    torch = _torch()
    a = 1.0 - Stencil(stencil).dt * linear_rate(shape, stencil, model, curvature)
    one_minus = 1.0 - a * a
    with np.errstate(divide="ignore", invalid="ignore"):
        g2 = np.where(np.abs(one_minus) > 1e-12, (1.0 - a ** (2 * K)) / (K * one_minus), 1.0)
    return torch.from_numpy(np.sqrt(np.clip(g2, 0.0, None)).astype(np.float32))


class LinearPart:
    """The stiff linear part of K plain steps, applied exactly and written as a face flux,
    and the K-step noise as a face flux.

    K explicit steps of the scheme linearised about the bulk multiply mode k by
    E(k) = a(k)^K. The face flux G with (face-difference) divergence
    div G = -(E - 1) phi / (K dt) is G_hat = -(E - 1) phi_hat conj(d) / (|d_x|^2 + |d_y|^2) / (K dt)
    per component, d_x = (1 - exp(-i k_x dx)) / dx the symbol of the face difference (zero
    at k = 0, where E = 1). Adding G to the network's flux makes a macro step propagate the
    linear part exactly (in particular the fast decay of short-wavelength fluctuations), and,
    as a flux, it keeps the fixed-point update exactly conservative.

    The noise of a macro step is noise_mag * W8 (g * xi) per component: one Philox draw xi,
    shaped by the noise_filter g and turned into face fluxes by the order-8 face sums W8 (the
    D8 derivative of the plain scheme's noise as a face difference). Both are linear filters,
    so ``extra`` forms linear part + noise with one inverse FFT per component (cuFFT through
    torch). ``with_linear=False`` keeps only the noise.
    """

    def __init__(self, shape, stencil, model, K: int, device=None, curvature: float | None = None,
                 with_linear: bool = True):
        torch = _torch()
        st = Stencil(stencil)
        ny, nx = shape
        self.shape = (ny, nx)
        a = 1.0 - st.dt * linear_rate(shape, st, model, curvature)
        e1 = (a ** K - 1.0) if with_linear else np.zeros_like(a)
        ty = 2 * np.pi * np.fft.fftfreq(ny)[:, None]
        tx = 2 * np.pi * np.fft.rfftfreq(nx)[None, :]
        dxs = (1.0 - np.exp(-1j * tx)) / st.dx
        dys = (1.0 - np.exp(-1j * ty)) / st.dy
        den = np.abs(dxs) ** 2 + np.abs(dys) ** 2
        den[0, 0] = 1.0
        dtk = K * st.dt
        mx = -e1 * np.conj(dxs) / den / dtk
        my = -e1 * np.conj(dys) / den / dtk
        mx[0, 0] = 0.0
        my[0, 0] = 0.0
        g = noise_filter(shape, st, model, K, curvature).numpy().astype(np.float64)
        c = (4.0 / 5.0, -1.0 / 5.0, 4.0 / 105.0, -1.0 / 280.0)
        w8 = [sum(c[d - 1] for d in range(max(e, 1 - e), 5)) for e in range(-3, 5)]
        # F(j + 1/2) = sum_e w_e xi(j + e)  <->  F_hat = xi_hat * sum_e w_e exp(i k e)
        sym_x = sum(w * np.exp(1j * tx * e) for w, e in zip(w8, range(-3, 5)))
        sym_y = sum(w * np.exp(1j * ty * e) for w, e in zip(w8, range(-3, 5)))
        dev = device if device is not None else "cuda"
        full = (ny, nx // 2 + 1)
        self.my = torch.from_numpy(np.broadcast_to(my, full).astype(np.complex64)).to(dev)
        self.mx = torch.from_numpy(np.broadcast_to(mx, full).astype(np.complex64)).to(dev)
        self.ny_ = torch.from_numpy(np.broadcast_to(g * sym_y, full).astype(np.complex64)).to(dev)
        self.nx_ = torch.from_numpy(np.broadcast_to(g * sym_x, full).astype(np.complex64)).to(dev)
        self._layout = None
        self._filters = None
        self._fft = None

    def flux(self, phi):
        """Linear part only: phi [B, H, W] -> G [B, 2, H, W] (component 0 = y face, 1 = x face)."""
        torch = _torch()
        spec = torch.fft.rfft2(phi)
        gy = torch.fft.irfft2(spec * self.my, s=self.shape)
        gx = torch.fft.irfft2(spec * self.mx, s=self.shape)
        return torch.stack([gy, gx], dim=1)

    def _extra_direct(self, phi, noise_mag: float, out, spectral_noise):
        """extra() without a per-site noise field, on the library's own cuFFT plans
        (``amb_learned_fft_*``): one forward transform, the combining kernel (noise drawn in it
        when ``spectral_noise`` is given), one batched inverse into ``out``; the spectra live in
        buffers made on the first call, so later calls can be captured in a CUDA graph."""
        torch = _torch()
        lib = N.lib()
        ny, nx = self.shape
        nk = nx // 2 + 1
        if self._fft is None:
            h = ctypes.c_void_p()
            _check(lib.amb_learned_fft_create(ny, nx, ctypes.byref(h)))
            self._fft = h
            self._spec = torch.empty(ny, nk, dtype=torch.complex64, device=phi.device)
            self._comb = torch.empty(2, ny, nk, dtype=torch.complex64, device=phi.device)
            inv_n = 1.0 / (ny * nx)  # the inverse transform is unnormalised
            self._filters_rm = [(f * inv_n).contiguous() for f in (self.my, self.mx, self.ny_, self.nx_)]
        if not (phi.is_contiguous() and out.is_contiguous() and phi.dtype == torch.float32
                and out.dtype == torch.float32 and tuple(out.shape) == (2, ny, nx)):
            raise ValueError("LinearPart.extra: phi [H, W] and out [2, H, W] must be contiguous float32")
        _check(lib.amb_learned_fft_forward(self._fft, _ptr(phi), _ptr(self._spec), _stream()))
        my, mx, nyf, nxf = self._filters_rm
        if spectral_noise is not None:
            seed, step = spectral_noise
            _check(lib.amb_learned_spectral_combine_noise(
                _ptr(self._spec), _ptr(my), _ptr(mx), _ptr(nyf), _ptr(nxf), float(noise_mag), ny, nx, nk, 1,
                int(seed), _ptr(step), _ptr(self._comb[0]), _ptr(self._comb[1]), _stream()))
        else:
            _check(lib.amb_learned_spectral_combine(
                _ptr(self._spec), None, _ptr(my), _ptr(mx), _ptr(nyf), _ptr(nxf), 0.0, ny * nk,
                _ptr(self._comb[0]), _ptr(self._comb[1]), _stream()))
        _check(lib.amb_learned_fft_inverse2(self._fft, _ptr(self._comb), _ptr(out), _stream()))
        return out

    def __del__(self):
        if getattr(self, "_fft", None) is not None:
            try:
                N.lib().amb_learned_fft_destroy(self._fft)
            except Exception:
                pass
            self._fft = None

    def extra(self, phi, xi, noise_mag: float, out, spectral_noise=None):
        """Linear part of phi [H, W] plus the noise flux of xi [2, H, W] (or None) into out [2, H, W]:
        forward FFTs, one combining kernel (``amb_learned_spectral_combine``), one batched
        inverse FFT of both components (its 1/(H W) folded into the filters).
        ``spectral_noise=(seed, step)`` draws the noise spectrum in the combining kernel
        (``amb_learned_spectral_combine_noise``: the draw of ``amb_learned_noise_spectral``,
        keyed by the device step counter) instead of transforming xi: statistically the same
        white noise, two forward FFTs and one kernel fewer."""
        torch = _torch()
        if not phi.is_cuda:
            raise CudaException("LinearPart.extra runs on the GPU")
        if xi is None:
            return self._extra_direct(phi, noise_mag, out, spectral_noise)
        spec = torch.fft.rfft2(phi)
        sxi = torch.fft.rfft2(xi)
        # cuFFT through torch may return the spectrum in a transposed (column-major) layout: the
        # combining kernel works in memory order, so the filters are kept in the FFT's layout
        # (converted once) and the spectra are used as they come when they are dense in it; a
        # drawn noise spectrum is written straight into that layout
        layout = tuple(spec.stride())
        n = spec.numel()
        if sum((d - 1) * st for d, st in zip(spec.shape, layout)) + 1 != n or min(layout) < 1:
            layout = (spec.shape[1], 1)   # not dense in its own strides: work row-major
        if self._layout != layout:
            # the inverse transform's 1/(H W) is folded into the filters (irfft2 with norm="forward")
            inv_n = 1.0 / (self.shape[0] * self.shape[1])
            self._filters = [torch.empty_strided(spec.shape, layout, dtype=spec.dtype, device=spec.device)
                             .copy_(f * inv_n) for f in (self.my, self.mx, self.ny_, self.nx_)]
            self._layout = layout
        if tuple(spec.stride()) != layout:
            spec = torch.empty_strided(spec.shape, layout, dtype=spec.dtype, device=spec.device).copy_(spec)
        comb = torch.empty_strided((2,) + tuple(spec.shape), (n,) + layout, dtype=spec.dtype, device=spec.device)
        my, mx, ny_, nx_ = self._filters
        if spectral_noise is not None:
            seed, step = spectral_noise
            _check(N.lib().amb_learned_spectral_combine_noise(
                _ptr(spec), _ptr(my), _ptr(mx), _ptr(ny_), _ptr(nx_), float(noise_mag), self.shape[0],
                self.shape[1], layout[0], layout[1], int(seed), _ptr(step), _ptr(comb[0]), _ptr(comb[1]),
                _stream()))
        else:
            if sxi is not None and (tuple(sxi.stride()[1:]) != layout or sxi.stride(0) != n):
                sxi = torch.empty_strided(sxi.shape, (n,) + layout, dtype=sxi.dtype, device=sxi.device).copy_(sxi)
            _check(N.lib().amb_learned_spectral_combine(
                _ptr(spec), _ptr(sxi), _ptr(my), _ptr(mx), _ptr(ny_), _ptr(nx_),
                float(noise_mag), n, _ptr(comb[0]), _ptr(comb[1]), _stream()))
        torch.fft.irfft2(comb, s=self.shape, norm="forward", out=out)
        return out


class LearnedStepper:
    """Advance one field by K Euler steps per network evaluation, with plain fallback.

    Args:
        net: trained :class:`FluxNet` (captured as it is when the first macro step runs).
        field: initial field (ny, nx), ncols % 128 == 0.
        stencil, model: as for :class:`Integrator` (dx = dy = 1 is what the network saw).
        K: Euler steps per macro step (the K the network was trained for).
        check_every: macro steps per verified span (the shortest interval between checks).
        max_check_every: longest interval; after each accepted check whose residual is below
            tol/4 the interval doubles up to this, a residual above tol/2 or a failed check
            resets it to ``check_every``. ``None`` (or ``check_every``) keeps it fixed. A failed
            check redoes its whole span with the plain integrator, so a longer interval trades
            a costlier rollback for fewer checks.
        tol: largest accepted relative residual ||learned - plain|| / ||plain - start|| of the
            checked deterministic macro step's increments.
        residual_sigma: if > 0, compare Gaussian low-passed increments (width in sites).
        atol: floor (RMS per site) on the increment norm the residual is divided by, so that
            nearly static states are judged by the absolute error of the macro step.
        bound: |phi| above which a state is rejected.
        use_graph: replay the learned macro step from a CUDA graph (captured on first use).
        filter_noise: shape the K-step noise draw with :func:`noise_filter` (the K-step
            accumulation of the linearised plain scheme); without it the K one-step draws
            are summed undamped, which overstates the high-wavenumber noise.
        spectral_noise: with ``filter_noise``, draw the noise spectrum directly
            (``amb_learned_noise_spectral``) instead of drawing two normals per site and
            transforming them; the same distribution, two forward FFTs fewer per macro step.
    """

    def __init__(self, net: FluxNet, field, stencil, model, *, K: int = 50, seed: int = 0, check_every: int = 40,
                 max_check_every: int | None = 320,
                 tol: float = 0.5, bound: float = 3.0, plain_precision: str = "f32", use_graph: bool = True,
                 filter_noise: bool = True, residual_sigma: float = 0.0, atol: float = 0.0,
                 spectral_noise: bool = True):
        torch = _torch()
        self.net = net
        self.stencil = Stencil(stencil)
        self.model = Model(model)
        self.K = int(K)
        self.dtk = self.K * self.stencil.dt
        self.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        self.check_every = int(check_every)
        self.max_check_every = max(self.check_every, int(max_check_every or check_every))
        self.interval = self.check_every
        self.checks = 0
        self.tol = float(tol)
        self.bound = float(bound)
        self.atol = float(atol)
        self.spectral_noise = bool(spectral_noise)
        host = np.asarray(field, dtype=np.float64)
        self.shape = host.shape
        dev = torch.device("cuda")
        self.phi_q = torch.from_numpy(np.rint(host * FIX).astype(np.int32)).to(dev)
        self.phi_f = (self.phi_q.double() / FIX).float()
        self.params = model_params_tensor([self.model], dev)
        # the network input of the current state: kept current by the update kernel inside a
        # macro step and by _refresh_input wherever the field changes outside one
        self._x = torch.zeros(1, 2, *self.shape, 8, dtype=torch.bfloat16, device=dev)
        self._refresh_input()
        self.flag = torch.zeros(1, dtype=torch.int32, device=dev)
        self.step_dev = torch.zeros(1, dtype=torch.int64, device=dev)
        self.xi = torch.zeros(2, *self.shape, dtype=torch.float32, device=dev)
        self.macro_steps = 0
        self.extra_steps = 0  # plain Euler steps outside macro steps (run_for_time's remainder)
        self.learned_steps = 0
        self.fallback_spans = 0
        self.residuals = []
        self._g = noise_filter(self.shape, self.stencil, self.model, self.K).to(dev) if filter_noise else None
        self._linear = LinearPart(self.shape, self.stencil, self.model, self.K, dev,
                                  with_linear=bool(getattr(net, "linear_split", False)))
        self._extra = torch.zeros(2, *self.shape, dtype=torch.float32, device=dev)
        self._wres = lowpass_weights(self.shape, residual_sigma, dev) if residual_sigma > 0 else None
        self.use_graph = bool(use_graph)
        self._graph = None
        quiet = Model(self.model)
        quiet.T = 0.0
        self._plain = Integrator(host, self.stencil, self.model, precision=plain_precision, seed=self.seed ^ 0x5EED)
        self._check_sim = Integrator(host, self.stencil, quiet, precision=plain_precision, seed=0)

    @property
    def time(self) -> float:
        return self.macro_steps * self.dtk + self.extra_steps * self.stencil.dt

    @property
    def field(self) -> np.ndarray:
        return (self.phi_q.cpu().numpy().astype(np.float64)) / FIX

    def mass_q(self) -> int:
        """Exact sum of the fixed-point field (integer)."""
        return int(self.phi_q.to(dtype=_torch().int64).sum().item())

    def _apply(self, noisy: bool) -> None:
        """Network flux, plus (one spectral pass) the linear part and the filtered noise flux,
        then the exactly conservative fixed-point update."""
        torch = _torch()
        lib = N.lib()
        ny, nx = self.shape
        net_flux = self.net.forward(self._x)
        noisy = noisy and self.model.T > 0
        mag = math.sqrt(2.0 * self.model.T) * math.sqrt(1.0 / (self.dtk * self.stencil.dx * self.stencil.dy))
        xi_direct = None
        if self._g is None and noisy:
            # unfiltered noise: the update kernel forms the face sums of xi itself
            _check(lib.amb_learned_noise(ny, nx, self.seed, _ptr(self.step_dev), _ptr(self.xi), _stream()))
            self._linear.extra(self.phi_f, None, 0.0, self._extra)
            xi_direct = self.xi
        elif noisy and self.spectral_noise:
            # filtered noise drawn directly as a spectrum, shaped and added in the spectral pass
            self._linear.extra(self.phi_f, None, mag, self._extra, spectral_noise=(self.seed, self.step_dev))
        elif noisy:
            _check(lib.amb_learned_noise(ny, nx, self.seed, _ptr(self.step_dev), _ptr(self.xi), _stream()))
            self._linear.extra(self.phi_f, self.xi, mag, self._extra)
        else:
            self._linear.extra(self.phi_f, None, 0.0, self._extra)
        _check(lib.amb_learned_update_input(_ptr(net_flux), _ptr(self._extra), ny, nx, self.dtk, self.stencil.dx,
                                            self.stencil.dy, _ptr(xi_direct), mag if xi_direct is not None else 0.0,
                                            _ptr(self.phi_q), _ptr(self.phi_f), self.bound, _ptr(self.flag),
                                            _ptr(self.step_dev), _ptr(self.params), _ptr(self._x), _stream()))

    def _refresh_input(self) -> None:
        _check(N.lib().amb_learned_input(_ptr(self.phi_f), _ptr(self.params), 1, self.shape[0], self.shape[1],
                                         _ptr(self._x), _stream()))

    def _macro_step(self) -> None:
        """One learned macro step (network, noise, fixed-point update, step counter).
        With use_graph the sequence is captured into a CUDA graph on first use and
        replayed afterwards (the network's weights are fixed from then on)."""
        torch = _torch()
        noisy = self.model.T > 0
        if self.use_graph and self._graph is None:
            self.net.refresh()
            saved = (self.phi_q.clone(), self.step_dev.clone(), self.flag.clone())
            side = torch.cuda.Stream()
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(side):  # one eager pass first: allocator pools, cuFFT plans
                self._apply(noisy=noisy)
            torch.cuda.current_stream().wait_stream(side)
            self.phi_q.copy_(saved[0])
            self.phi_f.copy_((self.phi_q.double() / FIX).float())
            self._refresh_input()
            self.step_dev.copy_(saved[1])
            self.flag.copy_(saved[2])
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):  # records only; the state changes at replay
                self._apply(noisy=noisy)
            self._graph = g
        if self._graph is not None:
            self._graph.replay()
        else:
            self._apply(noisy=noisy)

    def _set_from_float(self, f) -> None:
        self.phi_q.copy_(torch_round_fix(f))
        self.phi_f.copy_((self.phi_q.double() / FIX).float())
        self._refresh_input()

    def _run_plain(self, nsteps: int) -> None:
        sim = self._plain
        sim.field_tensor.copy_(self.phi_f)
        if sim._residual is not None:
            sim._residual.zero_()
        sim._timestep = self.macro_steps * self.K + self.extra_steps
        sim.run(nsteps)
        self._set_from_float(sim.field_tensor)

    def _residual(self, start):
        """Relative residual (device scalar) of one deterministic macro step, learned vs 50
        plain steps, from the state ``start`` [H, W], enqueued on the current stream. A
        non-finite plain or learned increment gives a non-finite residual."""
        torch = _torch()
        sim = self._check_sim
        sim.field_tensor.copy_(start)
        if sim._residual is not None:
            sim._residual.zero_()
        sim._launch(self.K)
        dplain = sim.field_tensor.float() - start
        flux = self.net.forward(network_input(start.unsqueeze(0), self.params))
        if getattr(self.net, "linear_split", False):
            flux = flux + self._linear.flux(start.unsqueeze(0))
        dpred = -self.dtk * divergence(flux, self.stencil.dx, self.stencil.dy)[0]
        if self._wres is not None:
            dpred, dplain = lowpass(dpred, self._wres), lowpass(dplain, self._wres)
        num = torch.linalg.vector_norm(dpred - dplain)
        # the increment's norm, floored at atol RMS per site so that near-static states
        # (tiny increments) are judged by the absolute error
        den = torch.clamp(torch.linalg.vector_norm(dplain), min=self.atol * math.sqrt(dplain.numel()) + 1e-30)
        return num / den

    def _accept(self, res: float) -> bool:
        self.residuals.append(res)
        return res <= self.tol and math.isfinite(res)

    def _check_step(self) -> bool:
        """One deterministic macro step learned vs plain from the current state; returns
        whether the relative residual of the increments is within tol (the state is not
        advanced)."""
        return self._accept(float(self._residual(self.phi_f.clone()).item()))

    def advance(self, n_macro: int) -> None:
        """Advance n_macro macro steps (each K Euler steps)."""
        left = int(n_macro)
        while left > 0:
            span = min(self.interval, left)
            snap_q = self.phi_q.clone()
            snap_step = self.step_dev.clone()
            self.flag.zero_()
            for _ in range(span - 1):
                self._macro_step()
            ok = self._check_step() and int(self.flag.item()) == 0
            self.checks += 1
            if ok:
                self._macro_step()
                ok = int(self.flag.item()) == 0
            self.interval = next_check_interval(self.interval, self.residuals[-1], ok, self.tol, self.check_every,
                                                self.max_check_every)
            if ok:
                self.learned_steps += span
            else:
                self.phi_q.copy_(snap_q)
                self.phi_f.copy_((self.phi_q.double() / FIX).float())
                self.step_dev.copy_(snap_step)
                self._run_plain(span * self.K)
                self.step_dev.add_(span)
                self.fallback_spans += 1
            self.macro_steps += span
            left -= span
        self.net.check_error()

    def run_for_time(self, t: float) -> None:
        """Advance by time t (a multiple of dt): as many macro steps of K dt as fit, then the
        remaining fewer than K Euler steps on the plain integrator."""
        dt = self.stencil.dt
        total = int(round(t / dt))
        if not math.isclose(total * dt, t, rel_tol=1e-9, abs_tol=1e-12):
            raise ValueError(f"t={t} is not a multiple of dt = {dt}")
        n, rem = divmod(total, self.K)
        self.advance(n)
        if rem:
            self._run_plain(rem)
            self.extra_steps += rem


def next_check_interval(interval: int, residual: float, accepted: bool, tol: float, base: int, longest: int) -> int:
    """Macro steps until the next residual check: doubled (up to ``longest``) after an accepted
    check whose residual is below tol/4, back to ``base`` after a residual above tol/2 or a
    failed check, unchanged otherwise."""
    if accepted and residual < 0.25 * tol:
        return min(2 * interval, longest)
    if not accepted or not residual <= 0.5 * tol:
        return base
    return interval


def torch_round_fix(f):
    """float field -> int32 fixed point (round to nearest)."""
    torch = _torch()
    return torch.round(f.double() * FIX).to(torch.int32)


# ---------------------------------------------------- training and evaluation runs

DEFAULT_SAMPLE_STEPS = (0, 1000, 3000, 10000, 30000, 100000, 200000, 400000, 700000, 1000000)


def train_default(out: str | None = None, *, n_traj: int = 512, size: int = 128, K=50, dt: float = 1e-3,
                  sample_steps=DEFAULT_SAMPLE_STEPS, iters: int = 8000, batch: int = 16, lr: float = 2e-3,
                  seed: int = 0, holdout: float = 0.1, lowpass_sigma: float = 0.0, highpass_weight: float = 1.0,
                  layers: int = NLAYERS, log=print):
    """Generate pairs with the plain integrator, train a FluxNet per K on the device kernels,
    report the held-out errors, and optionally save the weights (``FluxNet.load``; ``out``
    may contain ``{K}``). K may be one step count or a list sharing one set of trajectories.
    Returns {K: (net, info)}."""
    import time
    torch = _torch()
    Ks = list(K) if isinstance(K, (list, tuple)) else [int(K)]
    t0 = time.perf_counter()
    phi, deltas, params, _ = generate_pairs(n_traj, size, Ks, sample_steps, dt=dt, seed=seed)
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    n_test = max(1, int(round(holdout * n_traj)))
    results = {}
    for k in Ks:
        delta = deltas[k]
        tr = (phi[:, :-n_test], delta[:, :-n_test], params[:-n_test])
        te = (phi[:, -n_test:], delta[:, -n_test:], params[-n_test:])
        # the linear part depends on (a, c, kappa, dt, K, shape) only, which the pair set shares
        lin = LinearPart((size, size), Stencil(dt, 1, 1), Model(a=-0.25, b=0, c=0.25, kappa=1), k)
        zero = FluxNet(seed=seed, layers=layers)
        for w in zero.weights:
            w.zero_()
        linear_only = evaluate(zero, *te, K=k, dt=dt, linear=lin)
        net = FluxNet(seed=seed, layers=layers)
        before = evaluate(net, *te, K=k, dt=dt, linear=lin)
        t1 = time.perf_counter()
        hist = train(net, *tr, K=k, dt=dt, iters=iters, batch=batch, lr=lr, seed=seed,
                     log_every=max(1, iters // 20), lowpass_sigma=lowpass_sigma, highpass_weight=highpass_weight,
                     linear=lin)
        torch.cuda.synchronize()
        t_train = time.perf_counter() - t1
        after = evaluate(net, *te, K=k, dt=dt, linear=lin)
        after_lp = evaluate(net, *te, K=k, dt=dt, lowpass_sigma=2.0, linear=lin)
        net.K = k
        info = {"n_traj": n_traj, "size": size, "K": k, "layers": layers, "dt": dt, "sample_steps": list(sample_steps),
                "iters": iters, "batch": batch, "lr": lr, "seed": seed, "pairs": int(phi.shape[0] * phi.shape[1]),
                "data_seconds": t_data, "train_seconds": t_train, "heldout_rel_mse_linear_part_only": linear_only,
                "heldout_rel_mse_untrained": before, "heldout_rel_mse": after,
                "heldout_rel_mse_lowpass2": after_lp, "lowpass_sigma": lowpass_sigma,
                "highpass_weight": highpass_weight, "loss_history": hist}
        if log:
            log(f"K={k}, {layers} layers: data {t_data:.1f} s, train {t_train:.1f} s, held-out relative MSE: linear part alone "
                f"{linear_only:.3g}, untrained {before:.3g}, trained {after:.3g} (low-passed {after_lp:.3g})")
        if out:
            net.save(out.format(K=k), K=k, dt=dt, heldout_rel_mse=after, heldout_rel_mse_lowpass2=after_lp,
                     iters=iters, n_traj=n_traj, size=size, lowpass_sigma=lowpass_sigma)
        results[k] = (net, info)
    del phi, deltas
    return results


def _timed(fn):
    import time
    torch = _torch()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fn()
    torch.cuda.synchronize()
    return time.perf_counter() - t0


def _mean_rel_err(learned, plain) -> tuple[float, float]:
    """Signed relative difference of the means (learned - plain) / plain and its standard error
    (sample standard deviations, independent arms)."""
    learned, plain = np.asarray(learned, dtype=np.float64), np.asarray(plain, dtype=np.float64)
    se2 = sum(float(v.std(ddof=1)) ** 2 / len(v) for v in (plain, learned) if len(v) > 1)
    return float((learned.mean() - plain.mean()) / plain.mean()), float(np.sqrt(se2) / plain.mean())


def compare_with_plain(net: FluxNet, field, stencil, model, *, t_end: float, K: int | None = None, seed: int = 0,
                       check_every: int = 40, tol: float = 0.5, plain_seeds=tuple(range(1, 11)),
                       residual_sigma: float = 2.0, filter_noise: bool = True, atol: float = 0.0,
                       learned_runs: int = 10, max_check_every: int | None = 320, plain_launch: dict | None = None) -> dict:
    """Time to ``t_end`` and end-state statistics of the learned stepper against the plain
    FP32 integrator (the faster of the Integrator and a one-replica CUDA-graph ensemble)
    from the same initial field: the position of the S(k) peak (sub-bin estimate,
    ``analysis.peak_wavenumber``) and the S(k) mean wavenumber (both over the reference
    notebook's binned S(k)), droplet count, mass. The plain run is repeated with
    ``plain_seeds`` and the learned run with ``learned_runs`` noise seeds (``seed``, ``seed +
    1``, ...): each error is that of the learned mean against the plain mean with its standard
    error, the speed-up that of the fastest runs. ``plain_launch`` names the plain
    integrator's launch shape (``Integrator(kernel="tile", launch=...)``); by default the
    autotuner picks it."""
    from .analysis import count_droplets, mean_wavenumber, peak_wavenumber, structure_factor
    stencil, model = Stencil(stencil), Model(model)
    K = int(K if K is not None else getattr(net, "K", 50))
    nsteps = int(round(t_end / stencil.dt))
    field = np.asarray(field, dtype=np.float64)
    phi0 = float(field.mean())
    res = {"t_end": t_end, "K": K, "shape": list(field.shape), "model": model.as_dict(), "tol": tol, "atol": atol,
           "check_every": check_every, "max_check_every": max_check_every, "residual_sigma": residual_sigma,
           "filter_noise": filter_noise, "plain": []}
    probe = max(1, min(nsteps, 20000))
    plain_kw = {"kernel": "tile", "launch": plain_launch} if plain_launch else {}
    sim = Integrator(field, stencil, model, precision="f32", seed=0, **plain_kw)
    t_int = _timed(lambda: sim.run(probe))
    res["plain_kernel_config"] = getattr(sim, "kernel_config", None)
    del sim
    ens = Ensemble([field], stencil, model, precision="f32", seeds=[0], graph_steps=50)
    t_ens = _timed(lambda: ens.run(probe))
    ens.close()
    use_ensemble = t_ens < t_int
    res["plain_path"] = "ensemble" if use_ensemble else "integrator"
    res["plain_probe_us_per_step"] = {"integrator": 1e6 * t_int / probe, "ensemble": 1e6 * t_ens / probe}
    for sd in plain_seeds:
        if use_ensemble:
            ens = Ensemble([field], stencil, model, precision="f32", seeds=[sd], graph_steps=50)
            sec = _timed(lambda: ens.run(nsteps))
            f = ens.field(0)
            ens.close()
        else:
            sim = Integrator(field, stencil, model, precision="f32", seed=sd, **plain_kw)
            sec = _timed(lambda: sim.run(nsteps))
            f = sim.field
            del sim
        k, S, _ = structure_factor(f, stencil.dx, stencil.dy, phi0=phi0)
        res["plain"].append({"seconds": sec, "seed": sd, "k_avg": mean_wavenumber(k, S),
                             "k_peak": peak_wavenumber(k, S), "k_peak_bin": float(k[np.nanargmax(S)]),
                             "droplets": count_droplets(f, phi0), "mass_drift": float(f.sum() - field.sum())})
    res["learned_runs"] = []
    for sd in range(seed, seed + max(1, int(learned_runs))):
        st = LearnedStepper(net, field, stencil, model, K=K, seed=sd, check_every=check_every, tol=tol,
                            residual_sigma=residual_sigma, filter_noise=filter_noise, atol=atol,
                            max_check_every=max_check_every)
        m0 = st.mass_q()
        sec = _timed(lambda: st.run_for_time(t_end))
        f = st.field
        k, S, _ = structure_factor(f, stencil.dx, stencil.dy, phi0=phi0)
        res["learned_runs"].append({"seconds": sec, "seed": sd, "k_avg": mean_wavenumber(k, S),
                                    "k_peak": peak_wavenumber(k, S), "k_peak_bin": float(k[np.nanargmax(S)]),
                                    "droplets": count_droplets(f, phi0),
                                    "mass_q_drift": st.mass_q() - m0, "macro_steps": st.macro_steps,
                                    "learned_macro_steps": st.learned_steps, "fallback_spans": st.fallback_spans,
                                    "checks": st.checks, "max_residual": max(st.residuals) if st.residuals else None,
                                    "median_residual": float(np.median(st.residuals)) if st.residuals else None})
        del st
    runs = res["learned_runs"]
    res["learned"] = runs[0]
    plain_k = np.array([p["k_avg"] for p in res["plain"]])
    learned_k = np.array([r["k_avg"] for r in runs])
    res["plain_k_avg_mean"] = float(plain_k.mean())
    res["plain_k_avg_std"] = float(plain_k.std())
    res["learned_k_avg_mean"] = float(learned_k.mean())
    res["learned_k_avg_std"] = float(learned_k.std())
    err, se = _mean_rel_err(learned_k, plain_k)
    res["k_avg_rel_err"], res["k_avg_rel_err_se"] = abs(err), se
    for key in ("k_peak", "droplets"):
        err, se = _mean_rel_err([r[key] for r in runs], [p[key] for p in res["plain"]])
        res[f"{key}_rel_err"], res[f"{key}_rel_err_se"] = err, se
        res[f"plain_{key}_mean"] = float(np.mean([p[key] for p in res["plain"]]))
        res[f"learned_{key}_mean"] = float(np.mean([r[key] for r in runs]))
    res["plain_seconds_min"] = float(min(p["seconds"] for p in res["plain"]))
    res["learned_seconds_min"] = float(min(r["seconds"] for r in runs))
    res["learned_fallback_spans"] = int(sum(r["fallback_spans"] for r in runs))
    res["learned_mass_q_drift_max"] = int(max(abs(r["mass_q_drift"]) for r in runs))
    res["speedup"] = res["plain_seconds_min"] / res["learned_seconds_min"]
    return res


def _parse_launch(text: str) -> dict | None:
    """'pairs_per_cta=2,persistent=1' -> {"pairs_per_cta": 2, "persistent": True}; '' -> None."""
    if not text:
        return None
    out = {}
    for item in text.split(","):
        key, val = item.split("=")
        out[key.strip()] = bool(int(val)) if key.strip() == "persistent" else int(val)
    return out


def _main(argv=None) -> int:
    import argparse
    import json
    ap = argparse.ArgumentParser(prog="python -m activemodelbplus.learned")
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train", help="generate pairs with the plain integrator and train the flux network")
    t.add_argument("--out", required=True, help="weights path; may contain {K}")
    t.add_argument("--K", default="50", help="Euler steps per macro step; comma-separated for several")
    t.add_argument("--n-traj", type=int, default=512)
    t.add_argument("--size", type=int, default=128)
    t.add_argument("--iters", type=int, default=8000)
    t.add_argument("--batch", type=int, default=16)
    t.add_argument("--lr", type=float, default=2e-3)
    t.add_argument("--seed", type=int, default=0)
    t.add_argument("--info", default=None, help="write the run summary (JSON) here")
    t.add_argument("--sample-steps", default=",".join(str(v) for v in DEFAULT_SAMPLE_STEPS))
    t.add_argument("--lowpass-sigma", type=float, default=0.0)
    t.add_argument("--highpass-weight", type=float, default=1.0)
    t.add_argument("--layers", type=int, default=NLAYERS, help="convolution layers of the network")
    c = sub.add_parser("compare", help="time to t_end, learned vs plain FP32, from one seeded field")
    c.add_argument("--weights", required=True)
    c.add_argument("--size", type=int, default=512)
    c.add_argument("--t-end", type=float, default=1000.0)
    c.add_argument("--check-every", type=int, default=40)
    c.add_argument("--max-check-every", type=int, default=320)
    c.add_argument("--tol", type=float, default=0.5)
    c.add_argument("--seed", type=int, default=0)
    c.add_argument("--temperature", type=float, default=0.05)
    c.add_argument("--residual-sigma", type=float, default=2.0)
    c.add_argument("--no-noise-filter", action="store_true")
    c.add_argument("--plain-seeds", default=",".join(str(v) for v in range(1, 11)))
    c.add_argument("--learned-runs", type=int, default=10)
    c.add_argument("--plain-launch", default="",
                   help="plain integrator launch shape, e.g. 'pairs_per_cta=2,persistent=1' (tile kernel)")
    c.add_argument("--atol", type=float, default=0.0)
    a = ap.parse_args(argv)
    if a.cmd == "train":
        steps = [int(v) for v in a.sample_steps.split(",")]
        Ks = [int(v) for v in a.K.split(",")]
        res = train_default(a.out, n_traj=a.n_traj, size=a.size, iters=a.iters, batch=a.batch, lr=a.lr,
                            seed=a.seed, sample_steps=steps, lowpass_sigma=a.lowpass_sigma,
                            highpass_weight=a.highpass_weight, K=Ks if len(Ks) > 1 else Ks[0], layers=a.layers)
        if a.info:
            for k, (_, info) in res.items():
                with open(a.info.format(K=k), "w") as fh:
                    json.dump(info, fh, indent=1)
        return 0
    net = FluxNet.load(a.weights)
    rng = np.random.default_rng(a.seed)
    field = -0.4 + 0.01 * rng.standard_normal((a.size, a.size))
    model = Model(a=-0.25, b=0, c=0.25, kappa=1, lamb=-1, zeta=-4, T=a.temperature)
    res = compare_with_plain(net, field, Stencil(1e-3, 1, 1), model, t_end=a.t_end, seed=a.seed,
                             check_every=a.check_every, max_check_every=a.max_check_every, tol=a.tol,
                             residual_sigma=a.residual_sigma,
                             filter_noise=not a.no_noise_filter, atol=a.atol,
                             plain_seeds=tuple(int(v) for v in a.plain_seeds.split(",")),
                             learned_runs=a.learned_runs, plain_launch=_parse_launch(a.plain_launch))
    print(json.dumps(res))
    return 0


if __name__ == "__main__":
    raise SystemExit(_main())
