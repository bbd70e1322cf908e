"""Learned coarse stepper (no reference counterpart).

A periodic convolutional network maps (phi, zeta, lambda, T) to a face flux F
that advances the field by K explicit-Euler steps at once:

    phi(t + K dt) = phi(t) - K dt * div F  (+ the K-step noise flux when T > 0)

Because the update is a difference of face fluxes, applied in int32 fixed point
(phi * 2^24) with each face rounded once, the sum of the field is conserved
exactly. The network is 6 circular 5x5 convolutions, 32 channels, GELU (tanh form), BF16
weights and activations with FP32 accumulation; its forward and both backward
passes run on this package's own tcgen05 implicit-GEMM kernels
(``amb_conv5x5_forward`` / ``amb_conv5x5_wgrad``). Training targets are the
deterministic K-step increments of the plain integrator started from states of
noisy trajectories; the noise is added back per macro step as the exact K-step
aggregate of the plain scheme's noise flux. The plain integrator is the
fallback: every ``check_every`` macro steps one step is compared with K plain
deterministic steps from the same state, and if the residual exceeds ``tol``
(or the field left its bounds) the span since the last check is redone with
the plain integrator.
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
    """6 circular 5x5 convolutions (5 -> 32 -> 32 -> 32 -> 32 -> 32 -> 2), GELU between
    layers, BF16 weights/activations, FP32 accumulation and FP32 master weights."""

    def __init__(self, device=None, seed: int = 0):
        torch = _torch()
        device = torch.device("cuda") if device is None else torch.device(device)
        g = torch.Generator().manual_seed(int(seed))
        self.device = device
        self.cin = [CIN0] + [HIDDEN] * 5
        self.cin_used = [CIN0_USED] + [HIDDEN] * 5
        self.cout = [HIDDEN] * 5 + [NOUT]
        self.npad = [HIDDEN] * 5 + [NOUT_PAD]
        self.weights, self.biases = [], []
        for l in range(NLAYERS):
            fan_in = 25 * self.cin_used[l]
            std = math.sqrt(2.0 / fan_in) if l < NLAYERS - 1 else 0.1 / math.sqrt(fan_in)
            self.weights.append((torch.randn(self.cout[l], self.cin_used[l], 5, 5, generator=g) * std).to(device))
            self.biases.append(torch.zeros(self.npad[l], device=device))
        self.error = torch.zeros(1, dtype=torch.int32, device=device)
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
                                  for l in range(1, NLAYERS)]

    def state_dict(self) -> dict:
        d = {}
        for l in range(NLAYERS):
            d[f"w{l}"] = self.weights[l].cpu().numpy()
            d[f"b{l}"] = self.biases[l].cpu().numpy()
        return d

    def load_state_dict(self, d) -> None:
        torch = _torch()
        for l in range(NLAYERS):
            self.weights[l] = torch.as_tensor(np.asarray(d[f"w{l}"]), dtype=torch.float32).to(self.device)
            self.biases[l] = torch.as_tensor(np.asarray(d[f"b{l}"]), dtype=torch.float32).to(self.device)
        self._images = None

    def save(self, path: str, **meta) -> None:
        np.savez(path, **self.state_dict(), **{k: np.asarray(v) for k, v in meta.items()})

    @classmethod
    def load(cls, path: str, device=None) -> "FluxNet":
        z = np.load(path, allow_pickle=False)
        net = cls(device=device)
        net.load_state_dict({k: z[k] for k in z.files})
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
        for l in range(NLAYERS - 1):
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
        gw, gb = [None] * NLAYERS, [None] * NLAYERS
        dz = to_chunks(dflux, NOUT_PAD)
        L = NLAYERS - 1
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


def generate_pairs(n_traj: int, size: int, K: int, sample_steps, *, dt: float = 1e-3, seed: int = 0,
                   graph_steps: int = 50):
    """Training pairs from the plain integrator.

    ``n_traj`` noisy trajectories of size x size with parameters drawn uniformly from
    zeta in [-4, 4], lambda in [-1, 1], phi0 in [-0.6, 0.6], T in [0, 0.1] (a = -0.25,
    b = 0, c = 0.25, kappa = 1) and initial fields phi0 + 0.01 N(0, 1), advanced as one
    batched ensemble. At each sample step the states are copied into a second, noiseless
    ensemble with the same (zeta, lambda) that runs K steps: the pair is (state, its
    deterministic K-step increment). Returns device tensors phi [S, n, H, W],
    delta [S, n, H, W] and params [n, 3], and the model list.
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
    phi = torch.empty(S, n_traj, size, size, dtype=torch.float32, device="cuda")
    delta = torch.empty_like(phi)
    done = 0
    for s, st in enumerate(sample_steps):
        noisy.run(int(st) - done)
        done = int(st)
        x = noisy.gather(phi[s].reshape(-1))
        det.scatter(x)
        det.run(K)
        y = det.gather(delta[s].reshape(-1))
        delta[s].sub_(phi[s])
        del y
    noisy.close()
    det.close()
    return phi, delta, model_params_tensor(models, "cuda"), models


def train(net: FluxNet, phi, delta, params, *, K: int, dt: float, iters: int, batch: int = 16, lr: float = 2e-3,
          seed: int = 0, log_every: int = 0):
    """Fit the flux so that -K dt div F matches the deterministic K-step increments.

    phi, delta: [S, n, H, W]; params: [n, 3]. Adam on the FP32 master weights; the
    gradients come from the network's own backward kernels. Returns the loss history
    (relative mean-square error per iteration).
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
    hist = []
    for it in range(iters):
        si = torch.randint(0, S, (batch,), generator=g)
        ni = torch.randint(0, n, (batch,), generator=g)
        si, ni = si.to(phi.device), ni.to(phi.device)
        x = network_input(phi[si, ni].contiguous(), params[ni].contiguous())
        flux = net.forward(x, train=True)
        f = flux.detach().requires_grad_(True)
        pred = -dtk * divergence(f, 1.0, 1.0)
        loss = (pred - delta[si, ni]).square().mean() / scale
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


def evaluate(net: FluxNet, phi, delta, params, *, K: int, dt: float, batch: int = 16):
    """Relative mean-square error of the predicted K-step increments over a pair set."""
    torch = _torch()
    S, n, H, W = phi.shape
    num, den = 0.0, 0.0
    flat_phi = phi.reshape(S * n, H, W)
    flat_delta = delta.reshape(S * n, H, W)
    flat_params = params.repeat(S, 1)
    for i in range(0, S * n, batch):
        x = network_input(flat_phi[i:i + batch].contiguous(), flat_params[i:i + batch].contiguous())
        pred = -K * dt * divergence(net.forward(x), 1.0, 1.0)
        num += float((pred - flat_delta[i:i + batch]).square().sum().item())
        den += float(flat_delta[i:i + batch].square().sum().item())
    return num / max(den, 1e-30)


# -------------------------------------------------------------- stepper

class LearnedStepper:
    """Advance one field by K Euler steps per network evaluation, with plain fallback.

    Args:
        net: trained :class:`FluxNet`.
        field: initial field (ny, nx), ncols % 128 == 0.
        stencil, model: as for :class:`Integrator` (dx = dy = 1 is what the network saw).
        K: Euler steps per macro step (the K the network was trained for).
        check_every: macro steps per verified span.
        tol: largest accepted relative residual ||learned - plain|| / ||plain - start|| of the
            checked deterministic macro step.
        bound: |phi| above which a state is rejected.
    """

    def __init__(self, net: FluxNet, field, stencil, model, *, K: int = 50, seed: int = 0, check_every: int = 20,
                 tol: float = 0.5, bound: float = 3.0, plain_precision: str = "f32"):
        torch = _torch()
        self.net = net
        self.stencil = Stencil(stencil)
        self.model = Model(model)
        self.K = int(K)
        self.dtk = self.K * self.stencil.dt
        self.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        self.check_every = int(check_every)
        self.tol = float(tol)
        self.bound = float(bound)
        host = np.asarray(field, dtype=np.float64)
        self.shape = host.shape
        dev = torch.device("cuda")
        self.phi_q = torch.from_numpy(np.rint(host * FIX).astype(np.int32)).to(dev)
        self.phi_f = (self.phi_q.double() / FIX).float()
        self.params = model_params_tensor([self.model], dev)
        self.flag = torch.zeros(1, dtype=torch.int32, device=dev)
        self.step_dev = torch.zeros(1, dtype=torch.int64, device=dev)
        self.xi = torch.empty(2, *self.shape, dtype=torch.float32, device=dev)
        self.macro_steps = 0
        self.learned_steps = 0
        self.fallback_spans = 0
        self.residuals = []
        quiet = Model(self.model)
        quiet.T = 0.0
        self._plain = Integrator(host, self.stencil, self.model, precision=plain_precision, seed=self.seed ^ 0x5EED)
        self._check_sim = Integrator(host, self.stencil, quiet, precision=plain_precision, seed=0)

    @property
    def time(self) -> float:
        return self.macro_steps * self.dtk

    @property
    def field(self) -> np.ndarray:
        return (self.phi_q.cpu().numpy().astype(np.float64)) / FIX

    def mass_q(self) -> int:
        """Exact sum of the fixed-point field (integer)."""
        return int(self.phi_q.to(dtype=_torch().int64).sum().item())

    def _flux(self):
        return self.net.forward(network_input(self.phi_f.unsqueeze(0), self.params))

    def _apply(self, flux, noisy: bool) -> None:
        T = self.model.T if noisy else 0.0
        _check(N.lib().amb_learned_update(_ptr(flux), self.shape[0], self.shape[1], self.dtk, self.stencil.dx,
                                          self.stencil.dy, T, self.seed, _ptr(self.step_dev), _ptr(self.xi),
                                          _ptr(self.phi_q), _ptr(self.phi_f), self.bound, _ptr(self.flag),
                                          _stream()))
        self.step_dev.add_(1)

    def _set_from_float(self, f) -> None:
        self.phi_q.copy_(torch_round_fix(f))
        self.phi_f.copy_((self.phi_q.double() / FIX).float())

    def _run_plain(self, nsteps: int) -> None:
        sim = self._plain
        sim.field_tensor.copy_(self.phi_f)
        if sim._residual is not None:
            sim._residual.zero_()
        sim._timestep = self.macro_steps * self.K
        sim.run(nsteps)
        self._set_from_float(sim.field_tensor)

    def _check_step(self) -> bool:
        """One deterministic macro step learned vs plain from the current state;
        returns whether it is within tol (the state is not advanced)."""
        torch = _torch()
        start = self.phi_f.clone()
        sim = self._check_sim
        sim.field_tensor.copy_(start)
        if sim._residual is not None:
            sim._residual.zero_()
        sim.run(self.K)
        plain = sim.field_tensor.float()
        pred = start - self.dtk * divergence(self._flux(), self.stencil.dx, self.stencil.dy)[0]
        num = torch.linalg.vector_norm(pred - plain)
        den = torch.linalg.vector_norm(plain - start)
        res = float((num / torch.clamp(den, min=1e-30)).item())
        self.residuals.append(res)
        return res <= self.tol and math.isfinite(res)

    def advance(self, n_macro: int) -> None:
        """Advance n_macro macro steps (each K Euler steps)."""
        torch = _torch()
        left = int(n_macro)
        while left > 0:
            span = min(self.check_every, left)
            snap_q = self.phi_q.clone()
            snap_step = self.step_dev.clone()
            self.flag.zero_()
            for _ in range(span - 1):
                self._apply(self._flux(), noisy=self.model.T > 0)
            ok = self._check_step() and int(self.flag.item()) == 0
            if ok:
                self._apply(self._flux(), noisy=self.model.T > 0)
                ok = int(self.flag.item()) == 0
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
        del torch

    def run_for_time(self, t: float) -> None:
        n = int(round(t / self.dtk))
        if not math.isclose(n * self.dtk, t, rel_tol=1e-9, abs_tol=1e-12):
            raise ValueError(f"t={t} is not a multiple of K dt = {self.dtk}")
        self.advance(n)


def torch_round_fix(f):
    """float field -> int32 fixed point (round to nearest)."""
    torch = _torch()
    return torch.round(f.double() * FIX).to(torch.int32)
