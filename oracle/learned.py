"""CPU FP64 oracle for the learned coarse stepper's kernels. TEST INFRASTRUCTURE
ONLY: imported by tests/ and never by the product package.

The learned stepper has no counterpart in the reference (tranqui/active-model-bplus
has no learned component), so its oracle is the mathematics it implements:

* circular 5x5 convolution (cross-correlation, as torch.nn.functional.conv2d
  defines it) over periodically padded input, evaluated by torch on the CPU in
  float64;
* its data and weight gradients (torch autograd in float64);
* GELU in its tanh form (Hendrycks and Gimpel) and its derivative;
* the face-flux update in int64 fixed point (phi * 2^24), restated with the
  same IEEE single-precision operations in the same order as the device kernel
  (sums, product, then round half to even), so it is bit-exact;
* the order-8 central difference written as a difference of face sums, from
  the coefficients c = (4/5, -1/5, 4/105, -1/280) of the reference's D8
  operator (src/finite_difference.h:73).
"""
from __future__ import annotations

import math

import numpy as np

FIX = float(1 << 24)
D8 = (4.0 / 5.0, -1.0 / 5.0, 4.0 / 105.0, -1.0 / 280.0)


def _torch():
    import torch
    return torch


def bf16_round(x: np.ndarray) -> np.ndarray:
    """Round float values to bfloat16 (round to nearest even) and back to float64."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    rounding = ((u >> 16) & 1) + 0x7FFF
    r = ((u + rounding) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def conv5x5(x, w, b=None):
    """Circular 5x5 convolution: out[b, co, r, c] = sum w[co, ci, ky, kx] x[b, ci, r+ky-2, c+kx-2]."""
    torch = _torch()
    F = torch.nn.functional
    xt = torch.as_tensor(np.asarray(x, dtype=np.float64))
    wt = torch.as_tensor(np.asarray(w, dtype=np.float64))
    out = F.conv2d(F.pad(xt, (2, 2, 2, 2), mode="circular"), wt)
    if b is not None:
        out = out + torch.as_tensor(np.asarray(b, dtype=np.float64)).view(1, -1, 1, 1)
    return out.numpy()


def conv5x5_grads(x, w, dout):
    """(d input, d weights) of conv5x5 for the output gradient dout (float64 autograd)."""
    torch = _torch()
    F = torch.nn.functional
    xt = torch.as_tensor(np.asarray(x, dtype=np.float64)).requires_grad_(True)
    wt = torch.as_tensor(np.asarray(w, dtype=np.float64)).requires_grad_(True)
    out = F.conv2d(F.pad(xt, (2, 2, 2, 2), mode="circular"), wt)
    out.backward(torch.as_tensor(np.asarray(dout, dtype=np.float64)))
    return xt.grad.numpy(), wt.grad.numpy()


GELU_C0 = math.sqrt(2.0 / math.pi)
GELU_C1 = 0.044715


def gelu(z):
    """GELU in its tanh form (Hendrycks and Gimpel), as the device epilogue evaluates it."""
    z = np.asarray(z, dtype=np.float64)
    return 0.5 * z * (1.0 + np.tanh(GELU_C0 * (z + GELU_C1 * z ** 3)))


def gelu_grad(z):
    z = np.asarray(z, dtype=np.float64)
    t = np.tanh(GELU_C0 * (z + GELU_C1 * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * GELU_C0 * (1.0 + 3.0 * GELU_C1 * z * z)


def network_input(phi, params):
    """The network's 5 input channels for fields phi [B, H, W] and params [B, 3] = (zeta, lambda, T):
    bf16(phi), 256 (phi - bf16(phi)), zeta / 4, lambda, 10 T (float64, before bf16 storage)."""
    phi = np.asarray(phi, dtype=np.float32).astype(np.float64)
    hi = bf16_round(phi)
    lo = (phi - hi).astype(np.float32).astype(np.float64) * 256.0
    B, H, W = phi.shape
    p = np.asarray(params, dtype=np.float32).astype(np.float64)
    planes = [hi, lo] + [np.broadcast_to(v[:, None, None], (B, H, W)) for v in
                         (p[:, 0] * 0.25, p[:, 1], p[:, 2] * 10.0)]
    return np.stack(planes, axis=1)


def fluxnet(x, weights, biases, dflux=None, *, bf16_activations=True):
    """Forward (and, with dflux, backward) of the 6-layer flux network in float64.

    x: [B, 5, H, W]; weights[l]: [cout, cin, 5, 5]; biases[l]: [>= cout]. Hidden layers use
    GELU. With bf16_activations the stored activations, pre-activations and back-propagated
    gradients are rounded to bf16 where the device path stores them, and weights are rounded
    to bf16 as the device path reads them. Returns flux [B, 2, H, W] and, with dflux,
    (weight grads, bias grads).
    """
    rnd = bf16_round if bf16_activations else (lambda v: np.asarray(v, dtype=np.float64))
    L = len(weights)
    a = rnd(x)
    acts, pres = [], []
    for l in range(L):
        w = rnd(weights[l])
        b = np.asarray(biases[l], dtype=np.float64)[: w.shape[0]]
        if bf16_activations:
            b = b.astype(np.float32).astype(np.float64)  # the device keeps biases in FP32
        z = conv5x5(a, w, b)
        acts.append(a)
        if l < L - 1:
            pres.append(rnd(z))
            a = rnd(gelu(z))
        else:
            flux = z
    if dflux is None:
        return flux
    gw, gb = [None] * L, [None] * L
    dz = rnd(dflux)
    for l in range(L - 1, -1, -1):
        w = rnd(weights[l])
        dx, dw = conv5x5_grads(acts[l], w, dz)
        gw[l] = dw
        gb[l] = dz.sum(axis=(0, 2, 3))
        if l > 0:
            dz = rnd(dx * gelu_grad(pres[l - 1]))
    return flux, gw, gb


def d8_face_weights():
    """w_e (e = -3..4) with D8 f(j) = F(j+1/2) - F(j-1/2), F(j+1/2) = sum_e w_e f(j+e)."""
    out = []
    for e in range(-3, 5):
        d0 = max(e, 1 - e)
        out.append(sum(D8[d - 1] for d in range(d0, 5)))
    return np.array(out)


def face_update(phi_q, flux, dtk, dx=1.0, dy=1.0, xi=None, noise_mag=0.0, extra=None):
    """Fixed-point macro step: phi_q (int64 [H, W]) minus the integer face increments of the
    face flux [2, H, W] (component 0 = y face after (r, c), 1 = x face), plus extra [2, H, W] if
    given, plus the noise flux noise_mag * sum_e w_e xi(. + e) on each face (xi [2, H, W]).
    Face values are formed in float32 with the device's operation order (flux + extra, noise
    sum in increasing e, then times noise_mag, then times the scale dtk / d * 2^24), clamped to
    +-1e9 and rounded half to even."""
    f32 = np.float32
    flux = np.asarray(flux, dtype=f32)
    w = d8_face_weights().astype(f32)

    def faces(comp, axis, scale):
        v = flux[comp].copy()
        if extra is not None:
            v = (v + np.asarray(extra[comp], dtype=f32)).astype(f32)
        if xi is not None:
            x = np.asarray(xi[comp], dtype=f32)
            s = np.zeros_like(v)
            for i, e in enumerate(range(-3, 5)):
                s = (s + (w[i] * np.roll(x, -e, axis=axis)).astype(f32)).astype(f32)
            v = (v + (f32(noise_mag) * s).astype(f32)).astype(f32)
        q = (f32(scale) * v).astype(f32)
        q = np.clip(q, f32(-1e9), f32(1e9))
        return np.rint(q).astype(np.int64)

    qy = faces(0, 0, dtk / dy * FIX)
    qx = faces(1, 1, dtk / dx * FIX)
    dq = (qx - np.roll(qx, 1, axis=1)) + (qy - np.roll(qy, 1, axis=0))
    return np.asarray(phi_q, dtype=np.int64) - dq
