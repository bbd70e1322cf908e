"""Structure factor S(k) and droplet count of a field, on the GPU.

S(k) follows the reference's analysis notebook (examples/structureFactor.ipynb, cells
5-7): phi_q = FFT2(phi - phi0) dx dy; |phi_q|^2 is averaged over the modes whose |k|
falls in each radial bin, bins being ``np.digitize(|k|, edges, right=True)`` with
``edges = linspace(0, 3, 300)[1:]`` and k the bin mid-points; the mean wavenumber is
k_avg = simpson(k S, k) / simpson(S, k). The FFT runs in cuFFT (torch.fft); binning,
and the droplet labelling, run in this package's CUDA kernels (libamb_gb300.so).

Droplets: 4-connected components of {phi > threshold} with periodic wrap.
"""
from __future__ import annotations

import ctypes

import numpy as np

from .integrator import _native as N
from .integrator import CudaException


def _torch():
    import torch
    return torch


def _check(rc):
    if rc:
        raise (ValueError if rc == N.AMB_ERR_INVALID else CudaException)(N.last_error())


def default_edges() -> np.ndarray:
    """The notebook's radial bin edges, linspace(0, 3, 300)[1:]."""
    return np.linspace(0, 3, 300)[1:]


def _as_device(field, dtype=None):
    torch = _torch()
    if isinstance(field, torch.Tensor):
        t = field if field.is_cuda else field.cuda()
    else:
        t = torch.from_numpy(np.ascontiguousarray(field)).cuda()
    if dtype is not None:
        t = t.to(dtype)
    return t.contiguous()


def power_spectrum(field, dx: float = 1.0, dy: float = 1.0, phi0: float | None = None):
    """|FFT2(phi - phi0) dx dy|^2 on the device (phi0 defaults to the field mean)."""
    torch = _torch()
    phi = _as_device(field, torch.float64)
    if phi0 is None:
        phi0 = float(phi.mean())
    q = torch.fft.fft2(phi - phi0) * (dx * dy)
    return (q.real ** 2 + q.imag ** 2).contiguous()


def structure_factor(field, dx: float = 1.0, dy: float = 1.0, phi0: float | None = None, edges=None):
    """(k, S, counts): S[l] is the mean |phi_q|^2 of bin l (NaN where a bin has no mode),
    k[l] the mid-point of edges[l], edges[l+1], exactly as the reference notebook pairs them."""
    torch = _torch()
    edges = default_edges() if edges is None else np.asarray(edges, dtype=np.float64)
    power = power_spectrum(field, dx, dy, phi0)
    ny, nx = power.shape
    e = torch.from_numpy(edges).cuda()
    sums = torch.empty(len(edges), dtype=torch.float64, device="cuda")
    counts = torch.empty(len(edges), dtype=torch.int64, device="cuda")
    _check(N.lib().amb_radial_spectrum(power.data_ptr(), ny, nx, dx, dy, e.data_ptr(), len(edges), sums.data_ptr(),
                                       counts.data_ptr(), torch.cuda.current_stream().cuda_stream))
    k = 0.5 * (edges[1:] + edges[:-1])
    s = sums.cpu().numpy()[: len(k)]
    c = counts.cpu().numpy()[: len(k)]
    with np.errstate(invalid="ignore", divide="ignore"):
        S = np.where(c > 0, s / np.maximum(c, 1), np.nan)
    return k, S, c


def mean_wavenumber(k, S) -> float:
    """k_avg = simpson(k S, k) / simpson(S, k) over the bins that hold modes."""
    from scipy.integrate import simpson
    m = np.isfinite(S)
    return float(simpson(k[m] * S[m], x=k[m]) / simpson(S[m], x=k[m]))


def peak_wavenumber(k, S, frac: float = 0.5) -> float:
    """Sub-bin position of the maximum of a binned S(k): the vertex of the least-squares
    parabola through the contiguous bins around the largest one whose S is at least ``frac``
    of it (at least the three bins centred on the maximum). Falls back to the largest bin's
    k if the fit has no maximum inside those bins."""
    k = np.asarray(k, dtype=np.float64)
    S = np.asarray(S, dtype=np.float64)
    m = np.isfinite(S)
    k, S = k[m], S[m]
    i = int(np.argmax(S))
    lo, hi = i, i
    while lo > 0 and S[lo - 1] >= frac * S[i]:
        lo -= 1
    while hi < len(S) - 1 and S[hi + 1] >= frac * S[i]:
        hi += 1
    lo, hi = max(0, min(lo, i - 1)), min(len(S) - 1, max(hi, i + 1))
    if hi - lo < 2:
        return float(k[i])
    c2, c1, _ = np.polyfit(k[lo:hi + 1] - k[i], S[lo:hi + 1], 2)
    if c2 >= 0:
        return float(k[i])
    v = -c1 / (2 * c2) + k[i]
    return float(v) if k[lo] <= v <= k[hi] else float(k[i])


def label_droplets(field, threshold: float | None = None):
    """(labels, count): periodic 4-connected components of {phi > threshold} (threshold
    defaults to the field mean). labels is a device int32 tensor (-1 = background)."""
    torch = _torch()
    phi = _as_device(field)
    if phi.dtype not in (torch.float32, torch.float64):
        phi = phi.to(torch.float64)
    if threshold is None:
        threshold = float(phi.double().mean())
    ny, nx = phi.shape
    labels = torch.empty((ny, nx), dtype=torch.int32, device="cuda")
    count = torch.empty(1, dtype=torch.int32, device="cuda")
    fn = N.lib().amb_label_components_f64 if phi.dtype == torch.float64 else N.lib().amb_label_components_f32
    _check(fn(phi.data_ptr(), ny, nx, float(threshold), labels.data_ptr(), count.data_ptr(),
              torch.cuda.current_stream().cuda_stream))
    return labels, int(count.item())


def count_droplets(field, threshold: float | None = None) -> int:
    return label_droplets(field, threshold)[1]
