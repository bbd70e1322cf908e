"""ORACLE — test infrastructure, not the product.

CPU restatement of the field analysis: the structure factor exactly as the reference's
notebook computes it (examples/structureFactor.ipynb, cells 5-7: numpy fft2, fftfreq,
np.digitize(right=True), per-bin np.average, scipy simpson), and the periodic droplet
count via scipy.ndimage.label (4-connectivity) with labels merged across the wrap.
"""
from __future__ import annotations

import numpy as np


def structure_factor(phi, dx=1.0, dy=1.0, phi0=None, edges=None):
    from numpy import fft
    phi = np.asarray(phi, dtype=np.float64)
    ny, nx = phi.shape
    if phi0 is None:
        phi0 = np.average(phi)
    edges = np.linspace(0, 3, 300)[1:] if edges is None else np.asarray(edges)
    k = 0.5 * (edges[1:] + edges[:-1])
    kx = 2 * np.pi * fft.fftfreq(nx, d=dx)
    ky = 2 * np.pi * fft.fftfreq(ny, d=dy)
    Kx, Ky = np.meshgrid(kx, ky, indexing="xy")
    K = (Kx ** 2 + Ky ** 2) ** 0.5
    indices = np.digitize(K, edges, right=True)
    phiq = np.abs(fft.fft2(phi - phi0) * dx * dy) ** 2
    S = np.full(k.size, np.nan)
    counts = np.zeros(k.size, dtype=np.int64)
    for l in range(S.size):
        sel = indices == l
        counts[l] = sel.sum()
        if counts[l]:
            S[l] = np.average(phiq[sel])
    return k, S, counts


def count_droplets(phi, threshold=None):
    from scipy import ndimage
    phi = np.asarray(phi)
    if threshold is None:
        threshold = float(np.mean(phi))
    mask = phi > threshold
    labels, n = ndimage.label(mask)
    parent = list(range(n + 1))

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a

    def unite(a, b):
        a, b = find(a), find(b)
        if a != b:
            parent[max(a, b)] = min(a, b)

    for a, b in zip(labels[:, 0], labels[:, -1]):
        if a and b:
            unite(a, b)
    for a, b in zip(labels[0, :], labels[-1, :]):
        if a and b:
            unite(a, b)
    return len({find(i) for i in range(1, n + 1)})
