"""The analysis oracle on known answers (CPU)."""
import numpy as np

from oracle import analysis


def disks(shape, centres, radius):
    ny, nx = shape
    y, x = np.mgrid[0:ny, 0:nx]
    f = -np.ones(shape)
    for cy, cx in centres:
        dy = np.minimum(np.abs(y - cy), ny - np.abs(y - cy))
        dx = np.minimum(np.abs(x - cx), nx - np.abs(x - cx))
        f[dy ** 2 + dx ** 2 <= radius ** 2] = 1.0
    return f


def test_periodic_droplet_count():
    f = disks((64, 96), [(10, 10), (32, 48), (0, 0), (63, 95), (40, 2), (5, 60)], 4)
    # (0,0) and (63,95) are one droplet across the corner; (40,2) wraps across x
    assert analysis.count_droplets(f, 0.0) == 5


def test_structure_factor_single_mode():
    ny, nx = 128, 128
    y, x = np.mgrid[0:ny, 0:nx]
    k0 = 2 * np.pi * 8 / nx
    f = np.cos(k0 * x)
    k, S, c = analysis.structure_factor(f)
    l = np.nanargmax(S)
    assert abs(k[l] - k0) < 0.02  # the notebook pairs bin l with the next mid-point: within a bin
    assert c.sum() <= ny * nx
