"""S(k) and droplet count on the GPU against the CPU restatement of the reference
notebook's analysis (oracle/analysis.py)."""
import numpy as np
import pytest

from oracle import analysis as ref

pytestmark = pytest.mark.gpu


def evolved_field(shape=(256, 384), steps=30000, dy=1.0):
    """AMB+ spinodal decomposition to t = 300 (growth time ~64), so droplets have formed."""
    from activemodelbplus.integrator import Integrator, Model, Stencil
    rng = np.random.default_rng(1)
    f = -0.4 + 0.05 * rng.standard_normal(shape)
    sim = Integrator(f, Stencil(1e-2, 1.0, dy), Model(-0.25, 0, 0.25, 1, -1, -4, 0), precision="f32c")
    sim.run(steps)
    return sim.field


@pytest.mark.parametrize("dy", [1.0, 1.25])
def test_structure_factor_matches_notebook_definition(dy):
    from activemodelbplus import analysis
    f = evolved_field(dy=dy)
    k, S, c = analysis.structure_factor(f, dx=1.0, dy=dy)
    k0, S0, c0 = ref.structure_factor(f, dx=1.0, dy=dy)
    assert np.array_equal(c, c0)
    m = np.isfinite(S0)
    assert np.array_equal(m, np.isfinite(S))
    assert np.abs(S[m] - S0[m]).max() <= 1e-9 * np.abs(S0[m]).max()
    from scipy.integrate import simpson
    kavg0 = simpson(k0[m] * S0[m], x=k0[m]) / simpson(S0[m], x=k0[m])
    assert abs(analysis.mean_wavenumber(k, S) - kavg0) < 1e-9


def test_droplet_count_matches_scipy_label():
    from activemodelbplus import analysis
    f = evolved_field()
    counts = []
    for thr in (None, 0.0, -0.2):
        n = analysis.count_droplets(f, thr)
        assert n == ref.count_droplets(f, thr)
        counts.append(n)
    assert max(counts) > 0


def test_droplet_labels_partition():
    import torch
    from activemodelbplus import analysis
    rng = np.random.default_rng(5)
    f = rng.standard_normal((200, 300)).astype(np.float32)
    labels, n = analysis.label_droplets(f, 0.8)
    lab = labels.cpu().numpy()
    assert n == ref.count_droplets(f, 0.8)
    assert ((lab >= 0) == (f > 0.8)).all()
    # each label is the smallest index of its component: label of a root site is itself
    flat = lab.ravel()
    roots = np.unique(flat[flat >= 0])
    assert len(roots) == n and (flat[roots] == roots).all()
    del torch
