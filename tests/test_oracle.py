"""The oracle pinned against the reference: its golden fixtures (always) and
the reference's own compiled CPU scheme (where the reference checkout exists).
Tolerances follow the reference's tests: tight_tol = 1e-12, absolute
(test/test_utilities.h:7)."""
import os

import numpy as np
import pytest

import oracle
from oracle import Params
from conftest import GOLDEN

TIGHT = 1e-12


def load(name):
    return np.load(os.path.join(GOLDEN, name))


def tj_params(dt, A, K, lamb, zeta):
    return Params(dt=dt, dx=1.0, dy=1.0, a=-A, b=0.0, c=A, kappa=K, lamb=lamb, zeta=zeta, T=0.0)


def test_onestep_terms_match_golden():
    """test/test_tjhung.cc:24-40 restated against the stored reference outputs."""
    g = load("tjhung_onestep_64x32.npz")
    p = tj_params(float(g["dt"]), float(g["A"]), float(g["K"]), float(g["lamb"]), float(g["zeta"]))
    t = oracle.terms(g["initial"], p)
    assert np.abs(t["mu_p"] - g["mueq"]).max() < TIGHT
    assert np.abs(t["mu_a"] - g["muact"]).max() < TIGHT
    # Tjhung's "x" is the first (row) axis: Jxeq is the y component here.
    assert np.abs(t["jp_y"] - g["jxeq"]).max() < TIGHT
    assert np.abs(t["jp_x"] - g["jyeq"]).max() < TIGHT
    assert np.abs(t["jl_y"] + t["jc_y"] - g["jxact"]).max() < TIGHT
    assert np.abs(t["jl_x"] + t["jc_x"] - g["jyact"]).max() < TIGHT
    div = oracle.divergence(g["initial"], p)
    assert np.abs(div + g["dphi"]).max() < TIGHT * 100  # |divJ| ~ 45: 2e-14 relative
    assert np.abs(div + g["dphi"]).max() / np.abs(g["dphi"]).max() < TIGHT


def test_spinodal_run_matches_golden():
    """Config: Model B spinodal 256^2, 10^4 steps; 1e-12 relative to max|phi|."""
    g = load("tjhung_spinodal_256.npz")
    p = Params(dt=float(g["dt"]), a=-0.25, b=0.0, c=0.25, kappa=1.0)
    final = oracle.run(g["initial"], p, int(g["nsteps"]), nthreads=os.cpu_count() or 1)
    scale = float(g["final_absmax"])
    assert np.abs(final[::4, ::4] - g["final_sub"]).max() / scale < TIGHT
    assert abs(final.sum() - float(g["final_sum"])) < 1e-9
    assert abs(np.abs(final).max() - scale) / scale < TIGHT


def test_active_run_matches_golden():
    g = load("tjhung_active_64.npz")
    p = tj_params(float(g["dt"]), 0.25, 1.0, float(g["lamb"]), float(g["zeta"]))
    final = oracle.run(g["initial"], p, int(g["nsteps"]))
    assert np.abs(final - g["final"]).max() / np.abs(g["final"]).max() < TIGHT


@pytest.mark.skipif(oracle.reference_lib() is None, reason="reference checkout not present")
@pytest.mark.parametrize("shape", [(64, 32), (40, 72), (9, 9), (33, 17)])
def test_terms_match_reference_live(shape):
    rng = np.random.default_rng(hash(shape) % 2**32)
    phi = rng.uniform(-1, 1, shape)
    for A, K, lamb, zeta in [(0.25, 1.0, 1.0, 1.0), (0.3, 0.7, -1.3, 0.7), (0.25, 1.0, -1.0, -4.0)]:
        p = tj_params(1e-2, A, K, lamb, zeta)
        ref = oracle.tjhung_dphi(phi, 1e-2, 1.0, A, K, lamb, zeta)
        t = oracle.terms(phi, p)
        assert np.abs(t["mu_p"] - ref["mueq"]).max() < TIGHT
        assert np.abs(t["jp_y"] - ref["jxeq"]).max() < TIGHT
        assert np.abs(t["jl_x"] + t["jc_x"] - ref["jyact"]).max() < TIGHT
        div = oracle.divergence(phi, p)
        assert np.abs(div + ref["dphi"]).max() / np.abs(ref["dphi"]).max() < TIGHT


def test_general_spacing_terms_restate_reference_formulas():
    """dx != dy and b != 0 (the reference's per-term tests, test/test_integrator.cc:47-195,
    use dy = 0.75 and 1.25): check each term against a direct numpy restatement."""
    rng = np.random.default_rng(3)
    phi = rng.uniform(-1, 1, (32, 64))
    p = Params(dt=1e-2, dx=1.0, dy=0.75, a=1.0, b=2.0, c=3.0, kappa=0.5, lamb=0.7, zeta=-1.1)
    t = oracle.terms(phi, p)

    def sh(f, dy, dx):
        return np.roll(f, (-dy, -dx), axis=(0, 1))

    gx = (0.1 * (sh(phi, -1, 1) - sh(phi, -1, -1) + sh(phi, 1, 1) - sh(phi, 1, -1))
          + 0.3 * (sh(phi, 0, 1) - sh(phi, 0, -1))) / p.dx
    gy = (0.1 * (sh(phi, 1, -1) - sh(phi, -1, -1) + sh(phi, 1, 1) - sh(phi, -1, 1))
          + 0.3 * (sh(phi, 1, 0) - sh(phi, -1, 0))) / p.dy
    sxx = sum(w * (sh(phi, di, -1) - 2 * sh(phi, di, 0) + sh(phi, di, 1)) for di, w in ((-1, -.25), (0, 1.5), (1, -.25)))
    syy = sum(w * (sh(phi, -1, dj) - 2 * sh(phi, 0, dj) + sh(phi, 1, dj)) for dj, w in ((-1, -.25), (0, 1.5), (1, -.25)))
    lap = sxx / p.dx ** 2 + syy / p.dy ** 2
    mup = p.a * phi + p.b * phi ** 2 + p.c * phi ** 3 - p.kappa * lap
    assert np.abs(t["mu_p"] - mup).max() < TIGHT * 10
    assert np.abs(t["mu_a"] - p.lamb * (gx ** 2 + gy ** 2)).max() < TIGHT * 10
    assert np.abs(t["jc_y"] - p.zeta * lap * gy).max() < TIGHT * 10
    d8 = [4 / 5, -1 / 5, 4 / 105, -1 / 280]
    jpy = -sum(d * (sh(mup, k + 1, 0) - sh(mup, -k - 1, 0)) for k, d in enumerate(d8)) / p.dy
    assert np.abs(t["jp_y"] - jpy).max() < TIGHT * 100


# ------------------------------------------------------------------ noise

def test_philox_known_answers():
    """Philox4x32-10 known-answer vectors (Random123 distribution, kat_vectors)."""
    assert [hex(v) for v in oracle.philox4x32_10([0, 0, 0, 0], [0, 0])] == \
        ["0x6627e8d5", "0xe169c58d", "0xbc57ac4c", "0x9b00dbd8"]
    assert [hex(v) for v in oracle.philox4x32_10([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2)] == \
        ["0x408f276d", "0x41c83b0e", "0xa20bc7c6", "0x6d5451fd"]
    assert [hex(v) for v in oracle.philox4x32_10([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344],
                                                 [0xA4093822, 0x299F31D0])] == \
        ["0xd16cfe09", "0x94fdcceb", "0x5001e420", "0x24126ea1"]


def test_noise_is_standard_normal_and_keyed():
    xy, xx = oracle.normals(256, 256, seed=12345, step=7)
    for z in (xy, xx):
        assert abs(z.mean()) < 0.02
        assert abs(z.var() - 1) < 0.02
        kurt = ((z - z.mean()) ** 4).mean() / z.var() ** 2
        assert abs(kurt - 3) < 0.1
    assert abs(np.corrcoef(xy.ravel(), xx.ravel())[0, 1]) < 0.02
    # neighbours in a quad share a Philox call but are independent
    assert abs(np.corrcoef(xy[:, 0::4].ravel(), xy[:, 1::4].ravel())[0, 1]) < 0.03
    xy2, _ = oracle.normals(256, 256, seed=12345, step=8)
    assert abs(np.corrcoef(xy.ravel(), xy2.ravel())[0, 1]) < 0.02
    xy3, _ = oracle.normals(256, 256, seed=12345, step=7)
    assert np.array_equal(xy, xy3)


def test_injected_noise_is_linear():
    """With injected noise the update adds -dt * D8 . (m xi): linear in xi."""
    rng = np.random.default_rng(5)
    phi = rng.uniform(-0.5, 0.5, (24, 40))
    p = Params(dt=1e-3, dx=1, dy=1, a=-0.25, c=0.25, kappa=1, lamb=-1, zeta=-4, T=0.05)
    xi = rng.standard_normal((1, 2, 24, 40))
    a = oracle.run(phi, p, 1, noise="injected", injected=xi)
    b = oracle.run(phi, p, 1, noise="injected", injected=0 * xi)
    c = oracle.run(phi, p, 1, noise="injected", injected=2 * xi)
    assert np.abs((c - b) - 2 * (a - b)).max() < 1e-13


def test_mass_conserved_by_oracle():
    rng = np.random.default_rng(9)
    phi = 0.1 * rng.random((64, 128))
    phi -= phi.mean()
    p = Params(dt=1e-2, dx=1.0, dy=1.25, a=-0.25, b=0.5, c=0.25, kappa=1, lamb=1, zeta=1)
    out = oracle.run(phi, p, 200)
    assert abs(oracle.mass(out) - oracle.mass(phi)) < 1e-10
