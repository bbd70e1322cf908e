"""The FP32 kernels against each other and against the oracle, through the
device-pointer C ABI (amb_step_f32_ex).

Covers the warp-pair sliding kernel's decomposition (row segments, strips, the
overlapping last strip, periodic wrap of the row window), its Philox and
injected noise, and both FP32 storage modes. Both FP32 kernels (tile, sliding)
evaluate the same operations in the same order at every site (amb_canon.cuh),
so they agree bitwise with each other and under any decomposition; against the
FP64 oracle the tolerances are stated per test.
"""
import ctypes

import numpy as np
import pytest

import oracle
from oracle import Params

pytestmark = pytest.mark.gpu


def native():
    from activemodelbplus.integrator import _native as N
    return N


def run_f32(field, p: Params, nsteps, *, kernel=1, seg_rows=0, pairs=0, comp=True, seed=7, injected=None, step0=0,
            flags=0):
    import torch
    N = native()
    ny, nx = field.shape
    a = torch.from_numpy(field.astype(np.float32)).cuda()
    b = torch.empty_like(a)
    res = torch.zeros((ny, nx), dtype=torch.int16, device="cuda") if comp else None
    inj = None if injected is None else torch.from_numpy(injected.astype(np.float32)).cuda()
    s = N.amb_stencil(p.dt, p.dx, p.dy)
    m = N.amb_model(p.a, p.b, p.c, p.kappa, p.lamb, p.zeta, p.T)
    cfg = N.amb_kernel_config(kernel, seg_rows, pairs, flags)
    flag = ctypes.c_int(0)
    rc = N.lib().amb_step_f32_ex(ctypes.byref(s), ctypes.byref(m), seed, ny, nx, a.data_ptr(), b.data_ptr(),
                                 res.data_ptr() if comp else None, step0, nsteps,
                                 inj.data_ptr() if inj is not None else None, ctypes.byref(cfg),
                                 torch.cuda.current_stream().cuda_stream, ctypes.byref(flag))
    assert rc == 0, N.last_error()
    out = (b if flag.value else a).cpu().numpy().astype(np.float64)
    torch.cuda.synchronize()
    return out


AMB = dict(dt=1e-3, dx=1.0, dy=1.0, a=-0.25, b=0.0, c=0.25, kappa=1.0, lamb=0.5, zeta=-1.0)


def initial(shape, seed=0):
    rng = np.random.default_rng(seed)
    return -0.4 + 0.05 * rng.standard_normal(shape)


@pytest.mark.parametrize("shape", [(256, 256), (200, 140), (37, 340), (17, 256), (96, 448), (5, 136), (128, 128), (40, 112), (64, 116)])
@pytest.mark.parametrize("T", [0.0, 0.05])
def test_sliding_matches_tile(shape, T):
    """The tile and sliding FP32 kernels, 30 steps, plain FP32 and compensated: bitwise equal
    (the same arithmetic at every site, only the work decomposition differs)."""
    field = initial(shape, seed=shape[0])
    p = Params(T=T, **AMB)
    for comp in (False, True):
        tile = run_f32(field, p, 30, kernel=1, comp=comp)
        slid = run_f32(field, p, 30, kernel=2, comp=comp)
        assert np.isfinite(slid).all()
        assert np.array_equal(tile, slid), (comp, np.abs(tile - slid).max())


@pytest.mark.parametrize("seg_rows,pairs", [(0, 0), (16, 1), (37, 2), (100, 4), (1000, 2), (1, 1)])
def test_sliding_decomposition_is_exact(seg_rows, pairs):
    """Results do not depend on how rows are split into segments or warp pairs into CTAs
    (per-site arithmetic and Philox keys are decomposition independent): bitwise."""
    field = initial((144, 560), seed=3)
    p = Params(T=0.05, **AMB)
    ref = run_f32(field, p, 12, kernel=2, seg_rows=64, pairs=2)
    got = run_f32(field, p, 12, kernel=2, seg_rows=seg_rows, pairs=pairs)
    assert np.array_equal(ref, got)


@pytest.mark.parametrize("comp,tol", [(True, 2e-6), (False, 2e-5)])
def test_sliding_tracks_fp64_oracle(comp, tol):
    """AMB+ with Philox noise, 128 x 256, 100 steps: FP32 kernel vs the FP64 oracle with the
    same noise definition. Bounds from the FP32 rounding of field and normals."""
    field = initial((128, 256), seed=5)
    p = Params(T=0.05, **AMB)
    got = run_f32(field, p, 100, kernel=2, comp=comp, seed=11)
    ref = oracle.run(field, p, 100, noise="philox", seed=11, nthreads=4)
    assert np.abs(got - ref).max() < tol


def test_sliding_injected_noise():
    """Host-injected normals, 5 steps, FP32 compensated vs the FP64 oracle: < 1e-6."""
    rng = np.random.default_rng(8)
    field = initial((64, 272), seed=8)
    noise = rng.standard_normal((5, 2, 64, 272))
    p = Params(T=0.05, **AMB)
    got = run_f32(field, p, 5, kernel=2, comp=True, injected=noise)
    ref = oracle.run(field, p, 5, noise="injected", injected=noise.astype(np.float32).astype(np.float64))
    assert np.abs(got - ref).max() < 1e-6


def test_sliding_step_offset_and_chunking():
    """Running 20 steps as 7 + 13 (step0 carries the Philox key) equals 20 at once."""
    import torch
    field = initial((80, 224), seed=9)
    p = Params(T=0.05, **AMB)
    whole = run_f32(field, p, 20, kernel=2, comp=False)
    part = run_f32(field, p, 7, kernel=2, comp=False)
    part = run_f32(part, p, 13, kernel=2, comp=False, step0=7)
    assert np.array_equal(whole, part)
    del torch


def test_sliding_rejects_unsupported_shapes():
    import torch
    N = native()
    p = Params(T=0.0, **AMB)
    a = torch.zeros((32, 100), dtype=torch.float32, device="cuda")  # ncols < 112
    b = torch.empty_like(a)
    s = N.amb_stencil(p.dt, p.dx, p.dy)
    m = N.amb_model(p.a, p.b, p.c, p.kappa, p.lamb, p.zeta, p.T)
    cfg = N.amb_kernel_config(2, 0, 0, 0)
    rc = N.lib().amb_step_f32_ex(ctypes.byref(s), ctypes.byref(m), 0, 32, 100, a.data_ptr(), b.data_ptr(), None, 0, 1,
                                 None, ctypes.byref(cfg), torch.cuda.current_stream().cuda_stream, None)
    assert rc == N.AMB_ERR_UNSUPPORTED
    cfg = N.amb_kernel_config(0, 0, 0, 0)  # auto falls back to the tile kernel
    rc = N.lib().amb_step_f32_ex(ctypes.byref(s), ctypes.byref(m), 0, 32, 100, a.data_ptr(), b.data_ptr(), None, 0, 1,
                                 None, ctypes.byref(cfg), torch.cuda.current_stream().cuda_stream, None)
    assert rc == 0


def test_autotuner_choice_is_used_and_cached():
    """amb_autotune_f32 returns a valid configuration, caches it, and AMB_KERNEL_AUTO then
    runs exactly that configuration (bitwise equal to requesting it explicitly)."""
    import torch
    N = native()
    p = Params(T=0.05, **AMB)
    s = N.amb_stencil(p.dt, p.dx, p.dy)
    m = N.amb_model(p.a, p.b, p.c, p.kappa, p.lamb, p.zeta, p.T)
    cfg, us = N.amb_kernel_config(), ctypes.c_double()
    strm = torch.cuda.current_stream().cuda_stream
    assert N.lib().amb_autotune_f32(ctypes.byref(s), ctypes.byref(m), 96, 448, 1, 4, strm, ctypes.byref(cfg),
                                    ctypes.byref(us)) == 0, N.last_error()
    assert cfg.kernel in (N.AMB_KERNEL_TILE, N.AMB_KERNEL_SLIDING) and us.value > 0
    cfg2, us2 = N.amb_kernel_config(), ctypes.c_double()
    assert N.lib().amb_autotune_f32(ctypes.byref(s), ctypes.byref(m), 96, 448, 1, 4, strm, ctypes.byref(cfg2),
                                    ctypes.byref(us2)) == 0
    assert (cfg2.kernel, cfg2.seg_rows, cfg2.pairs_per_cta, us2.value) == (cfg.kernel, cfg.seg_rows,
                                                                           cfg.pairs_per_cta, us.value)
    field = initial((96, 448), seed=12)
    auto = run_f32(field, p, 10, kernel=0)
    explicit = run_f32(field, p, 10, kernel=cfg.kernel, seg_rows=cfg.seg_rows, pairs=cfg.pairs_per_cta)
    assert np.array_equal(auto, explicit)


def test_integrator_explicit_launch_shape():
    """Integrator(kernel="sliding" or "tile", launch=...) runs the given launch shape: bitwise
    equal to the device-pointer call with the same configuration; a tile height other than 32
    or 28 is refused."""
    from activemodelbplus.integrator import Integrator, Model, Stencil
    p = Params(T=0.05, **AMB)
    field = initial((96, 448), seed=13)
    sim = Integrator(field, Stencil(p.dt, p.dx, p.dy), Model(p.a, p.b, p.c, p.kappa, p.lamb, p.zeta, p.T),
                     precision="f32", seed=7, kernel="sliding", launch={"seg_rows": 16, "pairs_per_cta": 4})
    sim.run(10)
    ref = run_f32(field, p, 10, kernel=2, seg_rows=16, pairs=4, comp=False, seed=7)
    assert np.array_equal(sim.field, ref)
    tile = Integrator(field, Stencil(p.dt, p.dx, p.dy), Model(p.a, p.b, p.c, p.kappa, p.lamb, p.zeta, p.T),
                      precision="f32", seed=7, kernel="tile",
                      launch={"pairs_per_cta": 2, "persistent": True, "tile_rows": 28})
    tile.run(10)
    assert np.array_equal(tile.field, ref)
    with pytest.raises(ValueError):
        Integrator(field, Stencil(p.dt, p.dx, p.dy), Model(p.a, p.b, p.c, p.kappa, p.lamb, p.zeta, p.T),
                   precision="f32", kernel="tile", launch={"tile_rows": 24})


def test_kernels_match_pinned_bits():
    """Every FP32 kernel reproduces the pinned SHA-256 of the sliding kernel's output (and, for
    f32c, its residual plane), recorded on a GB300 by tests/golden/make_f32_pins.py: no kernel
    change may alter a bit of the step's results unnoticed."""
    import json
    import os
    from conftest import GOLDEN
    import sys
    sys.path.insert(0, GOLDEN)
    import make_f32_pins as M
    with open(os.path.join(GOLDEN, "f32_kernel_pins.json")) as f:
        pins = json.load(f)["pins"]
    for _, shape, comp, T in M.all_cases():
        want = pins[M.case_name("sliding", shape, comp, T)]
        for kernel in (1, 2):
            assert M.run_case(kernel, shape, comp, T) == want, (kernel, shape, comp, T)


# ------------------------------------------ tile kernel: thread groups and persistent launches

@pytest.mark.parametrize("shape", [(256, 256), (100, 72), (33, 17), (512, 512), (64, 1000)])
@pytest.mark.parametrize("groups", [1, 2, 4])
def test_tile_thread_groups_and_persistent_launch_are_bitwise(shape, groups):
    """256/512/1024 threads per CTA, 32 x 32 or 28 x 32 output tiles, one launch per step or all
    steps in one cooperative launch (grid barrier between steps): bitwise the single-step
    256-thread 32 x 32 result, for odd and even step counts (the result ends in either buffer)."""
    field = initial(shape, seed=shape[1])
    p = Params(T=0.05, **AMB)
    for comp in (False, True):
        for nsteps in (12, 13):
            ref = run_f32(field, p, nsteps, kernel=1, comp=comp)
            assert np.array_equal(run_f32(field, p, nsteps, kernel=1, pairs=groups, comp=comp), ref)
            assert np.array_equal(run_f32(field, p, nsteps, kernel=1, pairs=groups, flags=1, comp=comp), ref)
            # 28 x 32 output tiles (AMB_FLAG_TILE_ROWS_28), per step and persistent
            assert np.array_equal(run_f32(field, p, nsteps, kernel=1, pairs=groups, flags=4, comp=comp), ref)
            assert np.array_equal(run_f32(field, p, nsteps, kernel=1, pairs=groups, flags=5, comp=comp), ref)


def test_tile_persistent_injected_noise_and_fp64():
    """The persistent launch and the 28 x 32 tiles with host-injected noise (one pair of planes
    per step) and in FP64: bitwise one 32 x 32 launch per step."""
    import torch
    N = native()
    rng = np.random.default_rng(21)
    field = initial((96, 160), seed=21)
    noise = rng.standard_normal((7, 2, 96, 160))
    p = Params(T=0.05, **AMB)
    ref = run_f32(field, p, 7, kernel=1, comp=True, injected=noise)
    assert np.array_equal(run_f32(field, p, 7, kernel=1, comp=True, injected=noise, flags=1, pairs=2), ref)
    for flags in (4, 5):  # 28 x 32 tiles
        assert np.array_equal(run_f32(field, p, 7, kernel=1, comp=True, injected=noise, flags=flags, pairs=2), ref)
    s = N.amb_stencil(p.dt, p.dx, p.dy)
    m = N.amb_model(p.a, p.b, p.c, p.kappa, p.lamb, p.zeta, p.T)
    stream = torch.cuda.current_stream().cuda_stream
    outs = []
    for cfg in (None, N.amb_kernel_config(1, 0, 2, N.AMB_FLAG_PERSISTENT),
                N.amb_kernel_config(1, 0, 2, N.AMB_FLAG_TILE_ROWS_28),
                N.amb_kernel_config(1, 0, 4, N.AMB_FLAG_TILE_ROWS_28 | N.AMB_FLAG_PERSISTENT)):
        a = torch.from_numpy(field.copy()).cuda()
        b = torch.empty_like(a)
        flag = ctypes.c_int(0)
        rc = N.lib().amb_step_f64_ex(ctypes.byref(s), ctypes.byref(m), 5, 96, 160, a.data_ptr(), b.data_ptr(), 0, 9,
                                     None, ctypes.byref(cfg) if cfg is not None else None, stream, ctypes.byref(flag))
        assert rc == 0, N.last_error()
        outs.append((b if flag.value else a).cpu().numpy())
    for o in outs[1:]:
        assert np.array_equal(outs[0], o)


# ------------------------------------------------- the fused (one warp per strip) form

@pytest.mark.parametrize("shape", [(256, 256), (200, 140), (37, 340), (17, 256), (96, 448), (5, 136), (40, 112),
                                   (64, 116)])
@pytest.mark.parametrize("T", [0.0, 0.05])
def test_fused_is_bitwise_the_warp_pair(shape, T):
    """One warp per strip running every stage (AMB_FLAG_FUSED) gives the warp pair's results
    bit for bit, plain and compensated, for 1, 2 and 4 warps per CTA."""
    field = initial(shape, seed=shape[0] + 3)
    p = Params(T=T, **AMB)
    for comp in (False, True):
        ref = run_f32(field, p, 21, kernel=2, comp=comp)
        for warps in (1, 2, 4):
            got = run_f32(field, p, 21, kernel=2, comp=comp, pairs=warps, flags=2)
            assert np.array_equal(ref, got), (comp, warps, np.abs(ref - got).max())


def test_fused_injected_noise_and_segments():
    rng = np.random.default_rng(19)
    field = initial((144, 560), seed=19)
    noise = rng.standard_normal((6, 2, 144, 560))
    p = Params(T=0.05, **AMB)
    ref = run_f32(field, p, 6, kernel=2, comp=True, injected=noise)
    for seg in (1, 16, 37, 100):
        got = run_f32(field, p, 6, kernel=2, comp=True, injected=noise, seg_rows=seg, pairs=2, flags=2)
        assert np.array_equal(ref, got), seg
