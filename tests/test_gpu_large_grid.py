"""Fields past 2^31 sites on the GPU: 64-bit indexing in every kernel a step touches.

A 32 800 x 65 536 FP32-compensated field (2.15e9 sites, 8.6 GB per buffer) that is constant
along y: every y difference is then exactly zero, so each row of the result is bitwise the row
that a 64-row field with the same x profile gives, whatever the row's offset in memory. The
warp-pair kernel and the tile kernel each take two deterministic AMB+ steps (zeta = -4,
lambda = -1, T = 0); the finite check and the compensated FP64 mass then run over the whole
field (mass = ny x the row sum, to FP64 rounding).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NY, NX = 32800, 65536


def _run(N, torch, field, res, ny, kernel, pairs, nsteps=2):
    s = N.amb_stencil(1e-3, 1, 1)
    m = N.amb_model(-0.25, 0, 0.25, 1, -1, -4, 0.0)
    spare = torch.empty_like(field)
    cfg = N.amb_kernel_config(kernel, 0, pairs, 0)
    flag = ctypes.c_int(0)
    rc = N.lib().amb_step_f32_ex(ctypes.byref(s), ctypes.byref(m), 3, ny, NX, field.data_ptr(), spare.data_ptr(),
                                 res.data_ptr(), 0, nsteps, None, ctypes.byref(cfg),
                                 torch.cuda.current_stream().cuda_stream, ctypes.byref(flag))
    assert rc == 0, N.last_error()
    return spare if flag.value else field


@pytest.mark.parametrize("kernel,pairs", [(2, 4), (1, 2)])  # warp pairs (4 per CTA); tile kernel (512 threads)
def test_step_kernels_index_past_2_31_sites(kernel, pairs):
    import torch
    from activemodelbplus.integrator import _native as N
    assert NY * NX > 2 ** 31
    x = np.arange(NX)
    row = (-0.4 + 0.05 * np.sin(2 * np.pi * 3 * x / NX)
           + 0.01 * np.random.default_rng(11).standard_normal(NX)).astype(np.float32)
    row_dev = torch.from_numpy(row).cuda()
    # reference: 64 rows of the same profile
    small = row_dev.expand(64, NX).contiguous()
    small_res = torch.zeros((64, NX), dtype=torch.int16, device="cuda")
    want = _run(N, torch, small, small_res, 64, kernel, pairs)
    want_row, want_res = want[0].clone(), small_res[0].clone()
    assert torch.equal(want, want_row.expand(64, NX)) and torch.equal(small_res, want_res.expand(64, NX))
    del small, small_res, want
    big = row_dev.expand(NY, NX).contiguous()
    big_res = torch.zeros((NY, NX), dtype=torch.int16, device="cuda")
    try:
        got = _run(N, torch, big, big_res, NY, kernel, pairs)
        assert torch.equal(got, want_row.expand(NY, NX)), "rows differ from the 64-row run"
        assert torch.equal(big_res, want_res.expand(NY, NX)), "residual rows differ"
        # finite check and FP64 compensated mass over all 2.15e9 sites
        n = NY * NX
        flag = torch.zeros(1, dtype=torch.int32, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        assert N.lib().amb_check_finite_f32(got.data_ptr(), n, flag.data_ptr(), stream) == 0
        nbytes = N.lib().amb_mass_scratch_bytes(n)
        scratch = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        out = torch.zeros(1, dtype=torch.float64, device="cuda")
        assert N.lib().amb_mass_f32(got.data_ptr(), n, out.data_ptr(), scratch.data_ptr(), nbytes, stream) == 0
        torch.cuda.synchronize()
        assert int(flag.item()) == 0
        row_sum = float(want_row.double().sum().item())
        assert abs(out.item() - NY * row_sum) <= 1e-9 * NY * float(want_row.double().abs().sum().item())
    finally:
        del big, big_res
        got = None
        torch.cuda.empty_cache()
