"""amb_mass_f32_noalloc: the mass reduction for callers that cannot allocate device
memory (an allocator that already owns the device, a plugin handed only device
pointers, a loop that cannot pay for cudaMalloc's synchronization). Its scratch is a
static device array shared by all calls, so this file is collected last: a failure
here cannot stop the rest of the suite from running first.

Checked through the C ABI against amb_mass_f32 (caller scratch) on two calls in a row
with different fields; both are FP64 compensated sums of the same FP32 values in
different orders, compared at 1e-12 relative."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mass_with_scratch(N, torch, field, stream):
    nbytes = N.lib().amb_mass_scratch_bytes(field.numel())
    scratch = torch.empty((nbytes + 7) // 8, dtype=torch.float64, device="cuda")
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    rc = N.lib().amb_mass_f32(field.data_ptr(), field.numel(), out.data_ptr(), scratch.data_ptr(), nbytes, stream)
    assert rc == 0, N.last_error()
    return out


def test_noalloc_mass_matches_scratch_mass_twice():
    import torch
    from activemodelbplus.integrator import _native as N
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(31)
    for shape in ((4096, 4096), (1000, 777)):
        host = (-0.4 + 0.05 * rng.standard_normal(shape)).astype(np.float32)
        field = torch.from_numpy(host).cuda()
        out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        rc = N.lib().amb_mass_f32_noalloc(field.data_ptr(), field.numel(), out.data_ptr(), stream)
        assert rc == 0, N.last_error()
        ref = _mass_with_scratch(N, torch, field, stream)
        got, want = float(out.item()), float(ref.item())
        assert abs(got - want) <= 1e-12 * abs(want)
        assert abs(got - float(host.astype(np.float64).sum())) <= 1e-9 * abs(want)


def test_noalloc_mass_rejects_fields_beyond_its_scratch():
    import torch
    from activemodelbplus.integrator import _native as N
    small = torch.zeros(16, dtype=torch.float32, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = N.lib().amb_mass_f32_noalloc(small.data_ptr(), (1 << 30) + 1, out.data_ptr(),
                                      torch.cuda.current_stream().cuda_stream)
    assert rc == N.AMB_ERR_INVALID
    assert "2^30" in N.last_error()
