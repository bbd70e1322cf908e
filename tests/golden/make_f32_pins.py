"""Bitwise pins of the FP32 step kernels' output on a GB300 (sm_103a).

The FP32 kernels are deterministic: the same field, parameters, Philox key and step
count give the same bits on the same GPU architecture (their hardware approximations of
log, rsqrt, sin and cos are fixed per architecture). This script records the SHA-256 of
the output of each FP32 kernel (tile, sliding) in each storage mode (plain FP32 and the
compensated f32c, whose residual plane is hashed too), at T = 0 and T = 0.05, on two
shapes, into ``f32_kernel_pins.json``. ``tests/test_gpu_kernels.py`` recomputes them, so a
change to any kernel that alters a single bit of its results shows up, and any new kernel
that claims the same arithmetic can be held to the same pins.

Inputs: the AMB+ parameters of the bench workload (dt=1e-3, a=-0.25, b=0, c=0.25, kappa=1,
zeta=-1, lambda=0.5), phi = -0.4 + 0.05 N(0,1) (numpy seed = nrows), Philox seed 7, 40 steps.

Usage (needs the GPU): python tests/golden/make_f32_pins.py [output.json]
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
for _p in (ROOT, os.path.join(ROOT, "active-model-bplus_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

SHAPES = ((256, 256), (200, 336))
STEPS = 40
PARAMS = dict(dt=1e-3, dx=1.0, dy=1.0, a=-0.25, b=0.0, c=0.25, kappa=1.0, lamb=0.5, zeta=-1.0)
KERNELS = {"tile": 1, "sliding": 2}


def case_name(kernel: str, shape, comp: bool, T: float) -> str:
    return f"{kernel}_{shape[0]}x{shape[1]}_{'f32c' if comp else 'f32'}_T{T}"


def run_case(kernel_id: int, shape, comp: bool, T: float) -> str:
    """SHA-256 of the output field (float32 bytes) and, for f32c, of the residual plane."""
    import torch
    from activemodelbplus.integrator import _native as N
    ny, nx = shape
    rng = np.random.default_rng(ny)
    field = (-0.4 + 0.05 * rng.standard_normal(shape)).astype(np.float32)
    a = torch.from_numpy(field).cuda()
    b = torch.empty_like(a)
    res = torch.zeros(shape, dtype=torch.int16, device="cuda") if comp else None
    s = N.amb_stencil(PARAMS["dt"], PARAMS["dx"], PARAMS["dy"])
    m = N.amb_model(PARAMS["a"], PARAMS["b"], PARAMS["c"], PARAMS["kappa"], PARAMS["lamb"], PARAMS["zeta"], T)
    cfg = N.amb_kernel_config(kernel_id, 0, 0, 0)
    flag = ctypes.c_int(0)
    rc = N.lib().amb_step_f32_ex(ctypes.byref(s), ctypes.byref(m), 7, ny, nx, a.data_ptr(), b.data_ptr(),
                                 res.data_ptr() if comp else None, 0, STEPS, None, ctypes.byref(cfg),
                                 torch.cuda.current_stream().cuda_stream, ctypes.byref(flag))
    if rc:
        raise RuntimeError(N.last_error())
    out = (b if flag.value else a).cpu().numpy()
    h = hashlib.sha256(out.tobytes())
    if comp:
        h.update(res.cpu().numpy().tobytes())
    return h.hexdigest()


def all_cases():
    for kernel in KERNELS:
        for shape in SHAPES:
            for comp in (False, True):
                for T in (0.0, 0.05):
                    yield kernel, shape, comp, T


def main(path: str) -> None:
    pins = {case_name(k, sh, c, T): run_case(KERNELS[k], sh, c, T) for k, sh, c, T in all_cases()}
    with open(path, "w") as f:
        json.dump({"steps": STEPS, "shapes": SHAPES, "params": PARAMS, "pins": pins}, f, indent=1)
    print(f"wrote {len(pins)} pins to {path}")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "f32_kernel_pins.json"))
