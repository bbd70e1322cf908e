"""Generate the golden fixtures in tests/golden/ from the reference's own CPU scheme.

Runs ``test/tjhung_ambplus.h`` of the reference (compiled into ``oracle/_ref`` by
``oracle/build.py`` from the read-only reference checkout) on seeded inputs and
stores its outputs. The reference itself is not needed to USE the fixtures:
they let the oracle and the CUDA library be checked where the reference
checkout is absent.

Fixtures
  tjhung_onestep_64x32.npz   the reference's parity-pin case (test/test_tjhung.cc:10-40):
                             64x32, dt=1e-2, A=0.25, K=1, lambda=zeta=1, T=0;
                             initial U[-1,1) (numpy seed 2024); one calculate_dphi:
                             dphi, mueq, muact, J*eq, J*act.
  tjhung_spinodal_256.npz    Model B spinodal, 256x256, dt=1e-3, a=-0.25 b=0 c=0.25 kappa=1,
                             phi = 0.1 U[0,1) (numpy seed 7), mean shifted to 0; 10^4 steps.
                             Stores the initial field, every 4th row/column of the final
                             field, and the final field's sum, sum of squares and max |phi|.
  tjhung_active_64.npz       AMB+ 64x64, dt=1e-2, A=0.25, K=1, lambda=-1, zeta=-4, T=0,
                             phi = -0.4 + 0.1 (U[0,1) - 1/2) (numpy seed 11); 500 steps; full field.

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))

import oracle  # noqa: E402


def spinodal_initial() -> np.ndarray:
    rng = np.random.default_rng(7)
    phi = 0.1 * rng.random((256, 256))
    return phi - phi.mean()


def onestep_initial() -> np.ndarray:
    rng = np.random.default_rng(2024)
    return rng.uniform(-1.0, 1.0, (64, 32))


def active_initial() -> np.ndarray:
    rng = np.random.default_rng(11)
    return -0.4 + 0.1 * (rng.random((64, 64)) - 0.5)


def main() -> None:
    if oracle.reference_lib() is None:
        raise SystemExit("the reference CPU scheme could not be built here")

    phi = onestep_initial()
    out = oracle.tjhung_dphi(phi, dt=1e-2, h=1.0, A=0.25, K=1.0, lamb=1.0, zeta=1.0)
    np.savez(os.path.join(HERE, "tjhung_onestep_64x32.npz"), initial=phi, dt=1e-2, A=0.25, K=1.0, lamb=1.0,
             zeta=1.0, **out)

    phi = spinodal_initial()
    final = oracle.tjhung_run(phi, 10000, dt=1e-3, h=1.0, A=0.25, K=1.0, lamb=0.0, zeta=0.0)
    np.savez(os.path.join(HERE, "tjhung_spinodal_256.npz"), initial=phi, nsteps=10000, dt=1e-3,
             final_sub=final[::4, ::4], final_sum=final.sum(), final_sumsq=(final ** 2).sum(),
             final_absmax=np.abs(final).max())

    phi = active_initial()
    final = oracle.tjhung_run(phi, 500, dt=1e-2, h=1.0, A=0.25, K=1.0, lamb=-1.0, zeta=-4.0)
    np.savez(os.path.join(HERE, "tjhung_active_64.npz"), initial=phi, nsteps=500, dt=1e-2, lamb=-1.0, zeta=-4.0,
             final=final)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
