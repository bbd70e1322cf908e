"""Build recipe for the oracle (test infrastructure, not the product).

* ``oracle/_build/libamb_oracle.so`` — the C restatement (``amb_oracle.c``),
  IEEE double arithmetic (no fast-math), optional OpenMP.
* ``oracle/_ref/libtjhung_ref.so`` and ``libtjhung_ref_fast.so`` — the
  reference's own CPU scheme ``test/tjhung_ambplus.h`` compiled from the
  read-only reference checkout through ``tjhung_ref_driver.cc`` with the
  self-written Eigen stand-in. ``-O2`` for parity pins; ``-Ofast`` (the
  reference's CMAKE_CXX_FLAGS, CMakeLists.txt:21) for the timed CPU baseline.
  Built only where the reference checkout exists; elsewhere the prebuilt
  files (if any) are used as they are.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
REFERENCE_ROOT = os.environ.get("AMB_REFERENCE_ROOT", "/root/reference")

ORACLE_LIB = os.path.join(BUILD_DIR, "libamb_oracle.so")
TJHUNG_LIB = os.path.join(REF_DIR, "libtjhung_ref.so")
TJHUNG_FAST_LIB = os.path.join(REF_DIR, "libtjhung_ref_fast.so")


def _stale(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources if os.path.exists(s))


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + proc.stdout + proc.stderr)


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "amb_oracle.c")
    os.makedirs(BUILD_DIR, exist_ok=True)
    if force or _stale(ORACLE_LIB, [src, __file__]):
        tmp = ORACLE_LIB + f".tmp{os.getpid()}"
        _run(["gcc", "-std=c11", "-O2", "-fno-fast-math", "-ffp-contract=off", "-fopenmp",
              "-fPIC", "-shared", src, "-o", tmp, "-lm"])
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def reference_available() -> bool:
    return os.path.exists(os.path.join(REFERENCE_ROOT, "test", "tjhung_ambplus.h"))


def build_reference(force: bool = False) -> list[str]:
    """Compile the reference's CPU scheme into oracle/_ref (only where the checkout exists)."""
    if not reference_available():
        return []
    os.makedirs(REF_DIR, exist_ok=True)
    driver = os.path.join(HERE, "tjhung_ref_driver.cc")
    standin = os.path.join(HERE, "eigen_standin")
    header = os.path.join(REFERENCE_ROOT, "test", "tjhung_ambplus.h")
    built = []
    for lib, opt in ((TJHUNG_LIB, ["-O2", "-ffp-contract=off"]), (TJHUNG_FAST_LIB, ["-Ofast"])):
        if force or _stale(lib, [driver, header, os.path.join(standin, "Eigen", "Eigen"), __file__]):
            tmp = lib + f".tmp{os.getpid()}"
            _run(["g++", "-std=c++20", *opt, "-fPIC", "-shared",
                  "-I", os.path.join(REFERENCE_ROOT, "test"), "-I", os.path.join(REFERENCE_ROOT, "src"),
                  "-I", standin, driver, "-o", tmp])
            os.replace(tmp, lib)
        built.append(lib)
    return built


def build_all(force: bool = False) -> None:
    build_oracle(force)
    build_reference(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("oracle built:", ORACLE_LIB, "| reference:", build_reference())
