"""Build recipe for the oracle (test infrastructure, not the product).

* ``oracle/_build/libamb_oracle.so`` — the C restatement (``amb_oracle.c``),
  IEEE double arithmetic (no fast-math), optional OpenMP.
* ``oracle/_ref/libtjhung_ref.so`` and ``libtjhung_ref_fast.so`` — the
  reference's own CPU scheme ``test/tjhung_ambplus.h`` compiled through
  ``tjhung_ref_driver.cc`` with the self-written Eigen stand-in. ``-O2`` for
  parity pins; ``-Ofast`` (the reference's CMAKE_CXX_FLAGS, CMakeLists.txt:21)
  for the timed CPU baseline.

The reference checkout is found through ``AMB_REFERENCE_ROOT`` or, failing
that, as the directory ``reference`` beside the repository. Where it exists,
the two reference files the CPU scheme needs (``test/tjhung_ambplus.h`` and
``src/math_primitives.h``) are staged unmodified into ``oracle/_ref/src/``
(git-ignored, like every other file under ``oracle/_ref``) and compiled from
there, so a machine without the checkout (a GPU host of another architecture)
compiles the same scheme natively from the staged copy. Nothing under
``oracle/_ref`` is committed.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
REPO_ROOT = os.path.dirname(HERE)
REFERENCE_ROOT = os.environ.get("AMB_REFERENCE_ROOT") or os.path.join(os.path.dirname(REPO_ROOT), "reference")
STAGED_SRC = os.path.join(REF_DIR, "src")  # staged copy of the reference files the CPU scheme needs
STAGED_FILES = (os.path.join("test", "tjhung_ambplus.h"), os.path.join("src", "math_primitives.h"))

ORACLE_LIB = os.path.join(BUILD_DIR, "libamb_oracle.so")
REF_GPU_DRIVER = os.path.join(BUILD_DIR, "libref_gpu_driver.so")
REF_GPU_CUBIN = os.path.join(REF_DIR, "ref_integrator.cubin")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
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


def stage_reference_sources() -> bool:
    """Copy the reference files the CPU scheme needs into oracle/_ref/src (unmodified).
    Returns whether a staged copy exists afterwards."""
    if reference_available():
        import shutil
        for rel in STAGED_FILES:
            src, dst = os.path.join(REFERENCE_ROOT, rel), os.path.join(STAGED_SRC, rel)
            if not os.path.exists(dst) or os.path.getmtime(src) > os.path.getmtime(dst):
                os.makedirs(os.path.dirname(dst), exist_ok=True)
                shutil.copy2(src, dst)
    return all(os.path.exists(os.path.join(STAGED_SRC, rel)) for rel in STAGED_FILES)


def _loads(lib: str) -> bool:
    """Whether a built library loads on this machine (a copy built for another architecture does not)."""
    import ctypes
    try:
        ctypes.CDLL(lib)
        return True
    except OSError:
        return False


def build_reference(force: bool = False) -> list[str]:
    """Compile the reference's CPU scheme into oracle/_ref from the staged sources (staged here
    from the reference checkout where it exists; on other machines the staged copy that came
    with the repository copy is compiled natively)."""
    if not stage_reference_sources():
        return []
    os.makedirs(REF_DIR, exist_ok=True)
    driver = os.path.join(HERE, "tjhung_ref_driver.cc")
    standin = os.path.join(HERE, "eigen_standin")
    header = os.path.join(STAGED_SRC, "test", "tjhung_ambplus.h")
    built = []
    for lib, opt in ((TJHUNG_LIB, ["-O2", "-ffp-contract=off"]), (TJHUNG_FAST_LIB, ["-Ofast"])):
        if force or _stale(lib, [driver, header, os.path.join(standin, "Eigen", "Eigen"), __file__]) \
                or not _loads(lib):
            tmp = lib + f".tmp{os.getpid()}"
            _run(["g++", "-std=c++20", *opt, "-fPIC", "-shared",
                  "-I", os.path.join(STAGED_SRC, "test"), "-I", os.path.join(STAGED_SRC, "src"),
                  "-I", standin, driver, "-o", tmp])
            os.replace(tmp, lib)
        built.append(lib)
    return built


def build_reference_gpu_cubin(force: bool = False) -> str | None:
    """The reference's own device code (src/integrator.cu + src/parameters.cu), compiled with its
    CMake flags (CMakeLists.txt:15-22) for sm_103a and device-linked into one cubin. Only where
    the reference checkout exists; the cubin then travels with the repository copy."""
    if not reference_available():
        return REF_GPU_CUBIN if os.path.exists(REF_GPU_CUBIN) else None
    srcs = [os.path.join(REFERENCE_ROOT, "src", f) for f in ("integrator.cu", "parameters.cu")]
    if not force and not _stale(REF_GPU_CUBIN, srcs + [__file__]):
        return REF_GPU_CUBIN
    os.makedirs(REF_DIR, exist_ok=True)
    nvcc = os.path.join(CUDA_HOME, "bin", "nvcc")
    objs = []
    for src in srcs:
        obj = os.path.join(REF_DIR, os.path.basename(src) + ".rdc.cubin")
        _run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++20", "-O3", "--expt-relaxed-constexpr",
              "-diag-suppress", "20012", "--use_fast_math", "-ftz=true", "-prec-div=false", "-prec-sqrt=false",
              "-rdc=true", "-cubin", "-I", os.path.join(REFERENCE_ROOT, "src"), "-I", os.path.join(HERE, "eigen_standin"),
              src, "-o", obj])
        objs.append(obj)
    tmp = REF_GPU_CUBIN + f".tmp{os.getpid()}"
    _run([os.path.join(CUDA_HOME, "bin", "nvlink"), "--arch=sm_103a", *objs, "-o", tmp])
    os.replace(tmp, REF_GPU_CUBIN)
    for o in objs:
        os.remove(o)
    return REF_GPU_CUBIN


def build_ref_gpu_driver(force: bool = False) -> str:
    """Host driver (our own code, CUDA driver API) that runs the reference's cubin."""
    src = os.path.join(HERE, "ref_gpu_driver.cc")
    os.makedirs(BUILD_DIR, exist_ok=True)
    if force or _stale(REF_GPU_DRIVER, [src, __file__]):
        tmp = REF_GPU_DRIVER + f".tmp{os.getpid()}"
        _run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-I", os.path.join(CUDA_HOME, "include"), src,
              "-o", tmp, "-L", os.path.join(CUDA_HOME, "lib64", "stubs"), "-lcuda"])
        os.replace(tmp, REF_GPU_DRIVER)
    return REF_GPU_DRIVER


def build_all(force: bool = False) -> None:
    build_oracle(force)
    build_reference(force)
    build_reference_gpu_cubin(force)
    build_ref_gpu_driver(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("oracle built:", ORACLE_LIB, "| reference:", build_reference())
