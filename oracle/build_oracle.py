"""Build recipe for the CPU oracle (test infrastructure).

* ``oracle/_build/liboracle.so``: the C++17 FP64 restatement of the reference
  path (multifit_oracle.cpp) and the seeded synthetic-channel generator
  (synth_oracle.cpp), built with ``-ffp-contract=off`` so that only explicit
  ``std::fma`` calls fuse. Built on every machine.
* ``oracle/_ref/libref_linalgebra.so``: the reference project's own
  header-only linear-algebra primitives (``linalgebra/interface/*.hpp``),
  compiled in place from the reference tree with a small driver
  (ref_linalgebra_driver.cpp). Built only where the reference tree exists.
  gcc contracts each ``acc += a*b`` of those headers into one fused
  multiply-add (``-ffp-contract=fast``, FMA hardware, and the
  ``avoid-fma-max-bits`` heuristic off), which is the oracle's canonical
  order; the tests check that claim bit for bit.

* ``oracle/_build/liboracle_sep.so``: the same restatement built with
  ``ORACLE_SEPARATE_ROUNDING`` (each product and sum of an FMA expression
  rounded on its own), for the pin below.
* ``oracle/_ref/libref_ocl_fnnls_f64.so`` / ``_f32.so``: the reference's own
  plain-C twin of the incremental-Cholesky FNNLS, the OpenCL kernel source
  ``multifit_ocl/device/regression_inplace_fnnls.cl``, compiled unmodified as
  C through ref_ocl_fnnls_driver.c with ``-ffp-contract=off`` (the source's
  own roundings): once with its ``data_type`` float as written and once with
  float mapped to double. Built only where the reference tree exists. The
  FP64 build equals liboracle_sep.so's incremental FNNLS bit for bit.

* ``oracle/_ref/libref_dofit.so``: the reference's own multifit_cpu fit,
  ``multifit_cpu/src/PulseChiSqSNNLS.cpp`` (DoFit, Minimize, updateCov, NNLS,
  ComputeChiSq, ComputeApproxUncertainty) and ``nnls/src/inplace_fnnls.cu``,
  compiled unmodified through ref_dofit_driver.cpp. Both include Eigen, which
  the reference does not vendor and which is absent here: ``eigen_shim/``
  provides the small part of its API they use, with the oracle's canonical
  arithmetic order, and ``eigen_shim_stubs/`` an empty stand-in for the
  vendored Eigen NNLS module the fit includes but never calls. Built with
  ``-O3 -ffp-contract=fast`` (and FMA on x86) so that gcc fuses the
  accumulations written in the reference's own loops (transpose_multiply's
  ``+=``), as the oracle does; ``-fsigned-char`` because the fit keeps its
  BX offsets in plain char. Built only where the reference tree exists.

The reference tree is read from MULTIFIT_REFERENCE_ROOT, by default a
checkout named ``reference`` beside the repository's root; where it is
absent, every _ref library is skipped and the tests fall back on the
committed outputs in tests/golden/.
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
REFERENCE_ROOT = os.environ.get("MULTIFIT_REFERENCE_ROOT",
                                os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))

ORACLE_LIB = os.path.join(BUILD, "liboracle.so")
ORACLE_SEP_LIB = os.path.join(BUILD, "liboracle_sep.so")
REF_LIB = os.path.join(REF_OUT, "libref_linalgebra.so")
REF_DOFIT_LIB = os.path.join(REF_OUT, "libref_dofit.so")
REF_OCL_LIBS = {64: os.path.join(REF_OUT, "libref_ocl_fnnls_f64.so"),
                32: os.path.join(REF_OUT, "libref_ocl_fnnls_f32.so")}


def _fma_flag() -> list[str]:
    # x86 needs -mfma for the instruction; gcc's avoid-fma-max-bits heuristic
    # otherwise leaves loop-carried accumulations unfused, so it is switched off.
    if platform.machine() in ("x86_64", "AMD64"):
        return ["-mfma", "--param=avoid-fma-max-bits=0"]
    return []


def _stale(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _build_oracle_lib(target: str, defines: list[str], force: bool) -> str:
    srcs = [os.path.join(HERE, "multifit_oracle.cpp"), os.path.join(HERE, "synth_oracle.cpp")]
    if force or _stale(target, [*srcs, __file__]):
        os.makedirs(BUILD, exist_ok=True)
        tmp = target + ".tmp"
        cmd = ["g++", "-std=c++17", "-O3", "-ffp-contract=off", "-fPIC", "-shared", "-pthread", *defines,
               *srcs, "-o", tmp]
        subprocess.check_call(cmd)
        os.replace(tmp, target)
    return target


def build_oracle(force: bool = False) -> str:
    return _build_oracle_lib(ORACLE_LIB, [], force)


def build_oracle_separate(force: bool = False) -> str:
    return _build_oracle_lib(ORACLE_SEP_LIB, ["-DORACLE_SEPARATE_ROUNDING"], force)


def build_ref_ocl(force: bool = False) -> dict | None:
    """The reference's OpenCL FNNLS compiled as C, {64: path, 32: path}, or
    None where the reference tree is absent."""
    dev = os.path.join(REFERENCE_ROOT, "multifit_ocl", "device")
    cl = os.path.join(dev, "regression_inplace_fnnls.cl")
    if not os.path.exists(cl):
        return None
    src = os.path.join(HERE, "ref_ocl_fnnls_driver.c")
    for bits, target in REF_OCL_LIBS.items():
        if force or _stale(target, [src, __file__]):
            os.makedirs(REF_OUT, exist_ok=True)
            tmp = target + ".tmp"
            cmd = ["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                   *(["-DMF_REF_OCL_DOUBLE"] if bits == 64 else []), "-I", dev, "-x", "c", src, "-o", tmp, "-lm"]
            subprocess.check_call(cmd)
            os.replace(tmp, target)
    return dict(REF_OCL_LIBS)


def build_ref(force: bool = False) -> str | None:
    inc = os.path.join(REFERENCE_ROOT, "linalgebra", "interface")
    if not os.path.isdir(inc):
        return None
    src = os.path.join(HERE, "ref_linalgebra_driver.cpp")
    if force or _stale(REF_LIB, [src, __file__]):
        os.makedirs(REF_OUT, exist_ok=True)
        tmp = REF_LIB + ".tmp"
        cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=fast", *_fma_flag(), "-fPIC", "-shared",
               "-I", inc, src, "-o", tmp]
        subprocess.check_call(cmd)
        os.replace(tmp, REF_LIB)
    return REF_LIB


def build_ref_dofit(force: bool = False) -> str | None:
    """The reference's multifit_cpu fit compiled over the Eigen shim, or None
    where the reference tree is absent."""
    src_cpp = os.path.join(REFERENCE_ROOT, "multifit_cpu", "src", "PulseChiSqSNNLS.cpp")
    if not os.path.exists(src_cpp):
        return None
    shim = os.path.join(HERE, "eigen_shim", "Eigen", "Dense")
    stub = os.path.join(HERE, "eigen_shim_stubs", "nnls", "interface", "eigen_nnls.h")
    drv = os.path.join(HERE, "ref_dofit_driver.cpp")
    if force or _stale(REF_DOFIT_LIB, [drv, shim, stub, __file__]):
        os.makedirs(REF_OUT, exist_ok=True)
        tmp = REF_DOFIT_LIB + ".tmp"
        cmd = ["g++", "-std=c++17", "-O3", "-ffp-contract=fast", *_fma_flag(), "-fsigned-char", "-Wno-unknown-pragmas",
               "-fPIC", "-shared", "-I", os.path.join(HERE, "eigen_shim"), "-iquote",
               os.path.join(HERE, "eigen_shim_stubs"), "-I", REFERENCE_ROOT, drv, "-o", tmp]
        subprocess.check_call(cmd)
        os.replace(tmp, REF_DOFIT_LIB)
    return REF_DOFIT_LIB


def main() -> int:
    force = "--force" in sys.argv
    print(build_oracle(force))
    print(build_ref(force) or "reference tree absent: oracle/_ref not built")
    print(build_oracle_separate(force))
    print(build_ref_ocl(force) or "reference tree absent: OpenCL FNNLS not built")
    print(build_ref_dofit(force) or "reference tree absent: reference DoFit not built")
    return 0


if __name__ == "__main__":
    sys.exit(main())
