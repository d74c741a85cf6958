"""Host C++ under AddressSanitizer and UndefinedBehaviorSanitizer (CPU):
the oracle over every shape and option with edge channels (NaN/Inf samples,
zero/negative/NaN pederr, huge amplitudes, a covariance that is not positive
definite), and the C++ data-file reader (include/multifit_gb300_io.hpp) on
valid zlib streams, mutated zlib streams and mutated copies of the
reference's data files. The driver is tests/cpp/sanitize_host.cpp; any
sanitizer finding aborts it (-fno-sanitize-recover=all)."""
import os
import struct
import subprocess
import zlib

import numpy as np
import pytest

from _helpers import reference_data_dir

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DATA = reference_data_dir()
FILES = [os.path.join(DATA, "mysample_100_0.000_0.000_10_25.00_10.00_0.00_1.000_1.00_CRRC43_0.00_slew_1.00.root"),
         os.path.join(DATA, "EmptyFile.root")]
ENV = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=1", UBSAN_OPTIONS="print_stacktrace=1")


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("san") / "sanitize_host")
    cmd = ["g++", "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=all",
           "-fno-omit-frame-pointer", "-ffp-contract=off", "-Wall", "-Wextra", "-Werror", "-pthread",
           "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "sanitize_host.cpp"),
           os.path.join(ROOT, "oracle", "multifit_oracle.cpp"), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and "sanitize" in r.stderr and "unrecognized" in r.stderr:
        pytest.skip("this compiler has no sanitizers")
    assert r.returncode == 0, r.stderr[-2000:]
    return out


def run(exe, *args):
    r = subprocess.run([exe, *map(str, args)], capture_output=True, text=True, env=ENV, timeout=600)
    assert r.returncode == 0 and r.stdout.startswith("ok"), (r.stdout[-500:], r.stderr[-3000:])
    return r.stdout


def test_oracle_under_sanitizers(exe):
    out = run(exe, "oracle")
    assert int(out.split()[1]) > 1000


def test_inflate_under_sanitizers(exe, tmp_path):
    rng = np.random.default_rng(9)
    path = tmp_path / "streams.bin"
    with open(path, "wb") as f:
        for d in (b"", rng.bytes(20_000), b"abcd" * 3000, np.cumsum(rng.standard_normal(3000)).astype(">f8").tobytes()):
            for level in (0, 1, 6, 9):
                for strategy in (zlib.Z_DEFAULT_STRATEGY, zlib.Z_FIXED, zlib.Z_RLE):
                    c = zlib.compressobj(level, zlib.DEFLATED, 15, 9, strategy)
                    z = c.compress(d) + c.flush()
                    f.write(struct.pack("<QQ", len(d), len(z)) + z + d)
    run(exe, "inflate", path)


@pytest.mark.parametrize("which", [0, 1])
def test_reader_fuzz_under_sanitizers(exe, which):
    if not os.path.exists(FILES[which]):
        pytest.skip("the reference's data files are absent")
    run(exe, "rootio-fuzz", FILES[which], 800, 17 + which)


SAN_DIR = os.path.join(ROOT, "test-regression_gb300", "_build", "asan")
CSRC = os.path.join(ROOT, "test-regression_gb300", "csrc")


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return None


@pytest.fixture(scope="module")
def engine_host_exe():
    """The engine's sources with host-side sanitizers (device code as PTX
    only, since no GPU runs it), cached under _build/asan, linked with
    tests/cpp/sanitize_engine_host.cpp."""
    import concurrent.futures as cf

    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc absent")
    os.makedirs(SAN_DIR, exist_ok=True)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "multifit_gb300.h")]
    newest = max(os.path.getmtime(d) for d in deps)
    srcs = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))

    def compile_one(src):
        obj = os.path.join(SAN_DIR, src.replace(".cu", ".o"))
        if os.path.exists(obj) and os.path.getmtime(obj) >= newest:
            return obj
        cmd = [nvcc, "-gencode", "arch=compute_103a,code=compute_103a", "-O1", "-g", "-std=c++17",
               "-Xcompiler", "-fPIC", "-Xcompiler", "-fsanitize=address", "-Xcompiler", "-fsanitize=undefined",
               "-Xcompiler", "-fno-sanitize-recover=all", "-Xcompiler", "-fno-omit-frame-pointer",
               "-I", os.path.join(ROOT, "include"), "-I", CSRC, *(["--fmad=false"] if src == "fit_fp64.cu" else []),
               "-c", os.path.join(CSRC, src), "-o", obj + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-2000:]
        os.replace(obj + ".tmp", obj)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    exe = os.path.join(SAN_DIR, "sanitize_engine_host")
    cuda_lib = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "lib64")
    cmd = ["g++", "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=all",
           "-fno-omit-frame-pointer", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "sanitize_engine_host.cpp"), *objs, "-L", cuda_lib, "-lcudart",
           "-lpthread", f"-Wl,-rpath,{cuda_lib}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return exe


def test_engine_host_code_under_sanitizers(engine_host_exe, cuda_absent):
    """Argument checks, the pulse-matrix rule, all 1023 + 255 operator tables,
    the host generator and the device entry points' error paths (no GPU)."""
    run(engine_host_exe)


@pytest.fixture(scope="module")
def cuda_absent():
    # with a GPU present the driver's device entry points would run kernels
    # from a sanitizer build; this test is for the host paths only
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: the host-only driver is meant for machines without one")
