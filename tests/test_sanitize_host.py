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

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DATA = os.path.join(os.environ.get("MULTIFIT_REFERENCE_ROOT", "/root/reference"), "data")
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
