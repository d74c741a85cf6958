"""The C++ reader of the reference's data files (include/multifit_gb300_io.hpp,
driven by tests/cpp/rootio_check.cpp) on the CPU: its zlib decoder against
Python's zlib over every compression level and strategy, and its reading of
the reference's files against the fixture the Python reader made
(tests/golden/replay_mysample_100.npz), bit for bit."""
import os
import struct
import subprocess
import zlib

import numpy as np
import pytest

from _helpers import reference_data_dir

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "replay_mysample_100.npz")
DATA = reference_data_dir()
SAMPLE_100 = os.path.join(DATA, "mysample_100_0.000_0.000_10_25.00_10.00_0.00_1.000_1.00_CRRC43_0.00_slew_1.00.root")
SAMPLE_1000 = os.path.join(DATA,
                           "mysample_1000_0.000_0.000_10_25.00_10.00_0.00_1.000_1.00_CRRC43_0.00_slew_1.00.root")
SHAPE = os.path.join(DATA, "EmptyFile.root")
needs_data = pytest.mark.skipif(not (os.path.exists(SAMPLE_100) and os.path.exists(SHAPE)),
                                reason="the reference's data files are absent")


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("rootio") / "rootio_check")
    for extra in ((), ("-funsigned-char",)):  # plain char is unsigned on Arm
        subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", *extra, "-I",
                        os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "rootio_check.cpp"),
                        "-o", out], check=True, capture_output=True)
    return out


def run(exe, *args):
    # messages may quote mutated (non-UTF-8) names
    return subprocess.run([exe, *map(str, args)], capture_output=True, text=True, errors="replace")


def test_inflate_matches_zlib(exe, tmp_path):
    rng = np.random.default_rng(7)
    datas = [b"", b"x", b"abcabcabcabc" * 3, rng.bytes(70_000), bytes(100_000), b"0123456789" * 5000,
             np.cumsum(rng.standard_normal(20_000)).astype(">f8").tobytes(),
             rng.integers(0, 4, 50_000, dtype=np.uint8).tobytes()]
    strategies = (zlib.Z_DEFAULT_STRATEGY, zlib.Z_FILTERED, zlib.Z_HUFFMAN_ONLY, zlib.Z_RLE, zlib.Z_FIXED)
    path = tmp_path / "streams.bin"
    n = 0
    with open(path, "wb") as f:
        for d in datas:
            for level in range(10):
                for strategy in strategies:
                    c = zlib.compressobj(level, zlib.DEFLATED, 15, 9, strategy)
                    z = c.compress(d) + c.flush()
                    f.write(struct.pack("<QQ", len(d), len(z)) + z + d)
                    n += 1
    r = run(exe, "inflate", path)
    assert r.returncode == 0 and r.stdout.strip() == f"ok {n}", r.stdout


def test_inflate_rejects_corrupt_stream(exe, tmp_path):
    d = b"the quick brown fox " * 200
    z = bytearray(zlib.compress(d, 6))
    z[-1] ^= 1  # Adler-32
    path = tmp_path / "bad.bin"
    path.write_bytes(struct.pack("<QQ", len(d), len(z)) + bytes(z) + d)
    r = run(exe, "inflate", path)
    assert r.returncode == 2 and "Adler-32" in r.stdout


@pytest.mark.parametrize("level", [0, 1, 6, 9])
def test_inflate_stops_at_the_declared_size(exe, tmp_path, level):
    """A stream that inflates to more than its record declares is refused as
    soon as its output passes the declared size (stored, literal and
    back-reference output alike), not after it has been decoded whole."""
    d = b"0123456789" * 20_000 + bytes(range(256)) * 40
    z = zlib.compress(d, level)
    declared = len(d) // 3
    path = tmp_path / "over.bin"
    path.write_bytes(struct.pack("<QQ", declared, len(z)) + z + d[:declared])
    r = run(exe, "inflate", path)
    assert r.returncode == 2 and "exceeds the declared size" in r.stdout, r.stdout


@needs_data
def test_cpp_reader_matches_python_reader_fixture(exe, tmp_path):
    g = dict(np.load(GOLDEN))
    out = tmp_path / "dump.bin"
    r = run(exe, "dump", SAMPLE_100, SHAPE, out)
    assert r.returncode == 0, r.stdout
    b = out.read_bytes()
    n = struct.unpack_from("=q", b, 0)[0]
    assert n == 100
    f = np.frombuffer(b, dtype=np.float64, offset=8, count=n * 10 + n + 19 + 100 + 100 + 3)
    p = 0
    for name, size, shape in (("samples", n * 10, (n, 10)), ("truth", n, (n,)), ("fullpulse", 19, (19,)),
                              ("noisecor", 100, (10, 10)), ("P", 100, (10, 10)), ("tail", 3, (3,))):
        arr = f[p:p + size].reshape(shape)
        if name == "P":
            arr = arr.reshape(10, 10).T  # column-major
        assert np.array_equal(arr, g[name]), name
        p += size
    npts, srt = struct.unpack_from("=qq", b, 8 + 8 * p)
    assert npts == int(g["graph_points"]) and bool(srt) == bool(g["graph_sorted"])


@needs_data
def test_cpp_reader_errors(exe):
    if os.path.exists(SAMPLE_1000):
        r = run(exe, "expect-error", SAMPLE_1000, "Samples", "samples", "not closed")
        assert r.returncode == 0, r.stdout
    r = run(exe, "expect-error", SAMPLE_100, "Samples", "no_such_branch", "no baskets")
    assert r.returncode == 0, r.stdout
    r = run(exe, "patch-compression", SAMPLE_100, "samples")
    assert r.returncode == 0, r.stdout


def _read_branches_py(rootio, data):
    try:
        t = rootio.RootFile(data).tree("Samples")
        return t.array("amplitudeTruth", np.float64), t.vectors("samples")
    except (rootio.RootFormatError, KeyError):
        return None


def _read_branches_cpp(exe, path, out):
    r = run(exe, "branches", path, out)
    if r.returncode == 3:
        return None
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    b = out.read_bytes()
    n = struct.unpack_from("=q", b, 0)[0]
    truth = np.frombuffer(b, dtype=np.float64, count=n, offset=8)
    p = 8 + 8 * n
    m = struct.unpack_from("=q", b, p)[0]
    p += 8
    vecs = []
    for _ in range(m):
        k = struct.unpack_from("=q", b, p)[0]
        vecs.append(np.frombuffer(b, dtype=np.float64, count=k, offset=p + 8))
        p += 8 + 8 * k
    return truth, vecs


@needs_data
def test_cpp_and_python_readers_agree_on_mutated_files(exe, mf, tmp_path):
    """Differential check: on copies of the Samples file with random bytes
    changed, the C++ and the Python reader either both refuse the file or
    both return the same columns bit for bit."""
    import multifit_gb300.rootio as rootio

    orig = bytearray(open(SAMPLE_100, "rb").read())
    f = rootio.RootFile(bytes(orig))
    # most changes land in the records the two branches are read from: their
    # baskets, the tree record, the file header and the top keys list
    spans = [(k.pos, k.pos + k.nbytes) for k in f.walk()
             if (k.class_name == "TBasket" and k.name in ("samples", "amplitudeTruth")) or k.class_name == "TTree"]
    spans += [(0, f.begin + f.nbytes_name + 40), (f.top["seek_keys"], f.top["seek_keys"] + f.top["nbytes_keys"])]
    rng = np.random.default_rng(12)
    both_read = both_refused = 0
    for i in range(200):
        d = bytearray(orig)
        for _ in range(int(rng.integers(1, 6))):
            if rng.random() < 0.8:
                lo, hi = spans[int(rng.integers(len(spans)))]
                pos = int(rng.integers(lo, hi))
            else:
                pos = int(rng.integers(len(d)))
            d[pos] = int(rng.integers(256))
        path = tmp_path / "m.root"
        path.write_bytes(bytes(d))
        py = _read_branches_py(rootio, bytes(d))
        cpp = _read_branches_cpp(exe, path, tmp_path / "b.bin")
        assert (py is None) == (cpp is None), i
        if py is None:
            both_refused += 1
            continue
        both_read += 1
        assert np.array_equal(py[0], cpp[0], equal_nan=True)
        assert len(py[1]) == len(cpp[1]) and all(np.array_equal(a, b, equal_nan=True) for a, b in zip(py[1], cpp[1]))
    assert both_read > 0 and both_refused > 0
