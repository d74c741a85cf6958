"""The reference driver's run() in C++ against the engine
(tests/cpp/replay_driver.cpp: include/multifit_gb300_io.hpp reads the data
files, mfgb::PulseChiSqSNNLS / mfgb::BatchFitter fit them). It compiles and
links here; on a GPU, on the reference's two data files (the copies committed
under tests/golden/reference_data/, or a directory MULTIFIT_REPLAY_DATA
names), it reproduces the oracle's fits and physics check of
tests/golden/replay_mysample_100.npz bit for bit."""
import os
import subprocess

import numpy as np
import pytest

from _helpers import replay_data_dir

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "replay_mysample_100.npz")
DATA = replay_data_dir()
SAMPLE_100 = os.path.join(DATA, "mysample_100_0.000_0.000_10_25.00_10.00_0.00_1.000_1.00_CRRC43_0.00_slew_1.00.root")
SHAPE = os.path.join(DATA, "EmptyFile.root")


def build(mf, tmp_path, extra=()):
    exe = str(tmp_path / "replay_driver")
    lib_dir = os.path.dirname(mf.LIB_PATH)
    # -ffp-contract=off: the physics check's running sums round as the
    # oracle-side summary's do (no fused x*x + sum)
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", "-Wextra", "-Werror", *extra, "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "replay_driver.cpp"), "-L", lib_dir, "-lmultifit_gb300",
           f"-Wl,-rpath,{lib_dir}", "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


@pytest.mark.parametrize("extra", [(), ("-funsigned-char",)])
def test_replay_driver_compiles_and_links(mf, tmp_path, extra):
    exe = build(mf, tmp_path, extra)
    out = subprocess.run(["nm", "-u", exe], capture_output=True, text=True).stdout
    assert "mf_fit_host" in out


@pytest.mark.gpu
@pytest.mark.parametrize("batch", [0, 1])
def test_replay_driver_reproduces_oracle(mf, cuda, tmp_path, batch):
    if not (DATA and os.path.exists(SAMPLE_100) and os.path.exists(SHAPE)):
        pytest.skip("the reference's data files are absent")
    g = dict(np.load(GOLDEN))
    exe = build(mf, tmp_path)
    r = subprocess.run([exe, SAMPLE_100, SHAPE, "0", str(batch)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.split("\n")
    head = dict(line.split(" ", 1) for line in lines[:4])
    xs = np.array([[float(v) for v in line.split()[1:]] for line in lines[4:] if line.startswith("x ")])
    assert int(head["entries"]) == 100 and xs.shape == (100, 2)
    assert np.array_equal(xs[:, 0], g["ref_amplitudes"][:, 5])
    assert np.array_equal(xs[:, 1], g["ref_chi2"])
    assert float(head["mean"]) == g["ref_h01"][0] and float(head["rms"]) == g["ref_h01"][1]
