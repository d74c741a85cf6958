"""The C++ drop-in (include/multifit_gb300.hpp) used the way the reference's
driver uses PulseChiSqSNNLS (tests/cpp/dropin_driver.cpp follows
multifit_cpu/src/multifit.cpp:196-227): it compiles and links against the C
ABI here; on a GPU its per-channel DoFit and its batch path reproduce mf_fit
bit for bit (plain FP64, the multifit_cpu options)."""
import os
import struct
import subprocess

import numpy as np
import pytest

from _helpers import DeviceBatch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_driver(mf, tmp_path, extra=()):
    exe = str(tmp_path / "dropin_driver")
    lib_dir = os.path.dirname(mf.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", *extra, "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "dropin_driver.cpp"), "-L", lib_dir, "-lmultifit_gb300",
           f"-Wl,-rpath,{lib_dir}", "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


@pytest.mark.parametrize("extra", [(), ("-funsigned-char",)])
def test_dropin_compiles_and_links(mf, tmp_path, extra):
    """Also with plain char unsigned, as on Arm (the bx offsets are negative)."""
    exe = build_driver(mf, tmp_path, extra)
    out = subprocess.run(["nm", "-u", exe], capture_output=True, text=True).stdout
    assert "mf_fit_host" in out and "mf_set_conditions" in out


def ecal_fullpulse(mf):
    """The 19-sample fullpulse of the synthetic ECAL set, read back from its
    pulse matrix (bx = -5 fills fullpulse[9..18], bx = 0 the rest)."""
    cond, _ = mf.synth_conditions(mf.SYNTH_ECAL)
    P, R, bxs, _ = mf.conditions_arrays(cond)
    fp = np.zeros(19)
    fp[9:19] = P[0:10, list(bxs).index(-5)]
    k0 = list(bxs).index(0)
    fp[7:9] = P[3:5, k0]
    assert np.array_equal(mf.build_pulse_matrix(fp, bxs), P)
    return fp, P, R, bxs, cond


@pytest.mark.gpu
@pytest.mark.parametrize("batch_mode,n", [(0, 300), (1, 20_000)])
def test_dropin_matches_mf_fit(mf, cuda, tmp_path, batch_mode, n):
    exe = build_driver(mf, tmp_path)
    fp, P, R, bxs, cond = ecal_fullpulse(mf)
    data = mf.synth_generate_host(mf.synth_params(61, n, pileup_mean=2.0), 0, n, with_truth=False)
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        f.write(struct.pack("<q", n))
        f.write(np.ascontiguousarray(R, dtype="<f8").tobytes())
        f.write(np.asarray(bxs, dtype=np.int8).tobytes())
        f.write(np.asarray(fp, dtype="<f8").tobytes())
        f.write(np.zeros((19, 19), dtype="<f8").tobytes())
        rows = np.concatenate([data["samples"], data["pederr"][:, None]], axis=1)
        f.write(np.ascontiguousarray(rows, dtype="<f8").tobytes())
    out = tmp_path / "out.bin"
    subprocess.run([exe, str(inp), str(out), str(batch_mode)], check=True, timeout=600)
    rec = np.dtype([("chi2", "<f8"), ("ampl", "<f8"), ("status", "<i4"), ("x", "<f8", 10)])
    got = np.fromfile(out, dtype=rec)
    assert got.shape == (n,)
    eng = mf.Engine(0)
    eng.set_conditions(0, cond)
    db = DeviceBatch(mf, cuda, n)
    db.samples[:n] = cuda.from_numpy(data["samples"]).cuda()
    db.pederr[:n] = cuda.from_numpy(data["pederr"]).cuda()
    eng.fit_device(db.batch, mf.default_options())
    ref = db.outputs_host()
    assert np.array_equal(got["chi2"], ref["chi2"])
    x = np.zeros((n, 10))
    for k, b in enumerate(bxs):
        x[:, b + 5] = ref["amplitudes"][:, k]
    assert np.array_equal(got["x"], x)
    assert np.array_equal(got["ampl"], ref["intime"])
    assert (got["status"] == 1).all()
    eng.close()
