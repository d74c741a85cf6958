"""The reference's own ECAL data file (data/mysample_100_...root, 100 entries)
replayed through the engine as the reference driver replays it
(multifit_cpu/src/multifit.cpp:83-271): the inputs come from
tests/golden/replay_mysample_100.npz, which holds what the ROOT-format reader
read from the file and the oracle's fits of it.

Bars: the FP64 form (host-pointer entry, and the per-channel PulseChiSqSNNLS
shim the driver's lambda calls) reproduces the oracle's fits and the driver's
physics check bit for bit; the mixed and FP32 forms land within 1e-4 normwise
relative amplitude error of the KKT fits with identical active sets."""
import os

import numpy as np
import pytest

from _helpers import replay_data_dir

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "replay_mysample_100.npz")
DATA = replay_data_dir()
SAMPLE_100 = os.path.join(DATA, "mysample_100_0.000_0.000_10_25.00_10.00_0.00_1.000_1.00_CRRC43_0.00_slew_1.00.root")
SHAPE = os.path.join(DATA, "EmptyFile.root")
AMP_TOL = 1e-4  # normwise relative amplitude error of the mixed and FP32 forms


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLDEN))


@pytest.fixture(scope="module")
def eio(mf):
    import multifit_gb300.ecal_data_io as m

    return m


def test_replay_fp64_reproduces_oracle_and_physics_check(mf, cuda, eio, gold):
    eng = mf.Engine(0)
    r = eio.replay_arrays(eng, gold["samples"], gold["truth"], gold["fullpulse"], gold["noisecor"])
    assert np.array_equal(r["amplitudes"], gold["ref_amplitudes"])
    assert np.array_equal(r["chi2"], gold["ref_chi2"])
    assert np.array_equal(r["active_mask"], gold["ref_active_mask"])
    assert np.array_equal(r["status"], gold["ref_status"])
    assert np.array_equal(r["ampl"], gold["ref_amplitudes"][:, 5])
    assert np.array_equal(r["v_ampl"], gold["ref_amplitudes"])  # BXs -5..4 pack in order
    h = r["h01"]
    assert np.array_equal([h["mean"], h["rms"], h["entries"], h["in_range"]], gold["ref_h01"])
    eng.close()


def test_replay_driver_lambda_through_the_shim(mf, cuda, gold):
    """The driver's per-channel loop body: PulseChiSqSNNLS, error calculation
    off, DoFit(samples, noisecor, pederr 1.0, bxs, fullpulse, 0), X(), ChiSq()."""
    eng = mf.Engine(0)
    zero_cov = np.zeros((19, 19))
    for i in range(8):
        func = mf.PulseChiSqSNNLS(eng)
        func.disableErrorCalculation()
        assert func.DoFit(gold["samples"][i], gold["noisecor"], 1.0, gold["bxs"], gold["fullpulse"], zero_cov)
        assert np.array_equal(func.X(), gold["ref_amplitudes"][i])
        assert func.ChiSq() == gold["ref_chi2"][i]
        assert np.array_equal(func.BXs(), gold["bxs"])
    eng.close()


@pytest.mark.parametrize("prec", ["mixed", "fp32"])
def test_replay_mixed_forms_within_bounds_of_kkt_fits(mf, cuda, eio, gold, prec):
    eng = mf.Engine(0)
    precision = {"mixed": mf.PREC_MIXED, "fp32": mf.PREC_FP32}[prec]
    r = eio.replay_arrays(eng, gold["samples"], gold["truth"], gold["fullpulse"], gold["noisecor"],
                          options=mf.default_options(precision=precision, max_iter_nnls=1000))
    ref = gold["kkt_amplitudes"]
    err = np.abs(r["amplitudes"] - ref).max(axis=1) / np.abs(ref).max(axis=1)
    assert (err <= AMP_TOL).all(), err.max()
    assert np.array_equal(r["active_mask"], gold["kkt_active_mask"])
    assert (r["status"] == 0).all()
    h = r["h01"]
    assert abs(h["mean"] - gold["kkt_h01"][0]) <= AMP_TOL * 10.0
    eng.close()


@pytest.mark.skipif(not (DATA and os.path.exists(SAMPLE_100) and os.path.exists(SHAPE)),
                    reason="the reference's data files are absent")
def test_replay_from_the_root_file(mf, cuda, eio, gold):
    """The two data files (committed copies, or MULTIFIT_REPLAY_DATA's):
    read, condition and fit end to end."""
    eng = mf.Engine(0)
    r = eio.replay(eng, SAMPLE_100, SHAPE)
    assert np.array_equal(r["samples"], gold["samples"])
    assert np.array_equal(r["amplitudes"], gold["ref_amplitudes"])
    eng.close()
