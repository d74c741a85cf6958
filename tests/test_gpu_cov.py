"""The per-channel form of the mixed and FP32 precisions: what the
passive-set tables cannot serve alone -- a pulse covariance (the covariance
depends on the channel's amplitudes, multifit_cpu/src/PulseChiSqSNNLS.cpp:
169-194) and the MINOS-like errors (:75-146) -- fitted with the outer loop's
first iteration (covariance pederr^2 samplecor) through the tables and the
rest in FP64 from it; shapes without tables in FP64 throughout.

Bars, against the FP64 fit run to KKT convergence (support start, max_iter
1000; the plain kernel, bit-identical to the oracle, or the oracle's golden
fixtures): normwise relative amplitude error <= 1e-4 and identical active
sets (the support of X()) on every channel; chi2 within 1e-6 relative; the
MINOS error within 1e-4 relative."""
import os

import numpy as np
import pytest

from _helpers import DeviceBatch

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
AMP_TOL = 1e-4
CHI2_TOL = 1e-6
PRECS = ["mixed", "fp32"]


def prec_of(mf, name):
    return {"mixed": mf.PREC_MIXED, "fp32": mf.PREC_FP32}[name]


def relerr(a, r):
    return np.abs(a - r).max(axis=1) / np.maximum(np.abs(r).max(axis=1), 1e-300)


def pulse_covariance(scale=1e-4, length=3.0):
    F = np.zeros((19, 19))
    idx = np.arange(7, 19)
    F[np.ix_(idx, idx)] = scale * np.exp(-np.abs(np.subtract.outer(idx, idx)) / length)
    return F


def fit_fixture(mf, cuda, d, options):
    eng = mf.Engine(0)
    eng.set_conditions(0, mf.make_conditions(d["P"], d["R"], d["bxs"], fullpulsecov=d.get("fullpulsecov")))
    n = d["samples"].shape[0]
    db = DeviceBatch(mf, cuda, n)
    db.samples[:n] = cuda.from_numpy(d["samples"]).cuda()
    db.pederr[:n] = cuda.from_numpy(d["pederr"]).cuda()
    cuda.cuda.synchronize()
    eng.fit_device(db.batch, options)
    o = db.outputs_host()
    eng.close()
    return o


def _has_fpc(name):
    with np.load(os.path.join(GOLDEN, f"fits_{name}.npz")) as z:
        return "fullpulsecov" in z.files


# (fixture, errors): every fixture with MINOS errors; without errors only the
# fixtures with a pulse covariance (the others are served by the tables)
CASES = [(name, errors) for name in ["ecal_fpc", "ecal_c0", "ecal_logamp", "hcal", "edge"] for errors in (0, 1)
         if errors or _has_fpc(name)]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("name,errors", CASES)
def test_per_channel_form_on_fixtures(mf, cuda, name, errors, prec):
    d = dict(np.load(os.path.join(GOLDEN, f"fits_{name}.npz")))
    mode = "err" if errors else "kkt"
    o = fit_fixture(mf, cuda, d, mf.default_options(precision=prec_of(mf, prec), max_iter_nnls=1000,
                                                     compute_errors=errors))
    K = d["P"].shape[1]
    r = d[f"{mode}_amplitudes"]
    ok = d[f"{mode}_status"] == 0
    err = relerr(o["amplitudes"][:, :K], r)
    assert (err[ok] <= AMP_TOL).all(), err[ok].max()
    assert (o["status"][ok] == 0).all()
    diff = o["active_mask"] ^ d[f"{mode}_active_mask"]
    if name == "edge":
        # noise-free edge channels: columns of round-off-level amplitude may
        # enter or not (the absolute eps * pederr^2 is below FP64 round-off)
        scale = np.maximum(np.abs(r).max(axis=1), 1e-300)
        for i in np.nonzero(ok & (diff != 0))[0]:
            cols = [k for k in range(K) if (int(diff[i]) >> k) & 1]
            assert all(abs(r[i, k]) <= 1e-9 * scale[i] for k in cols)
    else:
        assert (diff[ok] == 0).all()
        c2 = np.abs(o["chi2"] - d[f"{mode}_chi2"]) / np.maximum(d[f"{mode}_chi2"], 1.0)
        assert (c2[ok] <= CHI2_TOL).all(), c2[ok].max()
    if errors:
        e, re = o["errors"], d["err_errors"]
        fin = ok & np.isfinite(re)
        assert (np.isfinite(e) == np.isfinite(re))[ok].all()
        assert (np.abs(e[fin] - re[fin]) <= AMP_TOL * np.abs(re[fin])).all()


@pytest.mark.parametrize("prec", PRECS)
def test_per_channel_form_pulse_covariance_100k(mf, cuda, prec):
    """100,000 ECAL channels (pileup 2) with a pulse covariance three times the
    fixture's, against the plain FP64 kernel at KKT convergence: the form
    follows the FP64 trajectory, so it also stops after as many outer
    iterations (on all but round-off-level ties of the stopping rule)."""
    P, R, bxs, _ = mf.conditions_arrays(mf.synth_conditions(mf.SYNTH_ECAL)[0])
    eng = mf.Engine(0)
    eng.set_conditions(0, mf.make_conditions(P, R, bxs, pulse_covariance(3e-4)))
    n = 100_000
    db = DeviceBatch(mf, cuda, n)
    db.generate(mf, mf.synth_params(21, n, pileup_mean=2.0))
    eng.fit_device(db.batch, mf.default_options(max_iter_nnls=1000, nnls_start=mf.START_SUPPORT))
    f64 = db.outputs_host()
    eng.fit_device(db.batch, mf.default_options(precision=prec_of(mf, prec), max_iter_nnls=1000))
    o = db.outputs_host()
    err = relerr(o["amplitudes"], f64["amplitudes"])
    assert (err <= AMP_TOL).all(), err.max()
    assert (o["active_mask"] == f64["active_mask"]).all()
    assert (o["status"] == f64["status"]).all()
    assert ((o["iters"] & 0xFF) == (f64["iters"] & 0xFF)).mean() >= 0.999


@pytest.mark.parametrize("prec", PRECS)
def test_per_channel_form_shape_without_tables(mf, cuda, prec):
    """N = 10 samples, K = 7 pulses (BX -3..3): no passive-set tables for this
    shape, so the per-channel form fits it."""
    P, R, bxs, _ = mf.conditions_arrays(mf.synth_conditions(mf.SYNTH_ECAL)[0])
    keep = slice(2, 9)
    eng = mf.Engine(0)
    eng.set_conditions(0, mf.make_conditions(P[:, keep], R, bxs[keep]))
    n = 20_000
    db = DeviceBatch(mf, cuda, n)
    db.generate(mf, mf.synth_params(22, n, pileup_mean=0.5))
    eng.fit_device(db.batch, mf.default_options(max_iter_nnls=1000, nnls_start=mf.START_SUPPORT))
    f64 = db.outputs_host()
    eng.fit_device(db.batch, mf.default_options(precision=prec_of(mf, prec), max_iter_nnls=1000))
    o = db.outputs_host()
    err = relerr(o["amplitudes"][:, :7], f64["amplitudes"][:, :7])
    assert (err <= AMP_TOL).all(), err.max()
    assert (o["active_mask"] == f64["active_mask"]).all()
    eng.close()


def test_per_channel_form_launches(mf, cuda):
    """The first iteration's table kernels, then one FP64 launch."""
    eng = mf.Engine(0)
    P, R, bxs, _ = mf.conditions_arrays(mf.synth_conditions(mf.SYNTH_ECAL)[0])
    eng.set_conditions(0, mf.make_conditions(P, R, bxs, pulse_covariance()))
    db = DeviceBatch(mf, cuda, 5000)
    db.generate(mf, mf.synth_params(23, 5000, pileup_mean=2.0))
    eng.profile(True)
    eng.fit_device(db.batch, mf.default_options(precision=mf.PREC_FP32, max_iter_nnls=1000))
    k = eng.profile_read()
    eng.profile(False)
    assert {"search_kernel", "judge_kernel", "fit_fp64_kernel"} <= set(k)
    assert k["fit_fp64_kernel"][0] == 1 and k["fit_fp64_kernel"][1] > 0
    eng.close()
