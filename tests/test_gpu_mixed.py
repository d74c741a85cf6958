"""GPU mixed-precision forms against the FP64 oracle run to KKT convergence
(support start, max_iter 1000), on the same seeded inputs: MF_PREC_MIXED
(FP32 search and screen, FP64 judge: refinement solve, residual, chi2) and
MF_PREC_FP32 (the same judge in double-float FP32 arithmetic).

Tolerances (floating point): per channel the normwise relative amplitude
error max_k |a_k - a_ref_k| / max_k |a_ref_k| must be <= 1e-4 (the headline
bound) on at least 99.9 % of channels and <= 1e-6 on the median; chi2 relative
error <= 1e-6 where the active sets agree; active sets (support of X())
identical on at least 99.9 % of channels. The FP64 oracle's own error on the
worst-conditioned passive sets is ~cond(G)^2 * 1.1e-16 ~ 3e-7 relative.
"""
import numpy as np
import pytest

from _helpers import DeviceBatch, oracle_fit_sets

pytestmark = pytest.mark.gpu

AMP_TOL = 1e-4
CHI2_TOL = 1e-6


def relerr(a, r):
    scale = np.maximum(np.abs(r).max(axis=1), 1e-300)
    return np.abs(a[:, : r.shape[1]] - r).max(axis=1) / scale


PRECISIONS = pytest.mark.parametrize("prec", ["mixed", "fp32"])


def prec_of(mf, prec):
    return {"mixed": mf.PREC_MIXED, "fp32": mf.PREC_FP32}[prec]


def run_mixed(mf, cuda, eng, params, n, ctype=False, prec="mixed", **opt):
    db = DeviceBatch(mf, cuda, n, ctype=ctype)
    db.generate(mf, params)
    eng.fit_device(db.batch, mf.default_options(precision=prec_of(mf, prec), max_iter_nnls=1000, **opt))
    return db.inputs_host(), db.outputs_host()


def check_against_oracle(mf, oracle, eng, inp, gpu, frac=0.999):
    ref = oracle_fit_sets(mf, oracle, eng, inp, max_iter_nnls=1000, start=1)
    err = relerr(gpu["amplitudes"], ref["amplitudes"])
    same = gpu["active_mask"] == ref["active_mask"]
    assert (err <= AMP_TOL).mean() >= frac, f"amp err p99.9={np.percentile(err, 99.9):.3g} max={err.max():.3g}"
    assert np.median(err) <= 1e-6
    assert same.mean() >= frac, f"active-set agreement {same.mean():.5f}"
    c = ref["chi2"][same]
    assert (np.abs(gpu["chi2"][same] - c) <= CHI2_TOL * np.maximum(c, 1.0)).mean() >= frac
    assert (gpu["status"] == 0).all()
    return err, same


@PRECISIONS
@pytest.mark.parametrize("wl", ["ecal-pu2", "ecal-logamp-pu4"])
def test_mixed_vs_oracle_ecal(mf, oracle, cuda, wl, prec):
    params = {"ecal-pu2": mf.synth_params(2, 50_000, pileup_mean=2.0),
              "ecal-logamp-pu4": mf.synth_params(3, 50_000, intime_log=True, lo=0.1, hi=1000.0,
                                                 pileup_mean=4.0)}[wl]
    eng = mf.Engine(0)
    cond, _ = mf.synth_conditions(mf.SYNTH_ECAL)
    eng.set_conditions(0, cond)
    inp, gpu = run_mixed(mf, cuda, eng, params, 50_000, prec=prec)
    check_against_oracle(mf, oracle, eng, inp, gpu)
    eng.close()


@PRECISIONS
def test_mixed_vs_oracle_ecal_hcal(mf, oracle, cuda, prec):
    eng = mf.Engine(0)
    eng.set_conditions(0, mf.synth_conditions(mf.SYNTH_ECAL)[0])
    eng.set_conditions(1, mf.synth_conditions(mf.SYNTH_HCAL)[0])
    params = mf.synth_params(4, 40_000, pileup_mean=-8.0, hcal_fraction=0.4)
    inp, gpu = run_mixed(mf, cuda, eng, params, 40_000, ctype=True, prec=prec)
    check_against_oracle(mf, oracle, eng, inp, gpu)
    eng.close()


@PRECISIONS
def test_mixed_matches_fp64_gpu_path(mf, cuda, prec):
    """Mixed forms vs the plain FP64 kernel run to convergence, full batch on the GPU."""
    eng = mf.Engine(0)
    eng.set_conditions(0, mf.synth_conditions(mf.SYNTH_ECAL)[0])
    n = 200_000
    p = mf.synth_params(3, n, intime_log=True, lo=0.1, hi=1000.0, pileup_mean=4.0)
    from _helpers import DeviceBatch

    db = DeviceBatch(mf, cuda, n)
    db.generate(mf, p)
    eng.fit_device(db.batch, mf.default_options(max_iter_nnls=1000, nnls_start=mf.START_SUPPORT))
    f64 = db.outputs_host()
    eng.fit_device(db.batch, mf.default_options(precision=prec_of(mf, prec), max_iter_nnls=1000))
    mix = db.outputs_host()
    err = relerr(mix["amplitudes"], f64["amplitudes"])
    assert (err <= AMP_TOL).mean() >= 0.999
    assert (mix["active_mask"] == f64["active_mask"]).mean() >= 0.999
    eng.close()


def test_profile_counts_and_times_every_launch(mf, cuda):
    """mf_profile: one record per kernel launch on the fit's stream, with
    positive device times, for the mixed form on two condition sets and for
    the plain FP64 form; nothing is recorded once it is disabled."""
    eng = mf.Engine(0)
    eng.set_conditions(0, mf.synth_conditions(mf.SYNTH_ECAL)[0])
    eng.set_conditions(1, mf.synth_conditions(mf.SYNTH_HCAL)[0])
    db = DeviceBatch(mf, cuda, 20_000, ctype=True)
    db.generate(mf, mf.synth_params(21, 20_000, pileup_mean=-8.0, hcal_fraction=0.4))
    eng.profile(True)
    for _ in range(2):
        eng.fit_device(db.batch, mf.default_options(precision=mf.PREC_MIXED, max_iter_nnls=1000))
    eng.fit_device(db.batch, mf.default_options())
    rec = eng.profile_read()
    # the FP64 form: two passes per condition set (first outer iterations in
    # lockstep, the rest with refill)
    assert {k: v[0] for k, v in rec.items()} == {"search_kernel": 4, "screen_kernel": 4, "fix_kernel": 4, "judge_kernel": 4,
                                                  "repair_kernel": 4, "fit_fp64_kernel": 4}
    assert all(ms > 0 for _, ms in rec.values())
    assert eng.profile_read() == {}  # the read clears the record
    eng.profile(False)
    eng.fit_device(db.batch, mf.default_options())
    with pytest.raises(mf.MultifitError):
        eng.profile_read()
    eng.close()


def test_fp32_judge_accuracy_and_agreement_with_fp64_judge(mf, cuda):
    """The double-float judge against the FP64 judge on the same search and
    screen: amplitudes within 1e-9 normwise relative (~cond(G_S) 2^-48), chi2
    within 1e-9 relative, the same active sets on >= 99.99 % of channels."""
    eng = mf.Engine(0)
    eng.set_conditions(0, mf.synth_conditions(mf.SYNTH_ECAL)[0])
    n = 200_000
    db = DeviceBatch(mf, cuda, n)
    db.generate(mf, mf.synth_params(3, n, intime_log=True, lo=0.1, hi=1000.0, pileup_mean=4.0))
    eng.fit_device(db.batch, mf.default_options(precision=mf.PREC_MIXED, max_iter_nnls=1000))
    f64 = db.outputs_host()
    eng.fit_device(db.batch, mf.default_options(precision=mf.PREC_FP32, max_iter_nnls=1000))
    df = db.outputs_host()
    same = df["active_mask"] == f64["active_mask"]
    assert same.mean() >= 0.9999
    err = relerr(df["amplitudes"], f64["amplitudes"])[same]
    assert np.percentile(err, 99.9) <= 1e-9 and err.max() <= 1e-6, (np.percentile(err, 99.9), err.max())
    c = f64["chi2"][same]
    assert (np.abs(df["chi2"][same] - c) <= 1e-9 * np.maximum(c, 1.0)).mean() >= 0.999
    eng.close()
