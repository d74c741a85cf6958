"""The oracle's outer fit pinned to the reference's own multifit_cpu code:
PulseChiSqSNNLS::DoFit / Minimize / updateCov / NNLS / ComputeChiSq /
ComputeApproxUncertainty (multifit_cpu/src/PulseChiSqSNNLS.cpp:21-273) with
inplace_fnnls (nnls/src/inplace_fnnls.cu:72-233), compiled unmodified over
the oracle's Eigen shim (oracle/eigen_shim/). The shim's arithmetic is the
oracle's canonical order, so what this pins is everything else: the outer
chi2 loop and its stopping rule, the covariance update with the pulse
covariance, the warm start with stale amplitudes, the FNNLS passive-set
bookkeeping, the permutations, and the MINOS-like error logic.

Bar: bit for bit (amplitudes, chi2, errors). The committed outputs
(tests/golden/dofit_ref.npz, made by tests/golden/make_dofit_golden.py) pin
the oracle where the reference tree is absent; where it is present, the
shimmed reference also runs live on fresh seeded channels."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "dofit_ref.npz")
SETS = ["c0", "logamp", "warm", "fpc", "edge"]


def golden():
    return dict(np.load(GOLDEN))


@pytest.mark.parametrize("variant", [0, 1])
@pytest.mark.parametrize("errors", [0, 1])
@pytest.mark.parametrize("name", SETS)
def test_oracle_equals_reference_dofit_outputs(oracle, name, errors, variant):
    """variant 0: the oracle's fresh-LLT FNNLS (inplace_fnnls); 1: its
    incremental-Cholesky twin (inplace_fnnls_test_cholesky); both must give
    the reference fit's bits."""
    g = golden()
    F = g["fullpulsecov"] if bool(g[f"{name}_has_fpc"]) else None
    o = oracle.fit_batch(g[f"{name}_samples"], g[f"{name}_pederr"], g["P"], g["R"], g["bxs"], fullpulsecov=F,
                         max_iter_nnls=10, start=0, variant=variant, compute_errors=bool(errors))
    assert np.array_equal(o["amplitudes"], g[f"{name}_e{errors}_amplitudes"])
    assert np.array_equal(o["chi2"], g[f"{name}_e{errors}_chi2"])
    if errors:
        assert np.array_equal(o["errors"], g[f"{name}_e{errors}_errors"], equal_nan=True)
    assert (g[f"{name}_e{errors}_ok"] == 1).all()  # DoFit returns true whatever happens


def test_fullpulse_of_inverts_the_sliding_window(oracle):
    P, R, bxs, _ = oracle.synth_conditions(oracle.SYNTH_ECAL)
    fp = oracle.fullpulse_of(P, bxs)
    for k, bx in enumerate(bxs):
        first = max(0, int(bx) + 3)
        assert np.array_equal(P[first:, k], fp[first + 4 - int(bx): 14 - int(bx)])
        assert (P[:first, k] == 0).all()
    bad = P.copy()
    bad[9, 9] += 1.0
    with pytest.raises(ValueError):
        oracle.fullpulse_of(bad, bxs)


def live(oracle):
    if oracle.ref_dofit_lib() is None:
        pytest.skip("the reference tree is absent (the committed outputs still pin the oracle)")


def test_committed_outputs_are_the_reference_fit(oracle):
    live(oracle)
    g = golden()
    fp = oracle.fullpulse_of(g["P"], g["bxs"])
    assert np.array_equal(fp, g["fullpulse"])
    for name in SETS:
        F = g["fullpulsecov"] if bool(g[f"{name}_has_fpc"]) else None
        for err in (0, 1):
            r = oracle.ref_dofit(g[f"{name}_samples"], g[f"{name}_pederr"], g["R"], g["bxs"], fp, F, bool(err))
            assert np.array_equal(r["amplitudes"], g[f"{name}_e{err}_amplitudes"]), name
            assert np.array_equal(r["chi2"], g[f"{name}_e{err}_chi2"]), name
            assert np.array_equal(r["errors"], g[f"{name}_e{err}_errors"], equal_nan=True), name


@pytest.mark.parametrize("workload,first,count,with_fpc,errors", [
    ("ecal-10k-pu0.5", 5000, 2000, False, True),
    ("ecal-1m-pu2", 700_000, 2000, True, True),
    ("warm-eval-10m", 9_000_000, 4000, False, False),
    ("ecal-10m-logamp-pu4", 3_000_000, 2000, True, True),
])
def test_live_reference_fit_equals_oracle(oracle, workload, first, count, with_fpc, errors):
    live(oracle)
    P, R, bxs, _ = oracle.synth_conditions(oracle.SYNTH_ECAL)
    fp = oracle.fullpulse_of(P, bxs)
    F = None
    if with_fpc:
        F = np.zeros((19, 19))
        idx = np.arange(7, 19)
        F[np.ix_(idx, idx)] = 3e-4 * np.exp(-np.abs(np.subtract.outer(idx, idx)) / 2.0)
    d = oracle.synth_generate(workload, first, count)
    r = oracle.ref_dofit(d["samples"], d["pederr"], R, bxs, fp, F, compute_errors=errors)
    o = oracle.fit_batch(d["samples"], d["pederr"], P, R, bxs, fullpulsecov=F, max_iter_nnls=10, start=0,
                         compute_errors=errors)
    assert np.array_equal(r["amplitudes"], o["amplitudes"])
    assert np.array_equal(r["chi2"], o["chi2"])
    if errors:
        assert np.array_equal(r["errors"], o["errors"], equal_nan=True)
