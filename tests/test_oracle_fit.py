"""The oracle's full per-channel fit (PulseChiSqSNNLS::DoFit,
multifit_cpu/src/PulseChiSqSNNLS.cpp:21-207) on synthetic channels.

The reference driver's physics check is the mean and RMS of (reconstructed -
true) in-time amplitude (multifit_cpu/src/multifit.cpp:254,268-271); the
same check runs here on seeded synthetic channels, plus consistency checks of
chi2, of the two FNNLS variants and of the MINOS-like uncertainty.
"""
import numpy as np
import pytest
import scipy.linalg as sl


def ecal_batch(mf, n, seed=1, pileup=0.5, log=False, lo=1.0, hi=100.0):
    cond, sigma = mf.synth_conditions(mf.SYNTH_ECAL)
    p = mf.synth_params(seed, n, intime_log=log, lo=lo, hi=hi, pileup_mean=pileup)
    data = mf.synth_generate_host(p, 0, n, stride=10)
    P, R, bxs, _ = mf.conditions_arrays(cond)
    return data, P, R, bxs, sigma


def test_synthetic_conditions(mf):
    cond, sigma = mf.synth_conditions(mf.SYNTH_ECAL)
    P, R, bxs, F = mf.conditions_arrays(cond)
    assert sigma == 0.044 and F is None
    assert list(bxs) == list(range(-5, 5))
    # column k (BX k-5) peaks at sample k with value 1 and, by the reference's
    # sliding-window rule, starts two samples before its peak
    for k in range(10):
        assert abs(P[k, k] - 1.0) < 1e-15
        assert P[:, k].argmax() == k
        assert (P[: max(0, k - 2), k] == 0).all() and (P[max(0, k - 2):, k] > 0).all()
    np.testing.assert_allclose(R, 0.7 ** np.abs(np.subtract.outer(np.arange(10), np.arange(10))))
    h, hs = mf.synth_conditions(mf.SYNTH_HCAL)
    Ph, Rh, bh, _ = mf.conditions_arrays(h)
    assert Ph.shape == (8, 8) and hs == 0.8 and list(bh) == list(range(-3, 5))
    assert abs(Ph[3, 3] - 1.0) < 1e-15


def test_generator_deterministic_and_chunk_invariant(mf):
    p = mf.synth_params(11, 5000, pileup_mean=2.0)
    a = mf.synth_generate_host(p, 0, 5000)
    b = mf.synth_generate_host(p, 1000, 2000)
    assert np.array_equal(a["samples"][1000:3000], b["samples"])
    assert np.array_equal(a["truth"][1000:3000], b["truth"])
    c = mf.synth_generate_host(mf.synth_params(12, 5000, pileup_mean=2.0), 0, 5000)
    assert not np.array_equal(a["samples"], c["samples"])


def test_generator_distributions(mf):
    n = 200_000
    p = mf.synth_params(3, n, pileup_mean=2.0)
    d = mf.synth_generate_host(p, 0, n)
    t = d["truth"]
    intime = t[:, 5]
    assert 1.0 <= intime.min() and intime.max() <= 100.0
    assert abs(intime.mean() - 50.5) < 0.5
    oot = np.delete(t, 5, axis=1)
    # compound Poisson(2) x Exp(1): mean 2, P(0) = e^-2
    assert abs(oot.mean() - 2.0) < 0.02
    assert abs((oot == 0).mean() - np.exp(-2.0)) < 0.005
    cond, sigma = mf.synth_conditions(mf.SYNTH_ECAL)
    P, R, _, _ = mf.conditions_arrays(cond)
    noise = d["samples"] - t @ P.T
    C = np.cov(noise.T)
    np.testing.assert_allclose(C, sigma ** 2 * R, atol=4e-5)


@pytest.mark.parametrize("max_iter", [10, 1000])
def test_fit_recovers_truth(mf, oracle, max_iter):
    # no pileup: the in-time amplitude is resolved to ~ sigma / ||L^-1 P_in|| = 0.03
    data, P, R, bxs, sigma = ecal_batch(mf, 20_000, seed=1, pileup=0.0)
    out = oracle.fit_batch(data["samples"], data["pederr"], P, R, bxs, max_iter_nnls=max_iter)
    d = out["amplitudes"][:, 5] - data["truth"][:, 5]
    # NNLS positivity: noise fitted by out-of-time pulses biases the in-time amplitude slightly low
    assert abs(np.median(d)) < 0.03
    assert np.percentile(np.abs(d), 68) < 0.06
    assert (out["status"] & 4).sum() == 0
    assert ((out["active_mask"] >> 5) & 1).all()  # the in-time pulse is always fitted
    # mask = support of the amplitudes
    sup = (out["amplitudes"] > 0) @ (1 << np.arange(10))
    assert np.array_equal(out["active_mask"], sup)


def test_fit_with_pileup_bias_is_physics(mf, oracle):
    # the slow CRRC4 pulse (tau = 43 ns) makes adjacent-BX pulses nearly
    # collinear, so pileup leaks into the in-time amplitude; the median stays close
    data, P, R, bxs, sigma = ecal_batch(mf, 20_000, seed=1, pileup=0.5)
    out = oracle.fit_batch(data["samples"], data["pederr"], P, R, bxs)
    d = out["amplitudes"][:, 5] - data["truth"][:, 5]
    assert np.isfinite(d).all()
    assert abs(np.median(d)) < 0.1


@pytest.mark.parametrize("seed", [1, 2, 3])
@pytest.mark.parametrize("start", [0, 1])
def test_fit_chi2_consistent(mf, oracle, seed, start):
    data, P, R, bxs, sigma = ecal_batch(mf, 2000, seed=seed, pileup=2.0)
    out = oracle.fit_batch(data["samples"], data["pederr"], P, R, bxs, max_iter_nnls=1000, start=start)
    L = np.linalg.cholesky(sigma ** 2 * R)
    r = out["amplitudes"] @ P.T - data["samples"]
    z = sl.solve_triangular(L, r.T, lower=True)
    chi2 = (z * z).sum(axis=0)
    np.testing.assert_allclose(out["chi2"], chi2, rtol=1e-9)
    if start == 1:
        # the NNLS optimum: chi2 ~ N minus the fitted amplitudes (loose sanity)
        assert 0.5 < chi2.mean() < 10.0 and chi2.max() < 60.0
    else:
        # the reference start leaves a fraction of channels in a stale,
        # non-optimal state whose chi2 is far above the optimum
        assert np.median(chi2) < 10.0


@pytest.mark.parametrize("pileup", [0.5, 2.0, 4.0])
def test_reference_start_quirk_vs_support_start(mf, oracle, pileup):
    """multifit_cpu restarts every FNNLS with an empty passive set but the
    previous amplitudes (PulseChiSqSNNLS.cpp:258, inplace_fnnls.cu:97), and its
    absolute eps = 1e-11 (PulseChiSqSNNLS.cpp:242) is below the round-off of w
    at these amplitudes, so the second outer iteration often adds an index
    spuriously and can stop with stale amplitudes outside the passive set.
    The support start reaches the NNLS optimum for every channel."""
    data, P, R, bxs, sigma = ecal_batch(mf, 3000, seed=13, pileup=pileup)
    ref = oracle.fit_batch(data["samples"], data["pederr"], P, R, bxs, max_iter_nnls=1000, start=0)
    sup = oracle.fit_batch(data["samples"], data["pederr"], P, R, bxs, max_iter_nnls=1000, start=1)
    assert (sup["chi2"] <= ref["chi2"] * (1 + 1e-9) + 1e-9).all()
    stuck = ref["chi2"] > sup["chi2"] * 1.01 + 1e-6
    assert stuck.mean() > 0.001  # the quirk is real on this data
    for c in range(0, 3000, 150):
        A, b = oracle.whiten(P, R, data["pederr"][c], data["samples"][c])
        xb, _ = oracle.nnls_bruteforce(A, b)
        np.testing.assert_allclose(sup["amplitudes"][c], xb, rtol=0, atol=1e-7 * max(1.0, np.abs(xb).max()))


def test_fit_variants_bitwise(mf, oracle):
    data, P, R, bxs, sigma = ecal_batch(mf, 5000, seed=5, pileup=4.0, log=True, lo=0.1, hi=1000.0)
    a = oracle.fit_batch(data["samples"], data["pederr"], P, R, bxs, variant=0)
    b = oracle.fit_batch(data["samples"], data["pederr"], P, R, bxs, variant=1)
    for k in ("amplitudes", "chi2", "active_mask", "status", "iters"):
        assert np.array_equal(a[k], b[k]), k


def test_fit_converged_solution_is_nnls_optimum(mf, oracle):
    data, P, R, bxs, sigma = ecal_batch(mf, 300, seed=9, pileup=2.0)
    out = oracle.fit_batch(data["samples"], data["pederr"], P, R, bxs, max_iter_nnls=1000, start=1)
    for c in range(300):
        A, b = oracle.whiten(P, R, data["pederr"][c], data["samples"][c])
        xb, _ = oracle.nnls_bruteforce(A, b)
        x = out["amplitudes"][c]
        np.testing.assert_allclose(x, xb, rtol=0, atol=1e-7 * max(1.0, np.abs(xb).max()))


@pytest.mark.parametrize("pileup", [0.0, 0.5])
def test_minos_errors(mf, oracle, pileup):
    """DoFit's MINOS-like in-time uncertainty (PulseChiSqSNNLS.cpp:75-146):
    with the support start it is finite for every channel and at least the
    Gaussian error 1/||L^-1 P_in|| of the in-time pulse alone (correlated
    pileup only widens it). With the reference start chisq0 can come from a
    stale, non-optimal state, and sqrt(chi2 - chisq0) is then NaN for some
    channels, as in the reference; the error calculation never changes X()
    or ChiSq()."""
    data, P, R, bxs, sigma = ecal_batch(mf, 2000, seed=4, pileup=pileup)
    L = np.linalg.cholesky(sigma ** 2 * R)
    approx = 1.0 / np.linalg.norm(sl.solve_triangular(L, P[:, 5], lower=True))
    sup = oracle.fit_batch(data["samples"], data["pederr"], P, R, bxs, compute_errors=True, start=1)
    err = sup["errors"]
    assert np.isfinite(err).all()
    assert np.percentile(err, 5) >= 0.95 * approx
    assert np.median(err) < 5.0 * approx
    for start in (0, 1):
        with_err = oracle.fit_batch(data["samples"], data["pederr"], P, R, bxs, compute_errors=True, start=start)
        plain = oracle.fit_batch(data["samples"], data["pederr"], P, R, bxs, compute_errors=False, start=start)
        assert np.array_equal(plain["amplitudes"], with_err["amplitudes"])
        assert np.array_equal(plain["chi2"], with_err["chi2"])
        assert np.isfinite(with_err["errors"]).mean() > 0.5


def test_fullpulsecov_iterates(mf, oracle):
    """With a non-zero pulse covariance the covariance depends on the
    amplitudes (updateCov, PulseChiSqSNNLS.cpp:177-191) and the outer loop
    runs more than the two iterations of the constant-covariance case."""
    data, P, R, bxs, sigma = ecal_batch(mf, 500, seed=8, pileup=2.0)
    F = np.zeros((19, 19))
    idx = np.arange(7, 19)
    F[np.ix_(idx, idx)] = 1e-4 * np.exp(-np.abs(np.subtract.outer(idx, idx)) / 3.0)
    a = oracle.fit_batch(data["samples"], data["pederr"], P, R, bxs, start=1)
    b = oracle.fit_batch(data["samples"], data["pederr"], P, R, bxs, fullpulsecov=F, start=1)
    outer_a = a["iters"][:, 0]
    outer_b = b["iters"][:, 0]
    assert (outer_a >= 2).all() and (outer_a == 2).mean() > 0.99
    assert outer_b.mean() > outer_a.mean()
    assert np.isfinite(b["amplitudes"]).all() and np.isfinite(b["chi2"]).all()
    # the covariance grows with the amplitudes, so the weighted chi2 of the same data shrinks
    assert np.median(b["chi2"]) < np.median(a["chi2"])
