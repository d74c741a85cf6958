"""The committed golden fixtures (tests/golden/, made by make_golden.py where
the reference tree is present) against the oracle and the generator, on the
CPU. linalgebra_ref.npz holds outputs of the reference's own linalgebra code
(compiled from its sources), so these tests pin the oracle to the reference
without reading the reference tree; fits_*.npz hold seeded channels and the
oracle's fits (reference start / max_iter 10, support start / max_iter 1000,
MINOS-like errors). Bit-exact comparisons throughout, except the generator
(host libm differs across machines in the last bits: 1e-12 relative)."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FITS = ["ecal_c0", "ecal_logamp", "hcal", "ecal_fpc", "edge"]
MODES = {"ref": dict(start=0, max_iter_nnls=10), "kkt": dict(start=1, max_iter_nnls=1000),
         "err": dict(start=1, max_iter_nnls=1000, compute_errors=True)}


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def test_oracle_linalgebra_reproduces_reference_outputs(oracle):
    o = oracle.lib()
    d = load("linalgebra_ref")
    n = 10
    for c in range(d["M"].shape[0]):
        M, b = d["M"][c], d["b"][c]
        for view in range(1, n + 1):
            L = np.zeros(n * n)
            o.oracle_cholesky(M.copy(), L, n, view)
            assert np.array_equal(L, d["L"][c, view - 1]), (c, view)
            y = np.zeros(n)
            o.oracle_forward(L, n, b, y, view)
            assert np.array_equal(y[:view], d["y"][c, view - 1, :view]), (c, view)
            x = np.zeros(n)
            o.oracle_backward(L, n, y, x, view)
            assert np.array_equal(x[:view], d["x"][c, view - 1, :view]), (c, view)
        view = int(d["add_view"][c])
        L, y = d["add_L0"][c].copy(), d["add_y0"][c].copy()
        o.oracle_rc_addition(M.copy(), L, n, b, y, view)
        assert np.array_equal(L, d["add_L"][c]) and np.array_equal(y[:view], d["add_y"][c, :view])
        pos = int(d["rm_pos"][c])
        L, y = d["rm_L0"][c].copy(), d["rm_y0"][c].copy()
        o.oracle_inbetween_removal(d["rm_M"][c].copy(), L, n, d["rm_b"][c].copy(), y, pos, n - 1)
        assert np.array_equal(L, d["rm_L"][c]) and np.array_equal(y[: n - 1], d["rm_y"][c, : n - 1])


@pytest.mark.parametrize("name", FITS)
@pytest.mark.parametrize("mode", list(MODES))
def test_oracle_reproduces_fit_fixtures(oracle, name, mode):
    d = load("fits_" + name)
    o = oracle.fit_batch(d["samples"], d["pederr"], d["P"], d["R"], d["bxs"], fullpulsecov=d.get("fullpulsecov"),
                         **MODES[mode])
    for k in ("amplitudes", "chi2", "active_mask", "status", "iters"):
        assert np.array_equal(o[k], d[f"{mode}_{k}"]), k
    if mode == "err":
        assert np.array_equal(o["errors"], d["err_errors"], equal_nan=True)


def test_fixture_inputs_regenerate(mf):
    """The synthetic fixtures are the first channels of the named workloads."""
    cases = {"ecal_c0": mf.WORKLOADS["ecal-10k-pu0.5"](), "ecal_logamp": mf.WORKLOADS["ecal-10m-logamp-pu4"](),
             "hcal": mf.synth_params(4, 256, pileup_mean=-8.0, hcal_fraction=1.0)}
    for name, p in cases.items():
        d = load("fits_" + name)
        g = mf.synth_generate_host(p, 0, d["samples"].shape[0], with_truth=False)
        np.testing.assert_allclose(g["samples"], d["samples"], rtol=1e-12, atol=1e-300)
        np.testing.assert_allclose(g["pederr"], d["pederr"], rtol=1e-12)


def test_fixture_sanity():
    """The fixtures cover what they claim: converged fits, an iterating outer
    loop with the pulse covariance, HCAL 8x8 shapes, non-trivial errors."""
    e = load("fits_ecal_c0")
    assert (e["kkt_status"] == 0).all() and e["P"].shape == (10, 10)
    assert load("fits_hcal")["P"].shape == (8, 8)
    assert load("fits_ecal_fpc")["kkt_iters"][:, 0].mean() > e["kkt_iters"][:, 0].mean()
    assert np.isfinite(load("fits_ecal_logamp")["err_errors"]).mean() > 0.5
