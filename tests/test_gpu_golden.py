"""The engine on the committed golden fixtures (tests/golden/): the plain FP64
kernel must reproduce the fixtures' fits bit for bit (reference start with
max_iter 10, support start to KKT convergence, MINOS-like errors, with and
without a pulse covariance, HCAL 8x8 and hand-made edge channels); the mixed
form must land within its bounds (<= 1e-4 normwise relative amplitude error,
identical active sets) of the KKT fixtures."""
import os

import numpy as np
import pytest

from _helpers import DeviceBatch

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FITS = ["ecal_c0", "ecal_logamp", "hcal", "ecal_fpc", "edge"]
MODES = {"ref": dict(nnls_start=0, max_iter_nnls=10), "kkt": dict(nnls_start=1, max_iter_nnls=1000),
         "err": dict(nnls_start=1, max_iter_nnls=1000, compute_errors=1)}


def setup(mf, cuda, name):
    d = dict(np.load(os.path.join(GOLDEN, f"fits_{name}.npz")))
    eng = mf.Engine(0)
    eng.set_conditions(0, mf.make_conditions(d["P"], d["R"], d["bxs"], fullpulsecov=d.get("fullpulsecov")))
    n = d["samples"].shape[0]
    db = DeviceBatch(mf, cuda, n)
    db.samples[:n] = cuda.from_numpy(d["samples"]).cuda()
    db.pederr[:n] = cuda.from_numpy(d["pederr"]).cuda()
    cuda.cuda.synchronize()
    return d, eng, db


@pytest.mark.parametrize("name", FITS)
@pytest.mark.parametrize("mode", list(MODES))
def test_fp64_kernel_reproduces_fixture(mf, cuda, name, mode):
    d, eng, db = setup(mf, cuda, name)
    eng.fit_device(db.batch, mf.default_options(**MODES[mode]))
    o = db.outputs_host()
    K = d["P"].shape[1]
    assert np.array_equal(o["amplitudes"][:, :K], d[f"{mode}_amplitudes"])
    for k in ("chi2", "active_mask", "status"):
        assert np.array_equal(o[k], d[f"{mode}_{k}"]), k
    if mode == "err":
        assert np.array_equal(o["errors"], d["err_errors"], equal_nan=True)
    eng.close()


@pytest.mark.parametrize("prec", ["mixed", "fp32"])
@pytest.mark.parametrize("name", ["ecal_c0", "ecal_logamp", "hcal", "edge"])
def test_mixed_form_within_bounds_of_kkt_fixture(mf, cuda, name, prec):
    d, eng, db = setup(mf, cuda, name)
    precision = {"mixed": mf.PREC_MIXED, "fp32": mf.PREC_FP32}[prec]
    eng.fit_device(db.batch, mf.default_options(precision=precision, max_iter_nnls=1000))
    o = db.outputs_host()
    K = d["P"].shape[1]
    r = d["kkt_amplitudes"]
    ok = d["kkt_status"] == 0
    err = np.abs(o["amplitudes"][:, :K] - r).max(axis=1) / np.maximum(np.abs(r).max(axis=1), 1e-300)
    assert (err[ok] <= 1e-4).all(), err[ok].max()
    # active sets agree, except on columns whose amplitude is at round-off
    # level in both fits (noise-free edge channels: with pederr -> 0 the
    # reference's absolute threshold eps * pederr^2 falls below FP64 round-off,
    # so such columns enter or not on rounding noise, in the oracle as well)
    diff = o["active_mask"] ^ d["kkt_active_mask"]
    scale = np.maximum(np.abs(r).max(axis=1), 1e-300)
    for i in np.nonzero(ok & (diff != 0))[0]:
        cols = [k for k in range(K) if (int(diff[i]) >> k) & 1]
        assert all(abs(r[i, k]) <= 1e-9 * scale[i] and abs(o["amplitudes"][i, k]) <= 1e-9 * scale[i]
                   for k in cols), (name, i, cols, r[i], o["amplitudes"][i])
    if name != "edge":
        assert (diff[ok] == 0).all()
    eng.close()


@pytest.mark.parametrize("errors", [0, 1])
@pytest.mark.parametrize("name", ["c0", "logamp", "warm", "fpc", "edge"])
def test_fp64_kernel_reproduces_reference_dofit(mf, cuda, name, errors):
    """The FP64 drop-in against the reference's own multifit_cpu fit
    (PulseChiSqSNNLS.cpp + inplace_fnnls.cu compiled over the oracle's Eigen
    shim; outputs in tests/golden/dofit_ref.npz): bit for bit, with the
    reference's settings (reference start, max_iter 10) and errors off or on."""
    g = dict(np.load(os.path.join(GOLDEN, "dofit_ref.npz")))
    F = g["fullpulsecov"] if bool(g[f"{name}_has_fpc"]) else None
    eng = mf.Engine(0)
    eng.set_conditions(0, mf.make_conditions(g["P"], g["R"], g["bxs"], fullpulsecov=F))
    s = g[f"{name}_samples"]
    n = s.shape[0]
    db = DeviceBatch(mf, cuda, n)
    db.samples[:n] = cuda.from_numpy(s).cuda()
    db.pederr[:n] = cuda.from_numpy(g[f"{name}_pederr"]).cuda()
    cuda.cuda.synchronize()
    eng.fit_device(db.batch, mf.default_options(compute_errors=errors))
    o = db.outputs_host()
    assert np.array_equal(o["amplitudes"], g[f"{name}_e{errors}_amplitudes"])
    assert np.array_equal(o["chi2"], g[f"{name}_e{errors}_chi2"])
    if errors:
        assert np.array_equal(o["errors"], g[f"{name}_e{errors}_errors"], equal_nan=True)
    eng.close()
