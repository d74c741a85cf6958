"""The mixed and FP32 precisions' device routines (csrc/mixed_device.cuh) with
their passive-set tables (csrc/tables.cu), compiled for the host
(tests/cpp/mixed_host.cpp) and run on the CPU through the grid schedule's
cold-start pipeline -- FP32 search, double-float KKT screen, FP32 fix, the FP64
(mixed) or double-float (FP32) judge, FP64 repair, queues included -- and its
warm-start pipeline from given predictions, against the oracle's fits to KKT
convergence: the golden fixtures, seeded ECAL and HCAL channels of the
benchmark generators, imperfect predictions, and noise-free channels whose fits
are exact (where the double-float judge's round-off bounds must send
undecidable channels to the FP64 repair rather than return a wrong active
set).

Tolerance: the forms' own bar, <= 1e-4 normwise relative amplitude error
against the FP64 KKT point, identical active sets (on noise-free channels a
column whose true amplitude is 0 may enter at round-off level, in the oracle
as well). The host build does not contract float expressions the
device compiler contracts, so it matches the GPU to these tolerances, not bit
for bit."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
CSRC = os.path.join(ROOT, "test-regression_gb300", "csrc")
CUDA_INCLUDE = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
AMP_TOL = 1e-4
PRECISIONS = {"mixed": 0, "fp32": 1}


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if not shutil.which("g++") or not os.path.exists(os.path.join(CUDA_INCLUDE, "cuda_runtime.h")):
        pytest.skip("needs g++ and the CUDA headers")
    out = str(tmp_path_factory.mktemp("mixedhost") / "libmixed_host.so")
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-w", "-I", CUDA_INCLUDE,
                    "-I", os.path.join(ROOT, "include"), "-I", CSRC, os.path.join(ROOT, "tests", "cpp", "mixed_host.cpp"),
                    "-x", "c++", os.path.join(CSRC, "tables.cu"), "-o", out], check=True)
    L = C.CDLL(out)
    L.mixed_host.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_int] + [C.c_void_p] * 8
    return L


def fit(lib, cond, samples, pederr, judge_df, max_iter=1000, warm_mask=None, warm_amp=None):
    """warm_mask / warm_amp: predicted passive sets and amplitudes (the warm
    start's pipeline), or None (cold start)."""
    n = samples.shape[0]
    N, K = cond.nsamples, cond.npulses
    s = np.ascontiguousarray(samples[:, :N], dtype=np.float64)
    pe = np.ascontiguousarray(pederr, dtype=np.float64)
    o = {"amplitudes": np.zeros((n, K)), "chi2": np.zeros(n), "active_mask": np.zeros(n, np.uint16),
         "status": np.zeros(n, np.uint8), "iters": np.zeros(n, np.int32)}
    q = np.zeros(2, np.uint32)
    wm = None if warm_mask is None else np.ascontiguousarray(warm_mask, dtype=np.uint16)
    wa = None if warm_amp is None else np.ascontiguousarray(warm_amp, dtype=np.float32)
    rc = lib.mixed_host(C.byref(cond), s.ctypes.data, pe.ctypes.data, n, judge_df, max_iter,
                        *[o[k].ctypes.data for k in ("amplitudes", "chi2", "active_mask", "status", "iters")],
                        q.ctypes.data, None if wm is None else wm.ctypes.data, None if wa is None else wa.ctypes.data)
    assert rc == 0
    o["fix_queue"], o["repair_queue"] = int(q[0]), int(q[1])
    return o


def rel_err(amp, ref):
    return np.abs(amp - ref).max(axis=1) / np.maximum(np.abs(ref).max(axis=1), 1e-300)


def check_against_kkt(o, ref_amp, ref_mask, ok, allow_roundoff_columns=False, roundoff=1e-9):
    err = rel_err(o["amplitudes"], ref_amp)
    assert (err[ok] <= AMP_TOL).all(), err[ok].max()
    diff = o["active_mask"] ^ ref_mask
    if not allow_roundoff_columns:
        assert (diff[ok] == 0).all(), np.nonzero(ok & (diff != 0))[0][:10]
        return
    scale = np.maximum(np.abs(ref_amp).max(axis=1), 1e-300)
    K = ref_amp.shape[1]
    for i in np.nonzero(ok & (diff != 0))[0]:
        cols = [k for k in range(K) if (int(diff[i]) >> k) & 1]
        assert all(abs(ref_amp[i, k]) <= roundoff * scale[i] and abs(o["amplitudes"][i, k]) <= roundoff * scale[i]
                   for k in cols), (i, cols)


@pytest.mark.parametrize("prec", list(PRECISIONS))
@pytest.mark.parametrize("name", ["ecal_c0", "ecal_logamp", "hcal", "edge"])
def test_fixture_within_bounds_of_kkt(mf, lib, name, prec):
    d = dict(np.load(os.path.join(GOLDEN, f"fits_{name}.npz")))
    cond = mf.make_conditions(d["P"], d["R"], d["bxs"])
    o = fit(lib, cond, d["samples"], d["pederr"], PRECISIONS[prec])
    ok = d["kkt_status"] == 0
    check_against_kkt(o, d["kkt_amplitudes"], d["kkt_active_mask"], ok, allow_roundoff_columns=name == "edge")
    assert np.array_equal(o["status"][ok], d["kkt_status"][ok])
    chi2_err = np.abs(o["chi2"] - d["kkt_chi2"]) / np.maximum(d["kkt_chi2"], 1.0)
    assert (chi2_err[ok] <= 1e-6).all(), chi2_err[ok].max()


@pytest.mark.parametrize("prec", list(PRECISIONS))
@pytest.mark.parametrize("workload", ["ecal-10m-logamp-pu4", "mixed-10m-ecal-hcal"])
def test_seeded_channels_within_bounds_of_kkt(mf, oracle, lib, workload, prec):
    """Seeded channels of the benchmark generators (log-uniform ECAL with
    pileup 4; the ECAL/HCAL mix with pileup U[0, 8]): every channel within the
    bar of the oracle's KKT fit, identical active sets, and the pipeline's
    queues in use (the screen finds columns for the fix; the judge sends a
    few channels to the FP64 repair)."""
    inp = oracle.synth_generate(workload, 0, 6000)
    fixq = repq = 0
    for kind in (0, 1):
        sel = np.nonzero(inp["ctype"] == kind)[0]
        if sel.size == 0:
            continue
        P, R, bxs, _ = oracle.synth_conditions(kind)
        cond = mf.make_conditions(P, R, bxs)
        s, pe = inp["samples"][sel], inp["pederr"][sel]
        ref = oracle.fit_batch(s, pe, P, R, bxs, max_iter_nnls=1000, start=1)
        o = fit(lib, cond, s, pe, PRECISIONS[prec])
        ok = ref["status"] == 0
        check_against_kkt(o, ref["amplitudes"], ref["active_mask"], ok)
        fixq += o["fix_queue"]
        repq += o["repair_queue"]
    assert fixq > 0
    if workload == "ecal-10m-logamp-pu4":
        assert repq > 0


@pytest.mark.parametrize("prec", list(PRECISIONS))
def test_exact_fits_keep_their_active_sets(mf, oracle, lib, prec):
    """Noise-free ECAL channels built from 6 to 10 positive pulses: the fit is
    exact (chi2 ~ 0), where the solve's round-off leaks into the residual and
    can flip the sign of a gradient. Every channel must still come out with
    the true pulses active and amplitudes within the bar; undecidable ones go
    to the FP64 repair."""
    P, R, bxs, _ = oracle.synth_conditions(0)
    rng = np.random.default_rng(23)
    n = 2000
    x = np.zeros((n, 10))
    for i in range(n):
        cols = rng.choice(10, size=rng.integers(6, 11), replace=False)
        x[i, cols] = 10.0 ** rng.uniform(-1, 3, size=cols.size)
    samples = x @ P.T
    pederr = np.full(n, 0.044)
    ref = oracle.fit_batch(samples, pederr, P, R, bxs, max_iter_nnls=1000, start=1)
    o = fit(lib, mf.make_conditions(P, R, bxs), samples, pederr, PRECISIONS[prec])
    # on ~2 % of such channels the oracle's FNNLS cycles on round-off until its
    # iteration cap (status NNLS_MAXITER), its amplitudes still exact
    # (a column whose true amplitude is 0 has a zero gradient at the exact fit
    # and enters or not on round-off, in the oracle as well; the oracle's normal
    # equations leave such columns at up to ~2e-7 of the largest amplitude, the
    # forms' QR-built tables at ~1e-15: the truth is the sharper check here)
    ok = ref["status"] == 0
    assert ok.mean() > 0.95
    assert (rel_err(o["amplitudes"], ref["amplitudes"])[ok] <= AMP_TOL).all()
    truth = ((x > 0).astype(np.uint16) << np.arange(10, dtype=np.uint16)).sum(axis=1).astype(np.uint16)
    assert ((o["active_mask"] & truth) == truth).all()  # every true pulse active
    extra = o["amplitudes"] * ((x == 0) & (o["amplitudes"] > 0))
    assert (extra.max(axis=1) <= 1e-9 * np.abs(x).max(axis=1)).all()  # others at round-off at most
    assert (rel_err(o["amplitudes"], x) <= 1e-6).all()


@pytest.mark.parametrize("prec", list(PRECISIONS))
def test_warm_pipeline_from_imperfect_predictions(mf, oracle, lib, prec):
    """The warm start's pipeline (search from a predicted set, judge queueing
    channels with provably missing columns for the fix, fix, second judge,
    repair), fed predictions that are the KKT sets with columns dropped and
    spurious ones added and amplitudes off by up to a factor of two, as a
    network's might be: every channel still ends within the bar of the KKT
    fit with the same active set, and the fix and second judge run."""
    P, R, bxs, _ = oracle.synth_conditions(0)
    inp = oracle.synth_generate("warm-eval-10m", 0, 6000)
    s, pe = inp["samples"], inp["pederr"]
    ref = oracle.fit_batch(s, pe, P, R, bxs, max_iter_nnls=1000, start=1)
    rng = np.random.default_rng(31)
    mask = ref["active_mask"].astype(np.uint32)
    drop = rng.random((len(pe), 10)) < 0.15
    add = rng.random((len(pe), 10)) < 0.05
    bits = 1 << np.arange(10)
    pred = (mask & ~(drop * bits).sum(axis=1)) | (add * bits).sum(axis=1)
    amp = (np.abs(ref["amplitudes"]) * rng.uniform(0.5, 2.0, size=(len(pe), 10)) + 0.01).astype(np.float32)
    o = fit(lib, mf.make_conditions(P, R, bxs), s, pe, PRECISIONS[prec], warm_mask=pred, warm_amp=amp)
    ok = ref["status"] == 0
    check_against_kkt(o, ref["amplitudes"], ref["active_mask"], ok)
    assert o["fix_queue"] > 0
    # a perfect prediction leaves nearly nothing to fix
    o2 = fit(lib, mf.make_conditions(P, R, bxs), s, pe, PRECISIONS[prec], warm_mask=ref["active_mask"],
             warm_amp=np.abs(ref["amplitudes"]).astype(np.float32))
    check_against_kkt(o2, ref["amplitudes"], ref["active_mask"], ok)
    assert o2["fix_queue"] < o["fix_queue"] / 4


@pytest.fixture(scope="module")
def fit_core_lib(tmp_path_factory):
    """The FP64 drop-in's routines compiled for the host (tests/cpp/fit_core_host.cpp)."""
    if not shutil.which("g++") or not os.path.exists(os.path.join(CUDA_INCLUDE, "cuda_runtime.h")):
        pytest.skip("needs g++ and the CUDA headers")
    out = str(tmp_path_factory.mktemp("fitcore_mixed") / "libfit_core_host.so")
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-w", "-I", CUDA_INCLUDE,
                    "-I", os.path.join(ROOT, "include"), "-I", CSRC,
                    os.path.join(ROOT, "tests", "cpp", "fit_core_host.cpp"), "-o", out], check=True)
    L = C.CDLL(out)
    L.fit_core_host.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int64] + \
        [C.c_int] * 4 + [C.c_int64, C.c_int, C.c_void_p, C.c_int] + [C.c_void_p] * 7
    return L


@pytest.mark.parametrize("errors", [0, 1])
@pytest.mark.parametrize("prec", list(PRECISIONS))
def test_per_channel_form_pulse_covariance(mf, oracle, lib, fit_core_lib, prec, errors):
    """The per-channel form on the CPU, as the engine composes it: the outer
    loop's first iteration through the tables (its covariance is pederr^2
    samplecor whatever the pulse covariance, the tables' problem), then the
    FP64 continuation with the pulse covariance and the reciprocal factor
    diagonal, seeded with that iteration's amplitudes, chi2 and status;
    against the oracle's FP64 fit to KKT convergence with the same pulse
    covariance: amplitudes and MINOS errors within 1e-4, identical active sets
    and outer-iteration counts."""
    import test_fit_core_host as fch

    F = np.zeros((19, 19))
    idx = np.arange(7, 19)
    F[np.ix_(idx, idx)] = 3e-4 * np.exp(-np.abs(np.subtract.outer(idx, idx)) / 3.0)
    P, R, bxs, _ = oracle.synth_conditions(0)
    inp = oracle.synth_generate("ecal-1m-pu2", 0, 3000)
    s, pe = inp["samples"], inp["pederr"]
    first = fit(lib, mf.make_conditions(P, R, bxs), s, pe, PRECISIONS[prec])
    o = fch.fit(fit_core_lib, mf.make_conditions(P, R, bxs, fullpulsecov=F), s, pe, 1, 1000, errors,
                fch.F_SEEDED | fch.F_RECIP, chunk=300, seed=first)
    ref = oracle.fit_batch(s, pe, P, R, bxs, fullpulsecov=F, max_iter_nnls=1000, start=1, compute_errors=bool(errors))
    ok = ref["status"] == 0
    assert ok.mean() > 0.99
    check_against_kkt(o, ref["amplitudes"], ref["active_mask"], ok)
    assert np.array_equal(o["iters"][ok] & 0xFF, np.minimum(ref["iters"][ok, 0], 255))
    assert (np.abs(o["chi2"] - ref["chi2"])[ok] <= 1e-6 * np.maximum(ref["chi2"][ok], 1.0)).all()
    if errors:
        fin = ok & np.isfinite(ref["errors"])
        assert (np.abs(o["errors"] - ref["errors"])[fin] <= 1e-4 * np.abs(ref["errors"][fin])).all()
    # the pulse covariance makes the outer loop iterate past the tables' first iteration
    assert (ref["iters"][:, 0] > 2).mean() > 0.5
