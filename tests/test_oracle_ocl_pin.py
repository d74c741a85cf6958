"""The oracle's FNNLS loop pinned to reference code compiled here: the
reference's plain-C twin of the incremental-Cholesky FNNLS, the OpenCL kernel
source multifit_ocl/device/regression_inplace_fnnls.cl:352-587 (N = K = 10),
compiled unmodified as C (oracle/ref_ocl_fnnls_driver.c, built by
oracle/build_oracle.py into oracle/_ref with the source's own roundings).

- Its FP64 build (float mapped to double) equals, bit for bit, the oracle
  built with separate rounding of every product and sum (ORACLE_SEPARATE_
  ROUNDING), from the empty start and from warm starts with stale entries --
  live where the reference tree is present, and always against the committed
  outputs in tests/golden/ocl_fnnls_ref.npz.
- The oracle's canonical build (every a*b + c one FMA) differs from that only
  at round-off: same active sets, amplitudes within 1e-7 relative (measured
  2.8e-9).
- The kernel as the reference wrote it, in FP32, is recorded against the FP64
  oracle: with the absolute eps 1e-11 and FP32 Cholesky updates it returns
  non-finite values or misses 1e-4 on a large share of ECAL problems. The
  engine's mixed form keeps FP64 for its judge for this reason."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ocl_fnnls_ref.npz")


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLDEN))


def relerr(x, r):
    return np.abs(x - r).max() / max(np.abs(r).max(), 1e-300)


def test_separate_rounding_oracle_equals_committed_reference_outputs(oracle, gold):
    for A, b, x0, x64 in zip(gold["A"], gold["b"], gold["x0"], gold["x64"]):
        for variant in (1, 0):  # incremental factor, and the fresh LLT per inner step
            x, _ = oracle.inplace_fnnls(A, b, x0, eps=1e-11, max_iter=1000, variant=variant, start=0,
                                        separate_rounding=True)
            assert np.array_equal(x, x64)


def test_separate_rounding_oracle_equals_live_reference_build(oracle, mf):
    if oracle.ref_ocl(64) is None:
        pytest.skip("the reference tree is absent (the committed outputs cover the pin)")
    assert oracle.ref_ocl(64).ref_ocl_data_type_bytes() == 8
    assert oracle.ref_ocl(32).ref_ocl_data_type_bytes() == 4
    cond, _ = mf.synth_conditions(mf.SYNTH_ECAL)
    P, R, _, _ = mf.conditions_arrays(cond)
    Lc = np.linalg.cholesky(R)
    d = mf.synth_generate_host(mf.synth_params(31, 600, intime_log=True, lo=0.1, hi=1000.0, pileup_mean=-8.0),
                               0, 600, with_truth=False)
    rng = np.random.default_rng(5)
    for i in range(600):
        Ls = Lc * d["pederr"][i]
        A = np.linalg.solve(Ls, P)
        b = np.linalg.solve(Ls, d["samples"][i])
        for x0 in (np.zeros(10), np.abs(rng.standard_normal(10)) * np.abs(b).max() * (rng.random(10) < 0.5)):
            ref = oracle.ref_ocl_inplace_fnnls(A, b, x0, bits=64)
            x, _ = oracle.inplace_fnnls(A, b, x0, eps=1e-11, max_iter=1000, variant=1, start=0,
                                        separate_rounding=True)
            assert np.array_equal(x, ref), i
    # a few random dense problems, well and badly conditioned
    for k in range(200):
        A = rng.standard_normal((10, 10)) @ np.diag(np.geomspace(1.0, 10.0 ** rng.uniform(0, 5), 10))
        b = rng.standard_normal(10) * 10
        ref = oracle.ref_ocl_inplace_fnnls(A, b, bits=64)
        x, _ = oracle.inplace_fnnls(A, b, eps=1e-11, max_iter=1000, variant=1, separate_rounding=True)
        assert np.array_equal(x, ref), k


def test_fma_and_separate_rounding_builds_agree_to_roundoff(oracle, gold):
    same_sets = 0
    for A, b, x0, x64 in zip(gold["A"], gold["b"], gold["x0"], gold["x64"]):
        x, _ = oracle.inplace_fnnls(A, b, x0, eps=1e-11, max_iter=1000, variant=1, start=0)
        same_sets += int(np.array_equal(x > 0, x64 > 0))
        if np.array_equal(x > 0, x64 > 0):
            # the normal-equations solve amplifies one rounding by up to
            # cond(A_S)^2 (about 2.5e9 for the ECAL set): 1e-7 relative
            assert relerr(x, x64) < 1e-7
    assert same_sets >= 0.999 * len(gold["A"])


def test_reference_fp32_kernel_against_fp64(oracle, gold):
    """What the reference's FP32 kernel gives on these ECAL problems (recorded:
    non-finite results and misses of 1e-4 on a large share)."""
    x32 = gold["x32"].astype(np.float64)
    finite = np.isfinite(x32).all(axis=1)
    errs = np.array([relerr(x32[i], gold["x64"][i]) for i in np.nonzero(finite)[0]])
    assert (~finite).mean() > 0.01           # an FP32 pivot that reached zero or below
    assert (errs > 1e-4).mean() > 0.05       # beyond the amplitude bound
    assert np.median(errs) < 1e-4            # typical channels are still FP32-accurate
    if oracle.ref_ocl(32) is not None:
        for i in range(0, len(gold["A"]), 37):
            live = oracle.ref_ocl_inplace_fnnls(gold["A"][i], gold["b"][i], gold["x0"][i], bits=32)
            assert np.array_equal(live, gold["x32"][i], equal_nan=True)
