"""Generates tests/golden/ocl_fnnls_ref.npz: outputs of the reference's own
plain-C FNNLS -- the OpenCL kernel source multifit_ocl/device/
regression_inplace_fnnls.cl, compiled unmodified as C into oracle/_ref by
oracle/build_oracle.py (build_ref_ocl) -- on seeded whitened ECAL problems,
so that the pin of the oracle's FNNLS loop holds where the reference tree is
absent.

Problems: A = L^-1 P and b = L^-1 s of synthetic ECAL channels (the engine's
counter-based generator: 1-100 GeV with pileup 0.5, and log-uniform
0.1-1000 GeV with pileup 4), each from the empty start (x0 = 0) and from a
warm start with stale entries (the reference's second-call situation:
non-zero x outside the passive set); eps 1e-11, max_iter 1000. Stored: A, b,
x0, the FP64 build's x (float mapped to double) and the FP32 build's x (the
kernel as written).

Usage: python tests/golden/make_ocl_golden.py
"""
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

spec = importlib.util.spec_from_file_location("multifit_gb300", os.path.join(ROOT, "test-regression_gb300",
                                                                             "__init__.py"))
mf = importlib.util.module_from_spec(spec)
sys.modules["multifit_gb300"] = mf
spec.loader.exec_module(mf)

OUT = os.path.join(HERE, "ocl_fnnls_ref.npz")
PER_SET = 300


def problems():
    cond, _ = mf.synth_conditions(mf.SYNTH_ECAL)
    P, R, _, _ = mf.conditions_arrays(cond)
    Lc = np.linalg.cholesky(R)
    rng = np.random.default_rng(77)
    out = []
    for seed, kw in ((21, dict(lo=1.0, hi=100.0, pileup_mean=0.5)),
                     (22, dict(intime_log=True, lo=0.1, hi=1000.0, pileup_mean=4.0))):
        d = mf.synth_generate_host(mf.synth_params(seed, PER_SET, **kw), 0, PER_SET, with_truth=False)
        for i in range(PER_SET):
            Ls = Lc * d["pederr"][i]
            A = np.linalg.solve(Ls, P)
            b = np.linalg.solve(Ls, d["samples"][i])
            out.append((A, b, np.zeros(10)))
            warm = np.abs(rng.standard_normal(10)) * np.abs(b).max() * (rng.random(10) < 0.5)
            out.append((A, b, warm))
    return out


def main():
    if oracle.ref_ocl(64) is None:
        raise SystemExit("the reference tree is needed to build the OpenCL FNNLS into oracle/_ref")
    probs = problems()
    A = np.stack([p[0] for p in probs])
    b = np.stack([p[1] for p in probs])
    x0 = np.stack([p[2] for p in probs])
    x64 = np.stack([oracle.ref_ocl_inplace_fnnls(a, bb, xx, bits=64) for a, bb, xx in probs])
    x32 = np.stack([oracle.ref_ocl_inplace_fnnls(a, bb, xx, bits=32) for a, bb, xx in probs])
    np.savez_compressed(OUT, A=A, b=b, x0=x0, x64=x64, x32=x32)
    print(OUT, A.shape, "non-finite FP32 results:", int((~np.isfinite(x32)).any(axis=1).sum()))


if __name__ == "__main__":
    main()
