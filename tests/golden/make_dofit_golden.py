"""Generates tests/golden/dofit_ref.npz: outputs of the reference's own
multifit_cpu fit -- PulseChiSqSNNLS::DoFit with its Minimize, updateCov,
NNLS and ComputeApproxUncertainty (multifit_cpu/src/PulseChiSqSNNLS.cpp) and
inplace_fnnls (nnls/src/inplace_fnnls.cu), compiled unmodified from the
reference tree over the oracle's Eigen shim (oracle/build_oracle.py,
build_ref_dofit) -- so that the oracle and the engine's FP64 kernel are pinned
to it where the reference tree is absent.

Inputs (seeded, from the oracle's generator, the ECAL condition set the
reference driver builds):
  c0      channels 0..399 of ecal-10k-pu0.5 (in-time U[1,100], pileup 0.5)
  logamp  channels 1000..1399 of ecal-10m-logamp-pu4 (log-uniform, pileup 4)
  warm    channels 5,000,000..5,000,399 of warm-eval-10m
  fpc     channels 0..199 of ecal-1m-pu2 with a non-zero pulse covariance
          (1e-4 exp(-|i-j|/3) over the template's samples; the outer loop
          iterates for real)
  edge    the hand-made edge channels of tests/golden/fits_edge.npz
Each set is fitted twice: errors off (disableErrorCalculation, as the
reference driver does) and on (the MINOS-like in-time uncertainty).

Usage: MULTIFIT_REFERENCE_ROOT=<reference tree> python tests/golden/make_dofit_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402


def pulse_covariance():
    F = np.zeros((19, 19))
    idx = np.arange(7, 19)
    F[np.ix_(idx, idx)] = 1e-4 * np.exp(-np.abs(np.subtract.outer(idx, idx)) / 3.0)
    return F


def inputs():
    edge = np.load(os.path.join(HERE, "fits_edge.npz"))
    sets = {
        "c0": (oracle.synth_generate("ecal-10k-pu0.5", 0, 400), None),
        "logamp": (oracle.synth_generate("ecal-10m-logamp-pu4", 1000, 400), None),
        "warm": (oracle.synth_generate("warm-eval-10m", 5_000_000, 400), None),
        "fpc": (oracle.synth_generate("ecal-1m-pu2", 0, 200), pulse_covariance()),
        "edge": ({"samples": edge["samples"], "pederr": edge["pederr"]}, None),
    }
    return sets


def main() -> int:
    if oracle.ref_dofit_lib() is None:
        print("the reference tree is absent: nothing generated")
        return 1
    P, R, bxs, _ = oracle.synth_conditions(oracle.SYNTH_ECAL)
    fp = oracle.fullpulse_of(P, bxs)
    out = {"P": P, "R": R, "bxs": bxs, "fullpulse": fp, "fullpulsecov": pulse_covariance()}
    for name, (d, F) in inputs().items():
        out[f"{name}_samples"] = d["samples"]
        out[f"{name}_pederr"] = d["pederr"]
        out[f"{name}_has_fpc"] = np.array(F is not None)
        for err in (0, 1):
            r = oracle.ref_dofit(d["samples"], d["pederr"], R, bxs, fp, F, compute_errors=bool(err))
            for k in ("amplitudes", "chi2", "errors", "ok"):
                out[f"{name}_e{err}_{k}"] = r[k]
    path = os.path.join(HERE, "dofit_ref.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")
    return 0


if __name__ == "__main__":
    sys.exit(main())
