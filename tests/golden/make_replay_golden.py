"""Generates tests/golden/replay_mysample_100.npz: the reference's own ECAL
data file replayed the way its driver replays it, so that the parity tests
can run where the data file is absent.

Reads, with the engine's ROOT-format reader (test-regression_gb300/rootio.py)
and the driver mirror (ecal_data_io.py), from the reference tree:
  data/mysample_100_0.000_0.000_10_25.00_10.00_0.00_1.000_1.00_CRRC43_0.00_slew_1.00.root
      the Samples tree: 100 entries of 10 samples and the true in-time
      amplitude, plus metadata branches (nSmpl, nFreq, pulse_tau,
      sigmaNoise, signalTruth) that the tests hold against the file name;
  data/EmptyFile.root
      the pulse shape (TGraph PulseShape/grPulseShape and the Tail tree)
      from which the driver builds its template (multifit_cpu/src/
      multifit.cpp:45-81).
Stores those inputs, the driver's fullpulse and noise correlation, and the
oracle's fits of every entry (pederr 1.0, no errors): the reference start
with max_iter 10 (the multifit_cpu configuration) and the support start at
KKT convergence (max_iter 1000), with the driver's physics check (mean and
RMS of reconstructed minus true in-time amplitude).

Usage: python tests/golden/make_replay_golden.py
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
import multifit_gb300.ecal_data_io as eio  # noqa: E402
import multifit_gb300.rootio as rootio  # noqa: E402

from oracle import build_oracle  # noqa: E402

DATA = os.path.join(build_oracle.REFERENCE_ROOT, "data")
SAMPLE_FILE = "mysample_100_0.000_0.000_10_25.00_10.00_0.00_1.000_1.00_CRRC43_0.00_slew_1.00.root"
SHAPE_FILE = "EmptyFile.root"
OUT = os.path.join(HERE, "replay_mysample_100.npz")


def main():
    sample_path = os.path.join(DATA, SAMPLE_FILE)
    shape_path = os.path.join(DATA, SHAPE_FILE)
    if not (os.path.exists(sample_path) and os.path.exists(shape_path)):
        raise SystemExit(f"the reference data files are needed under {DATA}")
    io = eio.ecal_data_io(sample_path, shape_path, mf)
    tree = rootio.RootFile(sample_path).tree("Samples")
    pulse = io.pulse
    R = eio.driver_noisecor(pulse)
    P = io.pulse_matrix
    n = io.entries
    pederr = np.full(n, eio.PEDRMS)
    d = {
        "samples": io.samples, "truth": io.truth, "fullpulse": io.fullpulse, "noisecor": R, "P": P,
        "bxs": eio.ACTIVE_BXS, "template": eio.driver_template(pulse),
        "tail": np.array([pulse.tmin, pulse.par0, pulse.par1]),
        "graph_points": np.array(len(pulse.gx)), "graph_sorted": np.array(pulse.sorted_x),
        "entries": np.array(tree.entries),
        "nSmpl": tree.array("nSmpl", np.int32), "nFreq": tree.array("nFreq", np.float32),
        "pulse_tau": tree.array("pulse_tau", np.float32), "sigmaNoise": tree.array("sigmaNoise", np.float32),
        "signalTruth": tree.array("signalTruth", np.float64),
    }
    for mode, kw in (("ref", dict(start=0, max_iter_nnls=10)), ("kkt", dict(start=1, max_iter_nnls=1000))):
        r = oracle.fit_batch(io.samples, pederr, P, R, eio.ACTIVE_BXS, **kw)
        for k in ("amplitudes", "chi2", "active_mask", "status"):
            d[f"{mode}_{k}"] = r[k]
        h = eio.h01_summary(r["amplitudes"][:, 5] - io.truth)
        d[f"{mode}_h01"] = np.array([h["mean"], h["rms"], h["entries"], h["in_range"]])
    np.savez_compressed(OUT, **d)
    print(OUT, {k: v.shape for k, v in d.items()}, "h01 ref", d["ref_h01"])


if __name__ == "__main__":
    main()
