"""The reference's ECAL data files replayed through the engine.

Mirrors, without ROOT (the files are read by ``rootio``):

- ``Pulse`` (multifit_cpu/interface/Pulse.h:38-168; io/interface/Pulse.h is
  the same file): the pulse shape of ``EmptyFile.root`` -- the TGraph
  ``PulseShape/grPulseShape`` below 800 ns, the exponential tail of the
  ``PulseShape/Tail`` tree above -- and the CRRC noise correlation of
  ``NoiseInit``;
- the driver's conditions (multifit_cpu/src/multifit.cpp:45-81): a 12-sample
  template at fullpulse(7..18), the correlation matrix corr(|i-j|), BXs -5..4;
- ``ecal_data_io`` (io/src/ecal_data_io.cpp:6-53): entries of the ``Samples``
  tree as (samples, pulse matrix), read round-robin;
- ``replay`` (multifit.cpp:83-271, its first iteration): every entry fitted
  with pederr 1.0 and the error calculation off, the in-time amplitude and the
  per-BX amplitudes packed as the driver packs them, and the driver's physics
  check -- mean and RMS of (reconstructed - true) in-time amplitude, as the
  histogram ``h01`` (1000 bins over [-5, 5)) reports them.

Every fit runs on the GPU through the engine's C ABI; this module only reads
files and prepares inputs.
"""
from __future__ import annotations

import math
import sys

import numpy as np

from . import rootio

NSAMPLES = 10
NFREQ = 25            # ns between samples
IDSTART = 150 + 13    # position of the first sample in the waveform (ns)
TAU = 43.0            # CRRC shaping time (ns), for the noise correlation
TAIL_START = 800.0    # the shape switches from the graph to the exponential tail here (ns)
ACTIVE_BXS = np.arange(-5, 5, dtype=np.int8)
PEDRMS = 1.0          # the driver's pederr
H01_RANGE = (-5.0, 5.0)


def graph_eval(x_pts: np.ndarray, y_pts: np.ndarray, x: float, sorted_x: bool) -> float:
    """Linear interpolation of a TGraph at x, as TGraph::Eval without a
    spline: the two neighbours of x (the two nearest points on one side when x
    lies outside the abscissa range), y = y_up + (x - x_up)(y_low - y_up) /
    (x_low - x_up). A graph not flagged sorted returns the point's own y where
    x equals an abscissa; a sorted one interpolates between the point at or
    below x and the next."""
    n = len(x_pts)
    if n == 0:
        return 0.0
    if n == 1:
        return float(y_pts[0])
    if sorted_x:
        low = int(np.searchsorted(x_pts, x, side="right")) - 1  # last index with x_pts <= x
        if low == n - 1:
            up, low = low, low - 1
        elif low == -1:
            low, up = 0, 1
        else:
            up = low + 1
    else:
        low = up = low2 = up2 = -1
        for i in range(n):
            xi = x_pts[i]
            if xi < x:
                if low == -1 or xi > x_pts[low]:
                    low2, low = low, i
                elif low2 == -1:
                    low2 = i
            elif xi > x:
                if up == -1 or xi < x_pts[up]:
                    up2, up = up, i
                elif up2 == -1:
                    up2 = i
            else:
                return float(y_pts[i])
        if up == -1:
            up, low = low, low2
        if low == -1:
            low, up = up, up2
    if x_pts[low] == x_pts[up]:
        return float(y_pts[low])
    return float(y_pts[up] + (x - x_pts[up]) * (y_pts[low] - y_pts[up]) / (x_pts[low] - x_pts[up]))


class Pulse:
    """Pulse shape and noise correlation of a pulse-shape file."""

    def __init__(self, shape_file: str):
        f = rootio.RootFile(shape_file)
        self.gx, self.gy, bits = f.graph("PulseShape/grPulseShape")
        self.sorted_x = bool(bits & rootio.IS_SORTED_X)
        tail = f.tree("PulseShape/Tail")
        # float branches, widened to double as the C++ arithmetic widens them
        self.tmin = float(tail.array("timeMin", np.float32)[0])
        self.par0 = float(tail.array("expAmplitude", np.float32)[0])
        self.par1 = float(tail.array("expTime", np.float32)[0])
        self.mC = np.zeros(NSAMPLES)
        for i in range(NSAMPLES):
            y = 1.0 - math.exp(-float(NFREQ * i) / (math.sqrt(2.0) * TAU))
            self.mC[i] = 1.0 - y * y

    def fShape(self, x: float) -> float:
        if x > 0.0:
            if x < TAIL_START:
                y = graph_eval(self.gx, self.gy, x, self.sorted_x)
                return 0.0 if y <= 0 else y
            return self.par0 * math.exp(-x * self.par1)
        return 0.0

    def corr(self, i: int) -> float:
        return float(self.mC[i])


def driver_template(pulse: Pulse) -> np.ndarray:
    """The 12 template samples (in-time at index 2): fShape at
    IDSTART + NFREQ*(i+3) + NFREQ - 250 ns."""
    return np.array([pulse.fShape(float(IDSTART + NFREQ * (i + 3) + NFREQ - 500 // 2))
                     for i in range(NSAMPLES + 2)])


def driver_fullpulse(pulse: Pulse) -> np.ndarray:
    fp = np.zeros(NSAMPLES + 9)
    fp[7:7 + NSAMPLES + 2] = driver_template(pulse)
    return fp


def driver_noisecor(pulse: Pulse) -> np.ndarray:
    idx = np.arange(NSAMPLES)
    return pulse.mC[np.abs(idx[:, None] - idx[None, :])]


def driver_conditions(mf, pulse: Pulse):
    """The driver's condition set: (MfConditions, fullpulse, noisecor)."""
    fp = driver_fullpulse(pulse)
    R = driver_noisecor(pulse)
    P = mf.build_pulse_matrix(fp, ACTIVE_BXS, NSAMPLES)
    return mf.make_conditions(P, R, ACTIVE_BXS), fp, R


class ecal_data_io:  # noqa: N801 -- the reference's class name
    """Entries of a ``Samples`` tree: ``get_one_entry`` returns (samples,
    pulse matrix) and advances round-robin over the tree."""

    def __init__(self, file_name: str, shape_file: str, mf=None):
        tree = rootio.RootFile(file_name).tree("Samples")
        self.entries = int(tree.entries)
        self.truth = tree.array("amplitudeTruth", np.float64)
        vecs = tree.vectors("samples", np.float64)
        self.samples = np.zeros((self.entries, NSAMPLES))
        for i, v in enumerate(vecs):
            if v.size > NSAMPLES:
                raise rootio.RootFormatError(f"{file_name}: entry {i} has {v.size} samples, more than {NSAMPLES}")
            self.samples[i, :v.size] = v
        self.pulse = Pulse(shape_file)
        self.fullpulse = driver_fullpulse(self.pulse)
        if mf is None:
            mf = sys.modules[__package__]  # the engine package this module belongs to
        self.pulse_matrix = mf.build_pulse_matrix(self.fullpulse, ACTIVE_BXS, NSAMPLES)
        self.ientry = 0

    def get_one_entry(self):
        i = self.ientry % self.entries
        self.ientry += 1
        return self.samples[i].copy(), self.pulse_matrix.copy()

    def get_n_entries(self, n: int):
        return [self.get_one_entry() for _ in range(n)]


def h01_summary(d: np.ndarray, lo: float = H01_RANGE[0], hi: float = H01_RANGE[1]) -> dict:
    """Mean, RMS and entry count of (reco - truth) as a fixed-range histogram
    reports them: each fill inside [lo, hi) adds to the running sums of x and
    x^2 in fill order (fills outside count as entries only); mean = sum x / n,
    RMS = sqrt(|sum x^2 / n - mean^2|)."""
    d = np.asarray(d, dtype=np.float64)
    sw = sx = sx2 = 0.0
    for v in d.tolist():
        if lo <= v < hi:
            sw += 1.0
            sx += v
            sx2 += v * v
    if sw == 0:
        return {"mean": 0.0, "rms": 0.0, "entries": int(d.size), "in_range": 0}
    mean = sx / sw
    rms = math.sqrt(abs(sx2 / sw - mean * mean))
    return {"mean": mean, "rms": rms, "entries": int(d.size), "in_range": int(sw)}


def replay_arrays(engine, samples: np.ndarray, truth: np.ndarray, fullpulse: np.ndarray, noisecor: np.ndarray,
                  options=None, pederr: float = PEDRMS) -> dict:
    """The driver's fit loop and physics check on channels already read:
    samples (n, 10), true in-time amplitudes (n,), the driver's fullpulse (19,)
    and noise correlation (10, 10). Fits on the GPU (the engine's FP64 form
    unless ``options`` says otherwise; error calculation off). Replaces the
    engine's condition set 0 with the driver's."""
    mf = sys.modules[__package__]
    samples = np.ascontiguousarray(samples, dtype=np.float64)
    n = samples.shape[0]
    P = mf.build_pulse_matrix(fullpulse, ACTIVE_BXS, NSAMPLES)
    engine.set_conditions(0, mf.make_conditions(P, noisecor, ACTIVE_BXS))
    opt = options if options is not None else mf.default_options(compute_errors=0)
    out = engine.fit_host(samples, np.full(n, pederr), options=opt)
    # multifit.cpp:203-223: ampl = X[first k with bx_k = 0]; v_ampl[bx_k + 5] = X[k]
    v_ampl = np.zeros((n, ACTIVE_BXS.size))
    v_ampl[:, ACTIVE_BXS.astype(np.int64) + 5] = out["amplitudes"][:, :ACTIVE_BXS.size]
    ampl = out["intime"]
    return {"ampl": ampl, "v_ampl": v_ampl, "amplitudes": out["amplitudes"][:, :ACTIVE_BXS.size],
            "chi2": out["chi2"], "status": out["status"], "active_mask": out["active_mask"],
            "h01": h01_summary(ampl - np.asarray(truth, dtype=np.float64))}


def replay(engine, file_name: str, shape_file: str, entries: int | None = None, options=None,
           pederr: float = PEDRMS) -> dict:
    """Fits ``entries`` channels of a ``Samples`` file (round-robin; default:
    every entry once) with the conditions the driver builds from the
    pulse-shape file; returns ``replay_arrays``'s outputs plus the inputs."""
    mf = sys.modules[__package__]
    io = ecal_data_io(file_name, shape_file, mf)
    n = io.entries if entries is None else int(entries)
    idx = np.arange(n) % io.entries
    noisecor = driver_noisecor(io.pulse)
    res = replay_arrays(engine, io.samples[idx], io.truth[idx], io.fullpulse, noisecor, options, pederr)
    res.update(samples=io.samples[idx], truth=io.truth[idx], fullpulse=io.fullpulse, noisecor=noisecor)
    return res
