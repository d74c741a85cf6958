"""The FP64 drop-in's device routines (csrc/fit_core.cuh) and its warp loop
compiled for the host (tests/cpp/fit_core_host.cpp, the warp's 32 lanes in
lockstep) and run on the CPU: bit for bit against the golden fixtures, the
reference's own DoFit outputs and the oracle (executed flop counts included),
for the specialised 10x10 / 8x8 and the generic-shape instantiations and for
warps given one batch, ragged ranges or hundreds of channels each (lanes
taking their next channel as their own finishes); the warp's staging of
samples with padded strides, amplitudes written to wider rows, channels of
another condition set skipped and out-of-range set indices flagged; and the
per-channel form's seeded continuation, which from the oracle's first outer
iteration must finish the oracle's fit bit for bit.

Tolerance: zero (same operations in the same order; IEEE fma, division and
sqrt on both sides)."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from _helpers import pack_iters

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
CUDA_INCLUDE = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
MODES = {"ref": (0, 10, 0), "kkt": (1, 1000, 0), "err": (1, 1000, 1)}
F_COUNT, F_RECIP, F_GENERIC, F_SEEDED = 1, 2, 4, 8


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if not shutil.which("g++") or not os.path.exists(os.path.join(CUDA_INCLUDE, "cuda_runtime.h")):
        pytest.skip("needs g++ and the CUDA headers")
    out = str(tmp_path_factory.mktemp("fitcore") / "libfit_core_host.so")
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-w", "-I", CUDA_INCLUDE,
                    "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "test-regression_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cpp", "fit_core_host.cpp"), "-o", out], check=True)
    L = C.CDLL(out)
    L.fit_core_host.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int64] + \
        [C.c_int] * 4 + [C.c_int64, C.c_int, C.c_void_p, C.c_int] + [C.c_void_p] * 7
    return L


def fit(lib, cond, samples, pederr, start, max_iter, errors, flags=0, chunk=96, ctype=None, sample_stride=None,
        amp_stride=None, seed=None, fill=0.0, max_iter_outer=50):
    """chunk: channels per warp; ctype: per-channel condition set (1: another
    launch's, 2: out of range), or None."""
    n = samples.shape[0]
    N, K = cond.nsamples, cond.npulses
    ss = sample_stride or N
    ast = amp_stride or K
    s = np.full((n, ss), 7.0)
    s[:, :N] = samples[:, :N]
    pe = np.ascontiguousarray(pederr, dtype=np.float64)
    o = {"amplitudes": np.full((n, ast), fill), "chi2": np.zeros(n), "intime": np.zeros(n), "errors": np.zeros(n),
         "active_mask": np.zeros(n, np.uint16), "status": np.zeros(n, np.uint8), "iters": np.zeros(n, np.int32),
         "flops": np.zeros(n)}
    if seed is not None:
        o["amplitudes"][:, :K] = seed["amplitudes"]
        o["chi2"][:] = seed["chi2"]
        o["status"][:] = seed["status"]
    ct = None if ctype is None else np.ascontiguousarray(ctype, dtype=np.uint8)
    rc = lib.fit_core_host(C.byref(cond), s.ctypes.data, ss, pe.ctypes.data, None if ct is None else ct.ctypes.data,
                           n, start, max_iter, errors, flags, chunk, max_iter_outer, o["amplitudes"].ctypes.data, ast,
                           *[o[k].ctypes.data for k in ("chi2", "intime", "errors", "active_mask", "status", "iters",
                                                        "flops")])
    assert rc == 0
    return o


@pytest.mark.parametrize("generic", [False, True])
@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("name", ["ecal_c0", "ecal_logamp", "hcal", "ecal_fpc", "edge"])
def test_fixture_bit_for_bit(mf, lib, name, mode, generic):
    d = dict(np.load(os.path.join(GOLDEN, f"fits_{name}.npz")))
    cond = mf.make_conditions(d["P"], d["R"], d["bxs"], fullpulsecov=d.get("fullpulsecov"))
    start, max_iter, errors = MODES[mode]
    # one warp for the whole fixture, or ragged 77-channel ranges
    o = fit(lib, cond, d["samples"], d["pederr"], start, max_iter, errors, F_GENERIC if generic else 0,
            chunk=77 if generic else 1 << 30)
    for k in ("amplitudes", "chi2", "active_mask", "status"):
        assert np.array_equal(o[k], d[f"{mode}_{k}"]), k
    assert np.array_equal(o["iters"], pack_iters(d[f"{mode}_iters"]))
    if errors:
        assert np.array_equal(o["errors"], d["err_errors"], equal_nan=True)


@pytest.mark.parametrize("errors", [0, 1])
@pytest.mark.parametrize("name", ["c0", "logamp", "warm", "fpc", "edge"])
def test_reference_dofit_bit_for_bit(mf, lib, name, errors):
    g = dict(np.load(os.path.join(GOLDEN, "dofit_ref.npz")))
    F = g["fullpulsecov"] if bool(g[f"{name}_has_fpc"]) else None
    cond = mf.make_conditions(g["P"], g["R"], g["bxs"], fullpulsecov=F)
    o = fit(lib, cond, g[f"{name}_samples"], g[f"{name}_pederr"], 0, 10, errors)
    assert np.array_equal(o["amplitudes"], g[f"{name}_e{errors}_amplitudes"])
    assert np.array_equal(o["chi2"], g[f"{name}_e{errors}_chi2"])
    if errors:
        assert np.array_equal(o["errors"], g[f"{name}_e{errors}_errors"], equal_nan=True)


def synthetic_sets(oracle, n):
    """(label, conditions arrays, samples, pederr) of seeded ECAL / HCAL channels,
    ECAL also with a pulse covariance."""
    fpc = dict(np.load(os.path.join(GOLDEN, "fits_ecal_fpc.npz")))["fullpulsecov"] * 3.0
    out = []
    for wl in ("ecal-1m-pu2", "ecal-10m-logamp-pu4", "mixed-10m-ecal-hcal"):
        inp = oracle.synth_generate(wl, 0, n)
        for kind in (0, 1):
            sel = np.nonzero(inp["ctype"] == kind)[0]
            if sel.size == 0:
                continue
            P, R, bxs, _ = oracle.synth_conditions(kind)
            for F in ([None, fpc] if kind == 0 and wl != "mixed-10m-ecal-hcal" else [None]):
                out.append((f"{wl}/set{kind}/fpc={F is not None}", (P, R, bxs, F), inp["samples"][sel],
                            inp["pederr"][sel]))
    return out


@pytest.mark.parametrize("setting", [(0, 10, 0), (1, 1000, 0), (1, 1000, 1), (0, 1000, 1)])
def test_oracle_bit_for_bit_with_flop_counts(mf, oracle, lib, setting):
    start, max_iter, errors = setting
    for label, (P, R, bxs, F), s, pe in synthetic_sets(oracle, 3000):
        cond = mf.make_conditions(P, R, bxs, fullpulsecov=F)
        ref = oracle.fit_batch(s, pe, P, R, bxs, fullpulsecov=F, max_iter_nnls=max_iter, start=start,
                               compute_errors=bool(errors), count_flops=True)
        for flags, chunk in ((0, 640), (F_COUNT, 32)):
            o = fit(lib, cond, s, pe, start, max_iter, errors, flags, chunk=chunk)
            keys = ["amplitudes", "chi2", "active_mask", "status"] + (["errors"] if errors else [])
            keys += ["flops"] if flags == F_COUNT else []
            for k in keys:
                assert np.array_equal(o[k], ref[k], equal_nan=True), (label, flags, k)
            assert np.array_equal(o["iters"], pack_iters(ref["iters"])), label


@pytest.mark.parametrize("chunk", [20, 77, 1 << 30])
@pytest.mark.parametrize("strides", [(13, 12), (10, 11), (16, 10), (10, 10)])
def test_staging_strides_and_other_sets(mf, lib, strides, chunk):
    """Samples read from rows wider than N, amplitudes written to rows wider than
    K (zeros up to KMAX, nothing beyond); channels of another condition set
    (every third one) neither fitted nor written, channels with an
    out-of-range set index flagged (status BADINPUT, chi2 0)."""
    d = dict(np.load(os.path.join(GOLDEN, "fits_ecal_logamp.npz")))
    cond = mf.make_conditions(d["P"], d["R"], d["bxs"])
    n = 250
    ss, ast = strides
    idx = np.arange(n)
    ctype = np.where(idx % 3 == 2, 1, 0)
    ctype[idx % 41 == 40] = 2
    o = fit(lib, cond, d["samples"][:n], d["pederr"][:n], 0, 10, 0, chunk=chunk, ctype=ctype, sample_stride=ss,
            amp_stride=ast, fill=-5.0)
    mine, other, bad = ctype == 0, ctype == 1, ctype == 2
    assert np.array_equal(o["amplitudes"][mine, :10], d["ref_amplitudes"][:n][mine])
    assert np.array_equal(o["chi2"][mine], d["ref_chi2"][:n][mine])
    assert np.array_equal(o["status"][mine], d["ref_status"][:n][mine])
    assert (o["amplitudes"][other | bad] == -5.0).all() and (o["chi2"][other] == 0).all()
    assert (o["status"][bad] == 8).all() and (o["chi2"][bad] == 0).all()
    assert (o["amplitudes"][:, 10:] == -5.0).all()


@pytest.mark.parametrize("errors", [0, 1])
def test_seeded_continuation_finishes_the_oracle_fit(mf, oracle, lib, errors):
    """The per-channel form hands the FP64 kernel the first outer iteration's
    amplitudes, chi2 and status; from the oracle's own first iteration the
    kernel's continuation (division variant) must end at the oracle's full fit."""
    fpc = dict(np.load(os.path.join(GOLDEN, "fits_ecal_fpc.npz")))["fullpulsecov"] * 3.0
    P, R, bxs, _ = oracle.synth_conditions(0)
    inp = oracle.synth_generate("ecal-1m-pu2", 0, 1500)
    s, pe = inp["samples"], inp["pederr"]
    cond = mf.make_conditions(P, R, bxs, fullpulsecov=fpc)
    first = oracle.fit_batch(s, pe, P, R, bxs, fullpulsecov=fpc, max_iter_nnls=1000, start=1, max_iter_outer=1)
    full = oracle.fit_batch(s, pe, P, R, bxs, fullpulsecov=fpc, max_iter_nnls=1000, start=1,
                            compute_errors=bool(errors))
    o = fit(lib, cond, s, pe, 1, 1000, errors, F_SEEDED, chunk=500, seed=first)
    for k in ["amplitudes", "chi2", "active_mask"] + (["errors"] if errors else []):
        assert np.array_equal(o[k], full[k], equal_nan=True), k
    outer = pack_iters(full["iters"]) & 0xFF
    assert np.array_equal(o["iters"] & 0xFF, outer)
    # the pulse covariance makes the loop iterate: most channels go on past the first iteration
    assert (outer > 2).mean() > 0.5


@pytest.mark.parametrize("max_outer", [0, 1, 2, 3])
def test_outer_iteration_caps_bit_for_bit(mf, oracle, lib, max_outer):
    """Minimize's iteration cap decides the kernel's passes (one lockstep pass
    for a cap of one or less, else the lockstep first iteration and the
    refilled rest): at every cap, with and without the error refits and a
    pulse covariance, the oracle's outputs (status bits included) bit for bit."""
    fpc = dict(np.load(os.path.join(GOLDEN, "fits_ecal_fpc.npz")))["fullpulsecov"] * 3.0
    P, R, bxs, _ = oracle.synth_conditions(0)
    inp = oracle.synth_generate("ecal-1m-pu2", 0, 1500)
    s, pe = inp["samples"], inp["pederr"]
    for F in (None, fpc):
        cond = mf.make_conditions(P, R, bxs, fullpulsecov=F)
        for errors in (0, 1):
            ref = oracle.fit_batch(s, pe, P, R, bxs, fullpulsecov=F, max_iter_nnls=10, start=0,
                                   compute_errors=bool(errors), max_iter_outer=max_outer)
            o = fit(lib, cond, s, pe, 0, 10, errors, chunk=300, max_iter_outer=max_outer)
            for k in ["amplitudes", "chi2", "active_mask", "status"] + (["errors"] if errors else []):
                assert np.array_equal(o[k], ref[k], equal_nan=True), (F is not None, errors, k)
            assert np.array_equal(o["iters"], pack_iters(ref["iters"]))
