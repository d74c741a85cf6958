"""CPU oracle of the multifit hot path -- TEST INFRASTRUCTURE ONLY.

ctypes bindings of ``_build/liboracle.so`` (multifit_oracle.cpp: the C++17
FP64 restatement of the reference's multifit_cpu fit) and of
``_ref/libref_linalgebra.so`` (the reference's own linear-algebra headers,
compiled in place where the reference tree exists). Only the tests, the smoke
check and the benchmark's CPU-baseline leg use this package, always as the
checker or the timed CPU baseline -- never on the engine's path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build_oracle

_lib = None
_lib_sep = None
_ref = None
_ref_ocl = {}

KMAX = 10

dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def _bind(L):
    L.oracle_cholesky.argtypes = [dp, dp, C.c_int, C.c_int]
    L.oracle_forward.argtypes = [dp, C.c_int, dp, dp, C.c_int]
    L.oracle_backward.argtypes = [dp, C.c_int, dp, dp, C.c_int]
    L.oracle_rc_addition.argtypes = [dp, dp, C.c_int, dp, dp, C.c_int]
    L.oracle_inbetween_removal.argtypes = [dp, dp, C.c_int, dp, dp, C.c_int, C.c_int]
    L.oracle_swap_sym.argtypes = [dp, C.c_int, C.c_int, C.c_int, C.c_int]
    L.oracle_inplace_fnnls.argtypes = [dp, dp, dp, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int,
                                       np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")]
    L.oracle_fit_batch.restype = C.c_int
    L.oracle_fit_batch.argtypes = [C.c_int64, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                                   C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int,
                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_void_p]
    L.oracle_kkt_violation.restype = C.c_double
    L.oracle_kkt_violation.argtypes = [dp, dp, dp, C.c_int, C.c_int]
    L.oracle_nnls_bruteforce.restype = C.c_double
    L.oracle_nnls_bruteforce.argtypes = [dp, dp, C.c_int, C.c_int, dp]
    L.oracle_nnls_lawson_hanson.restype = C.c_int
    L.oracle_nnls_lawson_hanson.argtypes = [dp, dp, C.c_int, C.c_int, dp, C.c_int]
    L.oracle_hardware_threads.restype = C.c_int
    L.oracle_synth_conditions.restype = C.c_int
    L.oracle_synth_conditions.argtypes = [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.POINTER(C.c_double)]
    L.oracle_synth_generate.restype = C.c_int
    L.oracle_synth_generate.argtypes = [C.c_uint64, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                        C.c_double, C.c_int64, C.c_int64, C.c_int, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_int, C.c_int]
    return L


def lib():
    global _lib
    if _lib is None:
        _lib = _bind(C.CDLL(build_oracle.build_oracle()))
    return _lib


def lib_separate():
    """The oracle built with each product and sum of its FMA expressions
    rounded separately (the build compared with the reference's plain-C FNNLS)."""
    global _lib_sep
    if _lib_sep is None:
        _lib_sep = _bind(C.CDLL(build_oracle.build_oracle_separate()))
    return _lib_sep


def ref_ocl(bits: int = 64):
    """The reference's OpenCL FNNLS (multifit_ocl/device/regression_inplace_fnnls.cl)
    compiled as C, FP64 (bits=64) or as written in FP32 (bits=32); None where
    the reference tree is absent."""
    if bits not in _ref_ocl:
        paths = build_oracle.build_ref_ocl()
        if paths is None:
            return None
        for b, path in paths.items():
            L = C.CDLL(path)
            L.ref_ocl_inplace_fnnls.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_uint]
            L.ref_ocl_data_type_bytes.restype = C.c_int
            _ref_ocl[b] = L
    return _ref_ocl[bits]


def ref_ocl_inplace_fnnls(A: np.ndarray, b: np.ndarray, x0: np.ndarray | None = None, eps: float = 1e-11,
                          max_iter: int = 1000, bits: int = 64) -> np.ndarray:
    """The reference's OpenCL FNNLS on one 10x10 problem (warm x0 as its
    final_s starts from x); returns x in the kernel's data type."""
    L = ref_ocl(bits)
    if L is None:
        raise RuntimeError("the reference tree is needed for the OpenCL FNNLS")
    dt = np.float64 if bits == 64 else np.float32
    A = np.ascontiguousarray(A, dtype=dt)  # row-major, as the kernel indexes it
    if A.shape != (10, 10):
        raise ValueError("the OpenCL kernel is fixed at 10 x 10")
    bb = np.ascontiguousarray(b, dtype=dt).copy()
    x = np.zeros(10, dtype=dt) if x0 is None else np.ascontiguousarray(x0, dtype=dt).copy()
    L.ref_ocl_inplace_fnnls(A.ctypes.data, bb.ctypes.data, x.ctypes.data, eps, max_iter)
    return x


_ref_dofit = None


def ref_dofit_lib():
    """The reference's multifit_cpu fit (PulseChiSqSNNLS.cpp + inplace_fnnls.cu
    over the Eigen shim), or None where the reference tree is absent."""
    global _ref_dofit
    if _ref_dofit is None:
        path = build_oracle.build_ref_dofit()
        if path is None:
            return None
        L = C.CDLL(path)
        L.ref_dofit_batch.restype = C.c_int
        L.ref_dofit_batch.argtypes = [C.c_long, C.c_int] + [C.c_void_p] * 6 + [C.c_int] + [C.c_void_p] * 4
        _ref_dofit = L
    return _ref_dofit


def fullpulse_of(P: np.ndarray, bxs) -> np.ndarray:
    """The 19-sample fullpulse that the reference's sliding-window rule
    (multifit_cpu/src/PulseChiSqSNNLS.cpp:49-62) turns into the 10 x K pulse
    matrix P; raises if P is not of that form."""
    P = np.asarray(P, dtype=np.float64)
    fp = np.zeros(19)
    seen = np.zeros(19, dtype=bool)
    for k, bx in enumerate(np.asarray(bxs, dtype=np.int64)):
        first = max(0, int(bx) + 3)
        for i in range(P.shape[0]):
            if i < first:
                if P[i, k] != 0:
                    raise ValueError("P is not a sliding window of one fullpulse")
                continue
            j = i + 4 - int(bx)
            if not 0 <= j < 19 or (seen[j] and fp[j] != P[i, k]):
                raise ValueError("P is not a sliding window of one fullpulse")
            fp[j], seen[j] = P[i, k], True
    return fp


def ref_dofit(samples, pederr, R, bxs, fullpulse, fullpulsecov=None, compute_errors: bool = False) -> dict:
    """The reference's own PulseChiSqSNNLS::DoFit on each channel (N = 10):
    X(), ChiSq(), the in-time Errors() entry and DoFit's return value."""
    L = ref_dofit_lib()
    if L is None:
        raise RuntimeError("the reference tree is needed for the reference DoFit")
    s = np.ascontiguousarray(samples, dtype=np.float64)
    n = s.shape[0]
    if s.shape[1] != 10:
        raise ValueError("the reference fit is fixed at 10 samples")
    bx = np.ascontiguousarray(bxs, dtype=np.int8)
    K = bx.shape[0]
    Rcm = np.ascontiguousarray(np.asarray(R, dtype=np.float64).T)
    fp = np.ascontiguousarray(fullpulse, dtype=np.float64)
    F = None if fullpulsecov is None else np.ascontiguousarray(np.asarray(fullpulsecov, dtype=np.float64).T)
    pe = np.ascontiguousarray(pederr, dtype=np.float64)
    out = {"amplitudes": np.zeros((n, K)), "chi2": np.zeros(n), "errors": np.zeros(n), "ok": np.zeros(n, np.int32)}
    rc = L.ref_dofit_batch(n, K, s.ctypes.data, Rcm.ctypes.data, pe.ctypes.data, bx.ctypes.data, fp.ctypes.data,
                           F.ctypes.data if F is not None else None, int(compute_errors), out["amplitudes"].ctypes.data,
                           out["chi2"].ctypes.data, out["errors"].ctypes.data, out["ok"].ctypes.data)
    if rc:
        raise ValueError(f"ref_dofit_batch rc={rc}")
    return out


def ref():
    """The reference's own linalgebra primitives, or None where the reference tree is absent."""
    global _ref
    if _ref is None:
        path = build_oracle.build_ref()
        if path is None:
            return None
        R = C.CDLL(path)
        R.ref_cholesky_decomp.argtypes = [dp, dp, C.c_int, C.c_int]
        R.ref_forward.argtypes = [dp, dp, dp, C.c_int, C.c_int]
        R.ref_backward.argtypes = [dp, dp, dp, C.c_int, C.c_int]
        R.ref_rc_addition.argtypes = [dp, dp, dp, dp, C.c_int, C.c_int]
        R.ref_inbetween_removal.argtypes = [dp, dp, dp, dp, C.c_int, C.c_int, C.c_int]
        R.ref_eigen_rc_addition.argtypes = [dp, dp, dp, dp, C.c_int, C.c_int]
        R.ref_eigen_inbetween_removal.argtypes = [dp, dp, dp, dp, C.c_int, C.c_int, C.c_int]
        R.ref_swap_row_column.argtypes = [dp, C.c_int, C.c_int, C.c_int, C.c_int]
        _ref = R
    return _ref


def hardware_threads() -> int:
    return int(lib().oracle_hardware_threads())


def inplace_fnnls(A: np.ndarray, b: np.ndarray, x0: np.ndarray | None = None, eps: float = 1e-11,
                  max_iter: int = 1000, variant: int = 0, start: int = 0, separate_rounding: bool = False):
    """FNNLS on a whitened problem. A: (N, K). Returns (x, stats dict).
    separate_rounding: use the build that rounds each product and sum."""
    A = np.asarray(A, dtype=np.float64)
    N, K = A.shape
    Acm = np.ascontiguousarray(A.T)  # column-major flat
    x = np.zeros(K) if x0 is None else np.array(x0, dtype=np.float64)
    st = np.zeros(5, dtype=np.int32)
    (lib_separate() if separate_rounding else lib()).oracle_inplace_fnnls(
        Acm.ravel(), np.ascontiguousarray(b, dtype=np.float64), x, N, K, eps, max_iter, variant, start, st)
    return x, {"outer": int(st[0]), "inner": int(st[1]), "converged": int(st[2]), "passive": int(st[3]),
               "mask": int(st[4])}


def fit_batch(samples: np.ndarray, pederr: np.ndarray, P: np.ndarray, R: np.ndarray, bxs=None,
              fullpulsecov=None, eps: float = 1e-11, max_iter_nnls: int = 10, max_iter_outer: int = 50,
              dchi2_tol: float = 1e-3, variant: int = 1, start: int = 0, compute_errors: bool = False,
              nthreads: int = 0, count_flops: bool = False):
    """Fits channels sharing one condition set. samples: (n, stride). P: (N, K), R: (N, N)."""
    samples = np.ascontiguousarray(samples, dtype=np.float64)
    pederr = np.ascontiguousarray(pederr, dtype=np.float64)
    n, stride = samples.shape
    P = np.asarray(P, dtype=np.float64)
    N, K = P.shape
    Pcm = np.ascontiguousarray(P.T)
    Rcm = np.ascontiguousarray(np.asarray(R, dtype=np.float64).T)
    if bxs is None:
        bxs = np.arange(K, dtype=np.int8) - 5
    bx = np.ascontiguousarray(bxs, dtype=np.int8)
    F = None
    if fullpulsecov is not None:
        F = np.ascontiguousarray(np.asarray(fullpulsecov, dtype=np.float64).T)
    out = {
        "amplitudes": np.zeros((n, K)),
        "chi2": np.zeros(n),
        "active_mask": np.zeros(n, dtype=np.uint16),
        "status": np.zeros(n, dtype=np.uint8),
        "iters": np.zeros((n, 3), dtype=np.int32),
        "errors": np.zeros(n),
        "flops": np.zeros(n) if count_flops else None,
    }
    rc = lib().oracle_fit_batch(
        n, N, K, samples.ctypes.data, stride, pederr.ctypes.data, Pcm.ctypes.data, Rcm.ctypes.data,
        F.ctypes.data if F is not None else None, bx.ctypes.data, eps, max_iter_nnls, max_iter_outer,
        dchi2_tol, variant, start, int(compute_errors), nthreads, out["amplitudes"].ctypes.data, out["chi2"].ctypes.data,
        out["active_mask"].ctypes.data, out["status"].ctypes.data, out["iters"].ctypes.data,
        out["errors"].ctypes.data, out["flops"].ctypes.data if count_flops else None)
    if rc != 0:
        raise ValueError(f"oracle_fit_batch rc={rc}")
    return out


# Seeded synthetic workloads (the benchmark configurations): seed, channels,
# in-time amplitude law and range, pileup mean per out-of-time BX (negative:
# drawn per channel uniform in [0, -mean]), hit energy mean, HCAL fraction.
SYNTH_ECAL, SYNTH_HCAL = 0, 1
WORKLOADS = {
    "ecal-10k-pu0.5": dict(seed=1, n=10_000, intime_log=False, lo=1.0, hi=100.0, pileup_mean=0.5),
    "ecal-1m-pu2": dict(seed=2, n=1_000_000, intime_log=False, lo=1.0, hi=100.0, pileup_mean=2.0),
    "ecal-10m-logamp-pu4": dict(seed=3, n=10_000_000, intime_log=True, lo=0.1, hi=1000.0, pileup_mean=4.0),
    "mixed-10m-ecal-hcal": dict(seed=4, n=10_000_000, intime_log=False, lo=1.0, hi=100.0, pileup_mean=-8.0,
                                hcal_fraction=0.4),
    "warm-train-5m": dict(seed=5, n=5_000_000, intime_log=True, lo=0.1, hi=1000.0, pileup_mean=4.0),
    "warm-eval-10m": dict(seed=6, n=10_000_000, intime_log=True, lo=0.1, hi=1000.0, pileup_mean=4.0),
}


def synth_conditions(kind: int):
    """(P (N,K), R (N,N), bxs (K,), sigma) of a synthetic condition set: the
    ECAL 10x10 set as the reference driver builds it, or the HCAL 8x8 set."""
    N, K = C.c_int(), C.c_int()
    P = np.zeros(KMAX * KMAX)
    R = np.zeros(KMAX * KMAX)
    bx = np.zeros(KMAX, dtype=np.int8)
    sg = C.c_double()
    if lib().oracle_synth_conditions(kind, C.byref(N), C.byref(K), P.ctypes.data, R.ctypes.data, bx.ctypes.data,
                                     C.byref(sg)):
        raise ValueError(f"unknown synthetic condition set {kind}")
    n, k = N.value, K.value
    return (P[: n * k].reshape(k, n).T.copy(), R[: n * n].reshape(n, n).T.copy(), bx[:k].copy(), sg.value)


def synth_generate(workload, first: int, count: int, stride: int = 10, with_truth: bool = False,
                   nthreads: int = 0) -> dict:
    """Channels [first, first + count) of a seeded workload (a WORKLOADS name
    or a dict of its parameters) on the host cores: samples, pederr, ctype and
    optionally the true amplitudes."""
    w = dict(WORKLOADS[workload]) if isinstance(workload, str) else dict(workload)
    hit_mean = w.get("hit_mean", 1.0)
    hcal = w.get("hcal_fraction", 0.0)
    samples = np.zeros((count, stride))
    pederr = np.zeros(count)
    ctype = np.zeros(count, dtype=np.uint8)
    truth = np.zeros((count, KMAX)) if with_truth else None
    rc = lib().oracle_synth_generate(int(w["seed"]), int(w["intime_log"]), float(w["lo"]), float(w["hi"]),
                                     float(w["pileup_mean"]), float(hit_mean), float(hcal), first, count, stride,
                                     samples.ctypes.data, pederr.ctypes.data, ctype.ctypes.data,
                                     truth.ctypes.data if with_truth else None, KMAX, nthreads)
    if rc:
        raise ValueError("oracle_synth_generate: bad arguments")
    return {"samples": samples, "pederr": pederr, "ctype": ctype, "truth": truth}


def kkt_violation(A, b, x) -> float:
    A = np.asarray(A, dtype=np.float64)
    N, K = A.shape
    return float(lib().oracle_kkt_violation(np.ascontiguousarray(A.T).ravel(), np.ascontiguousarray(b, float),
                                            np.ascontiguousarray(x, float), N, K))


def nnls_bruteforce(A, b):
    A = np.asarray(A, dtype=np.float64)
    N, K = A.shape
    x = np.zeros(K)
    r = lib().oracle_nnls_bruteforce(np.ascontiguousarray(A.T).ravel(), np.ascontiguousarray(b, float), N, K, x)
    return x, float(r)


def nnls_lawson_hanson(A, b, max_iter: int = 100):
    A = np.asarray(A, dtype=np.float64)
    N, K = A.shape
    x = np.zeros(K)
    lib().oracle_nnls_lawson_hanson(np.ascontiguousarray(A.T).ravel(), np.ascontiguousarray(b, float), N, K, x,
                                    max_iter)
    return x


def whiten(P, R, pederr, samples):
    """A = L^-1 P, b = L^-1 s with L = chol(pederr^2 R) (numpy, for cross-checks)."""
    Lc = np.linalg.cholesky(pederr * pederr * np.asarray(R))
    import scipy.linalg as sl
    A = sl.solve_triangular(Lc, P, lower=True)
    b = sl.solve_triangular(Lc, samples, lower=True)
    return A, b
