"""Python host mirror of the GB300 multifit engine's C ABI.

The engine itself is ``_build/libmultifit_gb300.so`` (C++/CUDA, built by
``build.py``); this module binds its ``extern "C"`` entry points
(``include/multifit_gb300.h``) with ctypes and mirrors the reference's
per-channel interface, ``PulseChiSqSNNLS`` (multifit_cpu/interface/
PulseChiSqSNNLS.h:9-59), for tests and scripts. There is no Python or CPU
fallback: every fit runs the CUDA kernels, and loading fails loudly when the
library has not been built.

Import it by path (the directory name is not a Python identifier)::

    spec = importlib.util.spec_from_file_location(
        "multifit_gb300", "test-regression_gb300/__init__.py")
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "_build", "libmultifit_gb300.so")
# loaded by path under the name multifit_gb300: make it a package so that its
# submodules (rootio, ecal_data_io) import as multifit_gb300.<name>
__path__ = [PKG_DIR]

MAX_SAMPLES = 10
MAX_PULSES = 10
MAX_CTYPES = 2
FULLPULSE_MAX = MAX_SAMPLES + 9

# return codes
OK, EINVAL, ECUDA, ETIMEOUT, ENOMEM, EUNSUPPORTED, ENOTRAINED = range(7)
# channel status bits
CH_NNLS_MAXITER, CH_OUTER_MAXITER, CH_NONFINITE, CH_BADINPUT = 1, 2, 4, 8
# options
PREC_FP64, PREC_MIXED, PREC_FP32 = 0, 1, 2
SCHED_GRID, SCHED_PERSISTENT = 0, 1
WARM_NONE, WARM_MLP = 0, 1
START_REFERENCE, START_SUPPORT = 0, 1
SYNTH_ECAL, SYNTH_HCAL = 0, 1


class MfConditions(C.Structure):
    _fields_ = [
        ("nsamples", C.c_int32),
        ("npulses", C.c_int32),
        ("pulse_matrix", C.c_double * (MAX_SAMPLES * MAX_PULSES)),
        ("noise_cor", C.c_double * (MAX_SAMPLES * MAX_SAMPLES)),
        ("bxs", C.c_int8 * MAX_PULSES),
        ("has_fullpulsecov", C.c_int32),
        ("fullpulsecov", C.c_double * (FULLPULSE_MAX * FULLPULSE_MAX)),
    ]


class MfOptions(C.Structure):
    _fields_ = [
        ("max_iter_nnls", C.c_int32),
        ("max_iter_outer", C.c_int32),
        ("dchi2_tol", C.c_double),
        ("nnls_eps", C.c_double),
        ("nnls_start", C.c_int32),
        ("precision", C.c_int32),
        ("schedule", C.c_int32),
        ("warm_start", C.c_int32),
        ("compute_errors", C.c_int32),
        ("block_size", C.c_int32),
        ("blocks_per_sm", C.c_int32),
        ("channels_per_warp", C.c_int32),
    ]


class MfBatch(C.Structure):
    _fields_ = [
        ("n", C.c_int64),
        ("sample_stride", C.c_int32),
        ("amp_stride", C.c_int32),
        ("samples", C.c_void_p),
        ("pederr", C.c_void_p),
        ("ctype", C.c_void_p),
        ("amplitudes", C.c_void_p),
        ("chi2", C.c_void_p),
        ("intime", C.c_void_p),
        ("errors", C.c_void_p),
        ("active_mask", C.c_void_p),
        ("status", C.c_void_p),
        ("iters", C.c_void_p),
    ]


class MfTunePoint(C.Structure):
    _fields_ = [("block_size", C.c_int32), ("channels_per_warp", C.c_int32), ("ms", C.c_double)]


TUNE_POINTS = 20  # MF_TUNE_POINTS


class MfSynthParams(C.Structure):
    _fields_ = [
        ("n", C.c_int64),
        ("seed", C.c_uint64),
        ("intime_log", C.c_int32),
        ("intime_lo", C.c_double),
        ("intime_hi", C.c_double),
        ("pileup_mean", C.c_double),
        ("pileup_hit_mean", C.c_double),
        ("hcal_fraction", C.c_double),
    ]


class MfMlpTrainParams(C.Structure):
    _fields_ = [("epochs", C.c_int32), ("batch", C.c_int32), ("lr", C.c_float), ("amp_weight", C.c_float)]


# Exported symbols and their signatures: (name, restype, argtypes).
NOALLOC_MAX_CHANNELS = 131072  # MF_NOALLOC_MAX_CHANNELS
# mf_kernel_kind: the kernels mf_profile times
KERNEL_KINDS = ("fit_fp64_kernel", "mlp_infer_tc_kernel", "search_kernel", "judge_kernel", "repair_kernel",
                "partition_kernel", "judge_fixed_kernel", "fix_kernel", "screen_kernel")

SIGNATURES = [
    ("mf_abi_version", C.c_int, []),
    ("mf_rc_string", C.c_char_p, [C.c_int]),
    ("mf_last_error", C.c_char_p, []),
    ("mf_default_options", None, [C.POINTER(MfOptions)]),
    ("mf_create", C.c_int, [C.POINTER(C.c_void_p), C.c_int]),
    ("mf_destroy", None, [C.c_void_p]),
    ("mf_set_conditions", C.c_int, [C.c_void_p, C.c_int, C.POINTER(MfConditions)]),
    ("mf_fit", C.c_int, [C.c_void_p, C.POINTER(MfBatch), C.POINTER(MfOptions), C.c_void_p]),
    ("mf_fit_count_flops", C.c_int, [C.c_void_p, C.POINTER(MfBatch), C.POINTER(MfOptions), C.c_void_p, C.c_void_p]),
    ("mf_fit_host", C.c_int, [C.c_void_p, C.POINTER(MfBatch), C.POINTER(MfOptions)]),
    ("mf_fit_noalloc", C.c_int, [C.c_void_p, C.POINTER(MfBatch), C.POINTER(MfOptions), C.c_void_p]),
    ("mf_autotune", C.c_int, [C.c_void_p, C.POINTER(MfBatch), C.POINTER(MfOptions), C.c_void_p, C.c_int,
                              C.POINTER(C.c_int)]),
    ("mf_profile", C.c_int, [C.c_void_p, C.c_int]),
    ("mf_profile_read", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("mf_build_pulse_matrix", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]),
    ("mf_table_operator", C.c_int, [C.POINTER(MfConditions), C.c_uint32, C.c_void_p, C.c_void_p]),
    ("mf_mlp_param_count", C.c_int, []),
    ("mf_mlp_init", C.c_int, [C.c_void_p, C.c_int, C.c_uint64]),
    ("mf_mlp_train", C.c_int, [C.c_void_p, C.POINTER(MfBatch), C.POINTER(MfMlpTrainParams), C.c_void_p, C.c_void_p]),
    ("mf_mlp_gradient", C.c_int, [C.c_void_p, C.POINTER(MfBatch), C.POINTER(MfMlpTrainParams), C.c_void_p,
                                  C.c_void_p, C.c_void_p, C.c_void_p]),
    ("mf_mlp_get_weights", C.c_int, [C.c_void_p, C.c_void_p]),
    ("mf_mlp_set_weights", C.c_int, [C.c_void_p, C.c_void_p]),
    ("mf_mlp_predict", C.c_int, [C.c_void_p, C.POINTER(MfBatch), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("mf_mlp_test_stall", C.c_int, [C.c_void_p, C.c_int]),
    ("mf_synth_conditions", C.c_int, [C.c_int, C.POINTER(MfConditions), C.POINTER(C.c_double)]),
    ("mf_synth_generate", C.c_int, [C.POINTER(MfSynthParams), C.c_int64, C.c_int64, C.c_int, C.c_void_p,
                                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]),
]

_lib = None


class MultifitError(RuntimeError):
    pass


def load_library(path: str = LIB_PATH):
    """Loads the engine library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise MultifitError(
            f"{path} is missing: build the CUDA engine first (python test-regression_gb300/build.py)")
    lib = C.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _check(rc: int, what: str):
    if rc != OK:
        lib = load_library()
        raise MultifitError(f"{what}: {lib.mf_rc_string(rc).decode()} ({rc}) {lib.mf_last_error().decode()}")


def default_options(**kw) -> MfOptions:
    o = MfOptions()
    load_library().mf_default_options(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise KeyError(k)
        setattr(o, k, v)
    return o


def make_conditions(pulse_matrix, noise_cor, bxs, fullpulsecov=None) -> MfConditions:
    """pulse_matrix: (N, K); noise_cor: (N, N); bxs: (K,) ints."""
    P = np.asarray(pulse_matrix, dtype=np.float64)
    R = np.asarray(noise_cor, dtype=np.float64)
    N, K = P.shape
    c = MfConditions()
    c.nsamples, c.npulses = N, K
    flatP = np.ascontiguousarray(P.T).ravel()  # column-major
    flatR = np.ascontiguousarray(R.T).ravel()
    for i, v in enumerate(flatP):
        c.pulse_matrix[i] = float(v)
    for i, v in enumerate(flatR):
        c.noise_cor[i] = float(v)
    for k, b in enumerate(np.asarray(bxs, dtype=np.int64)):
        c.bxs[k] = int(b)
    if fullpulsecov is not None:
        F = np.asarray(fullpulsecov, dtype=np.float64)
        NF = N + 9
        if F.shape != (NF, NF):
            raise ValueError(f"fullpulsecov must be {NF}x{NF}")
        c.has_fullpulsecov = 1
        for i, v in enumerate(np.ascontiguousarray(F.T).ravel()):
            c.fullpulsecov[i] = float(v)
    return c


def conditions_arrays(c: MfConditions):
    """Returns (P (N,K), R (N,N), bxs (K,), fullpulsecov or None) of a condition set."""
    N, K = c.nsamples, c.npulses
    P = np.array(c.pulse_matrix[: N * K]).reshape(K, N).T.copy()
    R = np.array(c.noise_cor[: N * N]).reshape(N, N).T.copy()
    bxs = np.array(c.bxs[:K], dtype=np.int8)
    F = None
    if c.has_fullpulsecov:
        NF = N + 9
        F = np.array(c.fullpulsecov[: NF * NF]).reshape(NF, NF).T.copy()
    return P, R, bxs, F


def synth_conditions(kind: int):
    """(MfConditions, sigma) of a synthetic condition set (SYNTH_ECAL / SYNTH_HCAL)."""
    c = MfConditions()
    sigma = C.c_double()
    _check(load_library().mf_synth_conditions(kind, C.byref(c), C.byref(sigma)), "mf_synth_conditions")
    return c, sigma.value


def build_pulse_matrix(fullpulse, bxs, nsamples: int = 10) -> np.ndarray:
    """Reference sliding-window rule (multifit_cpu/src/PulseChiSqSNNLS.cpp:49-62); returns (N, K)."""
    fp = np.ascontiguousarray(fullpulse, dtype=np.float64)
    bx = np.ascontiguousarray(bxs, dtype=np.int8)
    K = bx.shape[0]
    out = np.zeros(nsamples * K, dtype=np.float64)
    _check(load_library().mf_build_pulse_matrix(fp.ctypes.data, bx.ctypes.data, nsamples, K, out.ctypes.data),
           "mf_build_pulse_matrix")
    return out.reshape(K, nsamples).T.copy()


def table_operator(cond: MfConditions, mask: int):
    """(L_R^-1 (N,N), pseudo-inverse (p,N)) of the mixed-form tables (host computation)."""
    N = cond.nsamples
    p = bin(mask).count("1")
    W = np.zeros(N * N)
    P = np.zeros(p * N)
    _check(load_library().mf_table_operator(C.byref(cond), mask, W.ctypes.data, P.ctypes.data),
           "mf_table_operator")
    return W.reshape(N, N), P.reshape(p, N)


# Workloads of the benchmark configurations: (n, synth params).
def synth_params(seed: int, n: int, intime_log: bool = False, lo: float = 1.0, hi: float = 100.0,
                 pileup_mean: float = 0.5, hit_mean: float = 1.0, hcal_fraction: float = 0.0) -> MfSynthParams:
    p = MfSynthParams()
    p.n, p.seed, p.intime_log = n, seed, int(intime_log)
    p.intime_lo, p.intime_hi = lo, hi
    p.pileup_mean, p.pileup_hit_mean, p.hcal_fraction = pileup_mean, hit_mean, hcal_fraction
    return p


WORKLOADS = {
    # 10,000 ECAL channels, in-time U[1,100], pileup Poisson(0.5) x Exp(1) per out-of-time BX, seed 1
    "ecal-10k-pu0.5": lambda: synth_params(1, 10_000, pileup_mean=0.5),
    # 1,000,000 ECAL channels, pileup mean 2, seed 2
    "ecal-1m-pu2": lambda: synth_params(2, 1_000_000, pileup_mean=2.0),
    # 10,000,000 ECAL channels, in-time log-uniform [0.1,1000], pileup 4, seed 3
    "ecal-10m-logamp-pu4": lambda: synth_params(3, 10_000_000, intime_log=True, lo=0.1, hi=1000.0, pileup_mean=4.0),
    # 10,000,000 channels, 40% HCAL 8x8, pileup mean per channel U[0,8], seed 4
    "mixed-10m-ecal-hcal": lambda: synth_params(4, 10_000_000, pileup_mean=-8.0, hcal_fraction=0.4),
    # MLP training set (5,000,000, log-uniform, pileup 4, seed 5) and evaluation set (10,000,000, seed 6)
    "warm-train-5m": lambda: synth_params(5, 5_000_000, intime_log=True, lo=0.1, hi=1000.0, pileup_mean=4.0),
    "warm-eval-10m": lambda: synth_params(6, 10_000_000, intime_log=True, lo=0.1, hi=1000.0, pileup_mean=4.0),
}


def synth_generate_host(p: MfSynthParams, first: int, count: int, stride: int = 10, with_truth: bool = True):
    """Host-side generation: returns dict of numpy arrays."""
    lib = load_library()
    samples = np.zeros((count, stride), dtype=np.float64)
    pederr = np.zeros(count, dtype=np.float64)
    ctype = np.zeros(count, dtype=np.uint8)
    truth = np.zeros((count, MAX_PULSES), dtype=np.float64) if with_truth else None
    _check(lib.mf_synth_generate(C.byref(p), first, count, stride, samples.ctypes.data, pederr.ctypes.data,
                                 ctype.ctypes.data, truth.ctypes.data if with_truth else None, MAX_PULSES, 0, None),
           "mf_synth_generate(host)")
    return {"samples": samples, "pederr": pederr, "ctype": ctype, "truth": truth}


def synth_generate_device(p: MfSynthParams, first: int, count: int, samples_ptr: int, pederr_ptr: int,
                          ctype_ptr: int | None, stride: int = 10, truth_ptr: int | None = None,
                          stream: int | None = None):
    _check(load_library().mf_synth_generate(C.byref(p), first, count, stride, samples_ptr, pederr_ptr, ctype_ptr,
                                            truth_ptr, MAX_PULSES, 1, stream), "mf_synth_generate(device)")


class Engine:
    """A context of the engine bound to one CUDA device (mf_create / mf_destroy)."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = C.c_void_p()
        _check(self.lib.mf_create(C.byref(h), device), "mf_create")
        self.h = h
        self.conditions: dict[int, MfConditions] = {}

    def close(self):
        if self.h:
            self.lib.mf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_conditions(self, ctype: int, cond: MfConditions):
        _check(self.lib.mf_set_conditions(self.h, ctype, C.byref(cond)), "mf_set_conditions")
        self.conditions[ctype] = cond

    @staticmethod
    def _batch(n, sample_stride, amp_stride, samples, pederr, ctype, amplitudes, chi2, intime=None, errors=None,
               active_mask=None, status=None, iters=None) -> MfBatch:
        b = MfBatch()
        b.n, b.sample_stride, b.amp_stride = n, sample_stride, amp_stride
        b.samples, b.pederr, b.ctype = samples, pederr, ctype
        b.amplitudes, b.chi2, b.intime, b.errors = amplitudes, chi2, intime, errors
        b.active_mask, b.status, b.iters = active_mask, status, iters
        return b

    def fit_device(self, batch: MfBatch, options: MfOptions | None = None, stream: int | None = None):
        """mf_fit on device pointers (asynchronous on `stream`)."""
        _check(self.lib.mf_fit(self.h, C.byref(batch), C.byref(options or default_options()), stream), "mf_fit")

    def fit_noalloc(self, batch: MfBatch, options: MfOptions, stream: int | None = None) -> int:
        """mf_fit_noalloc on device pointers; returns the return code (the
        caller checks it: oversize batches are an expected MF_EINVAL)."""
        return int(self.lib.mf_fit_noalloc(self.h, C.byref(batch), C.byref(options), stream))

    def autotune(self, batch: MfBatch, options: MfOptions) -> list:
        """mf_autotune: sweep of the persistent schedule's launch shape on this
        device batch; returns [(block_size, channels_per_warp, ms)], the
        fastest being kept by the context."""
        pts = (MfTunePoint * TUNE_POINTS)()
        n = C.c_int(0)
        _check(self.lib.mf_autotune(self.h, C.byref(batch), C.byref(options), pts, TUNE_POINTS, C.byref(n)),
               "mf_autotune")
        return [(p.block_size, p.channels_per_warp, p.ms) for p in pts[: n.value]]

    def profile(self, enable: bool = True):
        """mf_profile: start (or stop) per-kernel launch timing of fits."""
        _check(self.lib.mf_profile(self.h, int(enable)), "mf_profile")

    def profile_read(self) -> dict:
        """mf_profile_read: {kernel: (launches, total device ms)} of the fits
        recorded since the last read (waits for them)."""
        n = len(KERNEL_KINDS)
        launches = (C.c_int32 * n)()
        ms = (C.c_double * n)()
        _check(self.lib.mf_profile_read(self.h, launches, ms), "mf_profile_read")
        return {k: (int(launches[i]), float(ms[i])) for i, k in enumerate(KERNEL_KINDS) if launches[i]}

    def fit_count_flops(self, batch: MfBatch, flops_ptr: int, options: MfOptions | None = None,
                        stream: int | None = None):
        _check(self.lib.mf_fit_count_flops(self.h, C.byref(batch), C.byref(options or default_options()),
                                           flops_ptr, stream), "mf_fit_count_flops")

    def fit_host(self, samples: np.ndarray, pederr: np.ndarray, ctype: np.ndarray | None = None,
                 options: MfOptions | None = None, amp_stride: int = MAX_PULSES):
        """mf_fit_host on numpy arrays; returns a dict of numpy outputs."""
        samples = np.ascontiguousarray(samples, dtype=np.float64)
        pederr = np.ascontiguousarray(pederr, dtype=np.float64)
        n, stride = samples.shape
        out = {
            "amplitudes": np.zeros((n, amp_stride), dtype=np.float64),
            "chi2": np.zeros(n, dtype=np.float64),
            "intime": np.zeros(n, dtype=np.float64),
            "errors": np.zeros(n, dtype=np.float64),
            "active_mask": np.zeros(n, dtype=np.uint16),
            "status": np.zeros(n, dtype=np.uint8),
            "iters": np.zeros(n, dtype=np.int32),
        }
        ct = None
        if ctype is not None:
            ctype = np.ascontiguousarray(ctype, dtype=np.uint8)
            ct = ctype.ctypes.data
        b = self._batch(n, stride, amp_stride, samples.ctypes.data, pederr.ctypes.data, ct,
                        out["amplitudes"].ctypes.data, out["chi2"].ctypes.data, out["intime"].ctypes.data,
                        out["errors"].ctypes.data, out["active_mask"].ctypes.data, out["status"].ctypes.data,
                        out["iters"].ctypes.data)
        _check(self.lib.mf_fit_host(self.h, C.byref(b), C.byref(options or default_options())), "mf_fit_host")
        return out


def mlp_params(epochs=3, batch=8192, lr=2e-3, amp_weight=1.0) -> MfMlpTrainParams:
    p = MfMlpTrainParams()
    p.epochs, p.batch, p.lr, p.amp_weight = epochs, batch, lr, amp_weight
    return p


# Flat parameter layout of the MLP: (name, shape) in order.
MLP_LAYOUT = [("W1", (128, 16)), ("b1", (128,)), ("W2", (128, 128)), ("b2", (128,)), ("W3", (32, 128)),
              ("b3", (32,))]


def mlp_unflatten(flat: np.ndarray) -> dict:
    out, o = {}, 0
    for name, shape in MLP_LAYOUT:
        size = int(np.prod(shape))
        out[name] = flat[o:o + size].reshape(shape)
        o += size
    return out


def _mlp_engine_methods():
    def mlp_init(self, ctype=0, seed=1):
        _check(self.lib.mf_mlp_init(self.h, ctype, seed), "mf_mlp_init")

    def mlp_train(self, batch: MfBatch, params: MfMlpTrainParams, stream=None):
        losses = np.zeros(max(params.epochs, 1), dtype=np.float32)
        _check(self.lib.mf_mlp_train(self.h, C.byref(batch), C.byref(params), losses.ctypes.data, stream),
               "mf_mlp_train")
        return losses[: params.epochs]

    def mlp_gradient(self, batch: MfBatch, params: MfMlpTrainParams):
        n = self.lib.mf_mlp_param_count()
        B = params.batch
        g = np.zeros(n, dtype=np.float32)
        f = np.zeros((B, 16), dtype=np.uint16)
        t = np.zeros((B, 20), dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        _check(self.lib.mf_mlp_gradient(self.h, C.byref(batch), C.byref(params), g.ctypes.data, f.ctypes.data,
                                        t.ctypes.data, loss.ctypes.data), "mf_mlp_gradient")
        feats = (f.astype(np.uint32) << 16).view(np.float32)
        return g, feats, t, float(loss[0])

    def mlp_get_weights(self):
        w = np.zeros(self.lib.mf_mlp_param_count(), dtype=np.float32)
        _check(self.lib.mf_mlp_get_weights(self.h, w.ctypes.data), "mf_mlp_get_weights")
        return w

    def mlp_set_weights(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        _check(self.lib.mf_mlp_set_weights(self.h, w.ctypes.data), "mf_mlp_set_weights")

    def mlp_test_stall(self, enable: bool):
        """Test hook: inference waits give up after 1 ms (mf_mlp_test_stall)."""
        _check(self.lib.mf_mlp_test_stall(self.h, 1 if enable else 0), "mf_mlp_test_stall")

    def mlp_predict(self, batch: MfBatch, mask_ptr, amp_ptr, logits_ptr=None, stream=None):
        _check(self.lib.mf_mlp_predict(self.h, C.byref(batch), mask_ptr, amp_ptr, logits_ptr, stream),
               "mf_mlp_predict")

    return dict(mlp_init=mlp_init, mlp_train=mlp_train, mlp_gradient=mlp_gradient, mlp_get_weights=mlp_get_weights,
                mlp_set_weights=mlp_set_weights, mlp_test_stall=mlp_test_stall, mlp_predict=mlp_predict)


for _k, _v in _mlp_engine_methods().items():
    setattr(Engine, _k, _v)


def save_mlp_weights(path: str, flat: np.ndarray, meta: dict | None = None):
    """Checkpoint: a JSON header line then the little-endian float32 parameters."""
    import json

    hdr = {"format": "multifit-gb300-mlp", "version": 1, "layout": MLP_LAYOUT, "count": int(flat.size)}
    hdr.update(meta or {})
    with open(path, "wb") as f:
        f.write((json.dumps(hdr) + "\n").encode())
        f.write(np.ascontiguousarray(flat, dtype="<f4").tobytes())


def load_mlp_weights(path: str):
    import json

    with open(path, "rb") as f:
        hdr = json.loads(f.readline().decode())
        flat = np.frombuffer(f.read(), dtype="<f4").copy()
    if hdr.get("format") != "multifit-gb300-mlp" or flat.size != hdr["count"]:
        raise ValueError(f"{path}: not an MLP checkpoint")
    return flat, hdr


def unpack_iters(iters: np.ndarray):
    it = iters.astype(np.int64)
    return it & 0xFF, (it >> 8) & 0xFFF, (it >> 20) & 0xFFF


class PulseChiSqSNNLS:
    """Mirror of the reference's per-channel fit object
    (multifit_cpu/interface/PulseChiSqSNNLS.h:9-59): DoFit, then X(), ChiSq(),
    BXs(), Errors(). Each DoFit is one mf_fit_host call with n=1 on the GPU."""

    _engine: Engine | None = None

    def __init__(self, engine: Engine | None = None):
        self.engine = engine
        self._compute_errors = True
        self._x = None
        self._chisq = 0.0
        self._bxs = None
        self._err = None
        self._status = 0

    def disableErrorCalculation(self):
        self._compute_errors = False

    def DoFit(self, samples, samplecor, pederr, bxs, fullpulse, fullpulsecov) -> bool:
        if self.engine is None:
            if PulseChiSqSNNLS._engine is None:
                PulseChiSqSNNLS._engine = Engine(0)
            self.engine = PulseChiSqSNNLS._engine
        samples = np.asarray(samples, dtype=np.float64)
        N = samples.shape[0]
        bxs = np.asarray(bxs, dtype=np.int8)
        P = build_pulse_matrix(fullpulse, bxs, N)
        fpc = np.asarray(fullpulsecov, dtype=np.float64)
        cond = make_conditions(P, samplecor, bxs, fpc if np.any(fpc != 0) else None)
        self.engine.set_conditions(0, cond)
        out = self.engine.fit_host(samples.reshape(1, N), np.array([pederr]),
                                   options=default_options(compute_errors=int(self._compute_errors)))
        K = bxs.shape[0]
        self._x = out["amplitudes"][0, :K].copy()
        self._chisq = float(out["chi2"][0])
        self._bxs = bxs.copy()
        self._err = np.zeros(K)
        kin = np.nonzero(bxs == 0)[0]
        if self._compute_errors and kin.size:
            self._err[kin[0]] = out["errors"][0]
        self._status = int(out["status"][0])
        return True

    def X(self):
        return self._x

    def ChiSq(self):
        return self._chisq

    def BXs(self):
        return self._bxs

    def Errors(self):
        return self._err

    def Status(self):
        return self._status
