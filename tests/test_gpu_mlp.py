"""Learned warm start on the GPU: the hand-written MLP kernels against the
CPU FP64 checker (oracle/mlp_oracle.py), training, and the warm fit against
the FP64 oracle.

Tolerances: gradients of the BF16/FP32 kernels vs the FP64 checker with the
same BF16 rounding points -- normwise relative error <= 2e-2 per parameter
tensor (FP32 accumulation order and rare BF16 tie flips), cosine >= 0.999;
against the exact FP64 gradient, cosine >= 0.99. The warm fit obeys the
mixed form's bounds (<= 1e-4 normwise relative amplitude error and identical
active sets on >= 99.9 % of channels vs the FP64 oracle at KKT convergence).
"""
import numpy as np
import pytest

from _helpers import DeviceBatch, oracle_fit_sets
from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu


def train_set(mf, cuda, eng, n, seed):
    """Channels of the log-uniform pileup-4 generator plus their converged FP64 fits (the targets)."""
    db = DeviceBatch(mf, cuda, n)
    db.generate(mf, mf.synth_params(seed, n, intime_log=True, lo=0.1, hi=1000.0, pileup_mean=4.0))
    eng.fit_device(db.batch, mf.default_options(max_iter_nnls=1000, nnls_start=mf.START_SUPPORT))
    cuda.cuda.synchronize()
    return db


@pytest.fixture(scope="module")
def mlp_engine(mf, cuda):
    eng = mf.Engine(0)
    eng.set_conditions(0, mf.synth_conditions(mf.SYNTH_ECAL)[0])
    eng.mlp_init(0, seed=7)
    yield eng
    eng.close()


def test_gradients_match_cpu_fp64(mf, cuda, mlp_engine):
    eng = mlp_engine
    B = 4096
    db = train_set(mf, cuda, eng, B, seed=31)
    p = mf.mlp_params(epochs=1, batch=B, amp_weight=1.0)
    g, X, T, loss = eng.mlp_gradient(db.batch, p)
    params = mo.unflatten(eng.mlp_get_weights())
    X = X.astype(np.float64)
    T = T.astype(np.float64)
    # features: 10 unit-normalised whitened samples, log SNR, pederr
    assert np.allclose(np.linalg.norm(X[:, :10], axis=1), 1.0, atol=2e-2)
    assert (X[:, 12:] == 0).all()
    lq, gq = mo.loss_and_grad(params, X, T, 1.0, quantized=True)
    le, ge = mo.loss_and_grad(params, X, T, 1.0, quantized=False)
    assert abs(loss - lq) <= 1e-4 * abs(lq)
    gg = mo.unflatten(g)
    for name, _ in mo.LAYOUT:
        a, r, ex = gg[name].ravel(), gq[name].ravel(), ge[name].ravel()
        if name in ("W3", "b3"):
            a, r, ex = gg[name][:20].ravel(), gq[name][:20].ravel(), ge[name][:20].ravel()
            assert (gg[name][20:] == 0).all()
        rel = np.linalg.norm(a - r) / np.linalg.norm(r)
        cos = a @ r / (np.linalg.norm(a) * np.linalg.norm(r))
        cos_exact = a @ ex / (np.linalg.norm(a) * np.linalg.norm(ex))
        assert rel <= 2e-2, (name, rel)
        assert cos >= 0.999, (name, cos)
        assert cos_exact >= 0.99, (name, cos_exact)


def test_training_reduces_loss_and_warm_fit_parity(mf, oracle, cuda, mlp_engine):
    eng = mlp_engine
    n = 262_144
    db = train_set(mf, cuda, eng, n, seed=5)
    losses = eng.mlp_train(db.batch, mf.mlp_params(epochs=4, batch=4096, lr=2e-3))
    assert np.isfinite(losses).all()
    assert losses[-1] < 0.85 * losses[0] and (np.diff(losses) < 0).all(), losses
    # fresh evaluation channels (seed 6)
    m = 20_000
    ev = DeviceBatch(mf, cuda, m)
    ev.generate(mf, mf.synth_params(6, m, intime_log=True, lo=0.1, hi=1000.0, pileup_mean=4.0))
    eng.fit_device(ev.batch, mf.default_options(precision=mf.PREC_FP32, warm_start=mf.WARM_MLP, max_iter_nnls=1000))
    warm = ev.outputs_host()
    eng.fit_device(ev.batch, mf.default_options(precision=mf.PREC_MIXED, max_iter_nnls=1000))
    cold = ev.outputs_host()
    ref = oracle_fit_sets(mf, oracle, eng, ev.inputs_host(), max_iter_nnls=1000, start=1)
    scale = np.maximum(np.abs(ref["amplitudes"]).max(axis=1), 1e-300)
    err = np.abs(warm["amplitudes"] - ref["amplitudes"]).max(axis=1) / scale
    assert (err <= 1e-4).mean() >= 0.999
    assert (warm["active_mask"] == ref["active_mask"]).mean() >= 0.999
    assert (warm["status"] == 0).all()
    # what the trained network gains: fewer FNNLS additions and solves than the cold start
    _, adds_w, solves_w = mf.unpack_iters(warm["iters"])
    _, adds_c, solves_c = mf.unpack_iters(cold["iters"])
    assert adds_w.mean() < 0.5 * adds_c.mean(), (adds_w.mean(), adds_c.mean())
    # predicted passive sets: most bits right (exact sets are rarer: the supports
    # of this ill-conditioned fit are partly decided by the noise)
    mask = cuda.zeros(m, dtype=cuda.int16, device="cuda")
    amp = cuda.zeros((m, 10), dtype=cuda.float32, device="cuda")
    eng.mlp_predict(ev.batch, mask.data_ptr(), amp.data_ptr())
    pred = mask.cpu().numpy().view(np.uint16)
    bit_acc = np.mean([((pred >> k) & 1) == ((ref["active_mask"] >> k) & 1) for k in range(10)])
    assert bit_acc > 0.8, bit_acc


def test_weights_roundtrip(mf, cuda, mlp_engine, tmp_path):
    eng = mlp_engine
    w = eng.mlp_get_weights()
    path = tmp_path / "mlp.bin"
    mf.save_mlp_weights(str(path), w, {"trained_on": "test"})
    w2, hdr = mf.load_mlp_weights(str(path))
    assert np.array_equal(w, w2) and hdr["trained_on"] == "test"
    eng.mlp_set_weights(w2)
    assert np.array_equal(eng.mlp_get_weights(), w)


def test_warm_fused_mixed_batch(mf, oracle, cuda):
    """The fused warm kernel on a batch mixing ECAL (learned start) and HCAL
    (cold start) channels, against the FP64 oracle."""
    eng = mf.Engine(0)
    eng.set_conditions(0, mf.synth_conditions(mf.SYNTH_ECAL)[0])
    eng.set_conditions(1, mf.synth_conditions(mf.SYNTH_HCAL)[0])
    eng.mlp_init(0, seed=3)
    tr = DeviceBatch(mf, cuda, 65_536)
    tr.generate(mf, mf.synth_params(5, 65_536, intime_log=True, lo=0.1, hi=1000.0, pileup_mean=4.0))
    eng.fit_device(tr.batch, mf.default_options(max_iter_nnls=1000, nnls_start=mf.START_SUPPORT))
    eng.mlp_train(tr.batch, mf.mlp_params(epochs=2, batch=4096))
    m = 30_000
    db = DeviceBatch(mf, cuda, m, ctype=True)
    db.generate(mf, mf.synth_params(4, m, pileup_mean=-8.0, hcal_fraction=0.4))
    eng.fit_device(db.batch, mf.default_options(precision=mf.PREC_MIXED, warm_start=mf.WARM_MLP, max_iter_nnls=1000))
    gpu = db.outputs_host()
    inp = db.inputs_host()
    ref = oracle_fit_sets(mf, oracle, eng, inp, max_iter_nnls=1000, start=1)
    scale = np.maximum(np.abs(ref["amplitudes"]).max(axis=1), 1e-300)
    err = np.abs(gpu["amplitudes"] - ref["amplitudes"]).max(axis=1) / scale
    assert (err <= 1e-4).mean() >= 0.999
    assert (gpu["active_mask"] == ref["active_mask"]).mean() >= 0.999
    assert (gpu["status"] == 0).all()
    eng.close()


def test_mixed_fp64_flop_counter(mf, cuda):
    """The instrumented mixed kernel reports its FP64 work; the outputs are unchanged by counting."""
    eng = mf.Engine(0)
    eng.set_conditions(0, mf.synth_conditions(mf.SYNTH_ECAL)[0])
    n = 8192
    db = DeviceBatch(mf, cuda, n)
    db.generate(mf, mf.synth_params(3, n, intime_log=True, lo=0.1, hi=1000.0, pileup_mean=4.0))
    opt = mf.default_options(precision=mf.PREC_MIXED, max_iter_nnls=1000)
    eng.fit_device(db.batch, opt)
    a = db.outputs_host()
    flops = cuda.zeros(n, dtype=cuda.float64, device="cuda")
    eng.fit_count_flops(db.batch, flops.data_ptr(), opt)
    b = db.outputs_host()
    assert np.array_equal(a["amplitudes"], b["amplitudes"])
    f = flops.cpu().numpy()
    # whitening 110 + chi2 22 at least (the judge's solve and residual run over
    # the passive set only: 40 per column)
    assert (f >= 110 + 22).all() and f.mean() < 2000 and (f > 132).mean() > 0.9
    eng.close()


def test_inference_matches_cpu_network(mf, cuda, mlp_engine):
    """The inference kernel (tcgen05.mma: BF16 operands from shared memory,
    FP32 accumulators in tensor memory; bias + ReLU + BF16 rounding in one
    packed convert per two activations) against the FP64 checker network with
    the same BF16 rounding points, on the same BF16 features. The two differ
    only by the FP32 accumulation order of the tensor cores, which can move a
    hidden activation across a BF16 rounding boundary (one ulp, 2^-8
    relative): the raw outputs must agree to 2 % of max(1, |output|) per value
    and 0.2 % on average."""
    eng = mlp_engine
    B = 4096
    db = train_set(mf, cuda, eng, B, seed=41)
    _, X, _, _ = eng.mlp_gradient(db.batch, mf.mlp_params(epochs=1, batch=B))
    logits = cuda.zeros((B, 32), dtype=cuda.float32, device="cuda")
    mask = cuda.zeros(B, dtype=cuda.int16, device="cuda")
    amp = cuda.zeros((B, 10), dtype=cuda.float32, device="cuda")
    eng.mlp_predict(db.batch, mask.data_ptr(), amp.data_ptr(), logits.data_ptr())
    cuda.cuda.synchronize()
    ref = mo.forward(mo.unflatten(eng.mlp_get_weights()), X.astype(np.float64))["O"]
    rel = np.abs(logits.cpu().numpy() - ref) / np.maximum(1.0, np.abs(ref))
    assert rel.max() <= 2e-2, rel.max()
    assert rel.mean() <= 2e-3, rel.mean()
    # the decode: a column is predicted where its logit exceeds -0.5
    lg = logits.cpu().numpy()
    want = np.zeros(B, np.uint16)
    for k in range(10):
        want |= (lg[:, k] > -0.5).astype(np.uint16) << k
    assert np.array_equal(mask.cpu().numpy().view(np.uint16), want)


def test_inference_timeout_reports_and_keeps_results(mf, cuda, mlp_engine):
    """The tensor-core inference's bounded waits: with the test hook every wait
    of the MLP kernel gives up after 1 ms (an mbarrier nothing arrives on).
    mf_fit_host returns MF_ETIMEOUT, the in-flight MMAs drain before the tensor
    memory is freed, the channels are fitted from a cold start -- the same
    results as the warm fit within the form's tolerance -- and the next fit,
    hook off, succeeds and matches the warm fit bit for bit."""
    import ctypes as C

    eng = mlp_engine
    tr = train_set(mf, cuda, eng, 16_384, seed=43)
    eng.mlp_train(tr.batch, mf.mlp_params(epochs=1, batch=4096))
    m = 20_000
    ev = DeviceBatch(mf, cuda, m)
    ev.generate(mf, mf.synth_params(44, m, intime_log=True, lo=0.1, hi=1000.0, pileup_mean=4.0))
    inp = ev.inputs_host()
    opt = mf.default_options(precision=mf.PREC_FP32, warm_start=mf.WARM_MLP, max_iter_nnls=1000)
    warm = eng.fit_host(inp["samples"], inp["pederr"], options=opt)

    out = {k: np.zeros_like(v) for k, v in warm.items()}
    b = mf.Engine._batch(m, 10, 10, inp["samples"].ctypes.data, inp["pederr"].ctypes.data, None,
                         out["amplitudes"].ctypes.data, out["chi2"].ctypes.data, out["intime"].ctypes.data,
                         out["errors"].ctypes.data, out["active_mask"].ctypes.data, out["status"].ctypes.data,
                         out["iters"].ctypes.data)
    eng.mlp_test_stall(True)
    try:
        rc = eng.lib.mf_fit_host(eng.h, C.byref(b), C.byref(opt))
    finally:
        eng.mlp_test_stall(False)
    assert rc == mf.ETIMEOUT, rc
    err = relerr_rows(out["amplitudes"], warm["amplitudes"])
    assert (err <= 1e-4).mean() >= 0.999
    assert (out["active_mask"] == warm["active_mask"]).mean() >= 0.999
    assert (out["status"] == 0).all()

    again = eng.fit_host(inp["samples"], inp["pederr"], options=opt)  # flag cleared, context healthy
    for k in ("amplitudes", "chi2", "active_mask"):
        assert np.array_equal(again[k], warm[k]), k


def test_training_timeout_reports_and_recovers(mf, cuda):
    """The training GEMMs' bounded waits: with the test hook every tcgen05
    wait of a training GEMM gives up after 1 ms (an mbarrier nothing arrives
    on). mf_mlp_train returns MF_ETIMEOUT and leaves the network untrained (a
    warm fit is refused with MF_ENOTRAINED); with the hook off the same
    training succeeds and the warm fit runs."""
    import ctypes as C

    eng = mf.Engine(0)
    eng.set_conditions(0, mf.synth_conditions(mf.SYNTH_ECAL)[0])
    eng.mlp_init(0, seed=9)
    tr = train_set(mf, cuda, eng, 8192, seed=45)
    p = mf.mlp_params(epochs=1, batch=4096)
    losses = np.zeros(1, dtype=np.float32)
    eng.mlp_test_stall(True)
    try:
        rc = eng.lib.mf_mlp_train(eng.h, C.byref(tr.batch), C.byref(p), losses.ctypes.data, None)
    finally:
        eng.mlp_test_stall(False)
    assert rc == mf.ETIMEOUT, rc
    assert "timed out" in mf.load_library().mf_last_error().decode()
    opt = mf.default_options(precision=mf.PREC_FP32, warm_start=mf.WARM_MLP, max_iter_nnls=1000)
    inp = tr.inputs_host()
    with pytest.raises(mf.MultifitError, match=rf"\({mf.ENOTRAINED}\)"):
        eng.fit_host(inp["samples"][:1000], inp["pederr"][:1000], options=opt)
    eng.mlp_train(tr.batch, p)  # hook off: trains, and the warm fit runs
    out = eng.fit_host(inp["samples"][:1000], inp["pederr"][:1000], options=opt)
    assert np.isfinite(out["amplitudes"]).all()
    eng.close()


def relerr_rows(a, r):
    return np.abs(a - r).max(axis=1) / np.maximum(np.abs(r).max(axis=1), 1e-300)
