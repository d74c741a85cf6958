"""GPU parity of the plain FP64 fit (mf_fit, precision FP64) against the CPU
oracle, through the C ABI, on the same seeded inputs.

The FP64 kernel and the oracle share one canonical operation order, so every
output is compared bit for bit: amplitudes, chi2, the active mask, the status
word and the iteration counters, for both FNNLS iteration caps of the
reference (10 as multifit_cpu, 1000 as multifit_gpu) and both FNNLS starts.
At the 1,000,000-channel size of the GPU configuration a random sample of
channels is re-fitted by the oracle (channels are independent), and the whole
batch is checked for size-independent properties.
"""
import numpy as np
import pytest

from _helpers import DeviceBatch, assert_bitwise, oracle_fit_sets

pytestmark = pytest.mark.gpu


def ecal_engine(mf, engine):
    cond, _ = mf.synth_conditions(mf.SYNTH_ECAL)
    engine.set_conditions(0, cond)
    engine.conditions.pop(1, None)
    return cond


def mixed_engine(mf, engine):
    e, _ = mf.synth_conditions(mf.SYNTH_ECAL)
    h, _ = mf.synth_conditions(mf.SYNTH_HCAL)
    engine.set_conditions(0, e)
    engine.set_conditions(1, h)


WORKLOADS = {
    "ecal-pu0.5": dict(seed=1, pileup_mean=0.5),
    "ecal-pu2": dict(seed=2, pileup_mean=2.0),
    "ecal-logamp-pu4": dict(seed=3, intime_log=True, lo=0.1, hi=1000.0, pileup_mean=4.0),
}


@pytest.mark.parametrize("wl", list(WORKLOADS))
@pytest.mark.parametrize("max_iter", [10, 1000])
@pytest.mark.parametrize("start", [0, 1])
def test_fp64_bitwise_ecal(mf, oracle, engine, cuda, wl, max_iter, start):
    ecal_engine(mf, engine)
    n = 8192
    db = DeviceBatch(mf, cuda, n)
    db.generate(mf, mf.synth_params(n=n, **WORKLOADS[wl]))
    opt = mf.default_options(max_iter_nnls=max_iter, nnls_start=start)
    engine.fit_device(db.batch, opt)
    gpu = db.outputs_host()
    ref = oracle_fit_sets(mf, oracle, engine, db.inputs_host(), max_iter_nnls=max_iter, start=start)
    assert_bitwise(gpu, ref)
    assert np.array_equal(gpu["intime"], gpu["amplitudes"][:, 5])


@pytest.mark.parametrize("block", [32, 64, 96, 128])
def test_fp64_launch_shapes_bitwise(mf, oracle, engine, cuda, block):
    """The kernel's schedule (one wave of resident blocks, each warp a range
    of channels, the first outer iterations in lockstep, the rest with lanes
    taking their warp's next channel) changes with the block size and the
    batch size; the fits must not: every block size on an ECAL/HCAL batch
    whose size is no multiple of 32, with the error refits, bit for bit."""
    mixed_engine(mf, engine)
    n = 50_021
    db = DeviceBatch(mf, cuda, n, ctype=True)
    db.generate(mf, mf.synth_params(seed=17, n=n, pileup_mean=-8.0, hcal_fraction=0.4))
    opt = mf.default_options(compute_errors=1, block_size=block)
    engine.fit_device(db.batch, opt)
    gpu = db.outputs_host()
    ref = oracle_fit_sets(mf, oracle, engine, db.inputs_host(), compute_errors=True)
    assert_bitwise(gpu, ref, fields=("amplitudes", "chi2", "active_mask", "status", "errors"))


@pytest.mark.parametrize("start", [0, 1])
def test_fp64_bitwise_mixed_ecal_hcal(mf, oracle, engine, cuda, start):
    mixed_engine(mf, engine)
    n = 8192
    db = DeviceBatch(mf, cuda, n, ctype=True)
    db.generate(mf, mf.synth_params(4, n, pileup_mean=-8.0, hcal_fraction=0.4))
    inp = db.inputs_host()
    assert 0.3 < inp["ctype"].mean() < 0.5
    engine.fit_device(db.batch, mf.default_options(nnls_start=start))
    gpu = db.outputs_host()
    ref = oracle_fit_sets(mf, oracle, engine, inp, start=start)
    assert_bitwise(gpu, ref)
    h = inp["ctype"] == 1
    assert (gpu["amplitudes"][h, 8:] == 0).all()


def test_fp64_errors_bitwise(mf, oracle, engine, cuda):
    ecal_engine(mf, engine)
    n = 4096
    db = DeviceBatch(mf, cuda, n)
    db.generate(mf, mf.synth_params(7, n, pileup_mean=0.5))
    engine.fit_device(db.batch, mf.default_options(compute_errors=1))
    gpu = db.outputs_host()
    ref = oracle_fit_sets(mf, oracle, engine, db.inputs_host(), compute_errors=True)
    assert_bitwise(gpu, ref, fields=("amplitudes", "chi2", "errors", "active_mask", "status"))


def test_fp64_flop_count_matches_oracle(mf, oracle, engine, cuda):
    ecal_engine(mf, engine)
    n = 2048
    db = DeviceBatch(mf, cuda, n)
    db.generate(mf, mf.synth_params(2, n, pileup_mean=2.0))
    flops = cuda.zeros(n, dtype=cuda.float64, device="cuda")
    engine.fit_count_flops(db.batch, flops.data_ptr(), mf.default_options())
    gpu = db.outputs_host()
    ref = oracle_fit_sets(mf, oracle, engine, db.inputs_host(), count_flops=True)
    assert_bitwise(gpu, ref)
    assert np.array_equal(flops.cpu().numpy(), ref["flops"])


def test_fp64_full_size_1m(mf, oracle, engine, cuda):
    """1,000,000 ECAL channels at pileup 2 (the GPU FP64 configuration):
    bitwise parity on a random sample and batch-wide properties."""
    ecal_engine(mf, engine)
    n = 1_000_000
    db = DeviceBatch(mf, cuda, n)
    db.generate(mf, mf.synth_params(2, n, pileup_mean=2.0))
    engine.fit_device(db.batch, mf.default_options())
    gpu = db.outputs_host()
    inp = db.inputs_host()
    rng = np.random.default_rng(0)
    sel = np.sort(rng.choice(n, 20_000, replace=False))
    sub = {k: v[sel] for k, v in inp.items()}
    ref = oracle_fit_sets(mf, oracle, engine, sub)
    assert_bitwise({k: v[sel] for k, v in gpu.items()}, ref)
    # properties of the whole batch
    assert np.isfinite(gpu["amplitudes"]).all() and np.isfinite(gpu["chi2"]).all()
    assert (gpu["amplitudes"] >= 0).all()
    sup = ((gpu["amplitudes"] > 0) * (1 << np.arange(10))).sum(axis=1)
    assert np.array_equal(gpu["active_mask"].astype(np.int64), sup)
    assert (gpu["status"] & ~np.uint8(1) == 0).all()  # only FNNLS-cap flags (max_iter 10) may appear


def test_fit_host_equals_fit_device(mf, engine, cuda):
    ecal_engine(mf, engine)
    n = 3000
    db = DeviceBatch(mf, cuda, n)
    db.generate(mf, mf.synth_params(9, n, pileup_mean=2.0))
    engine.fit_device(db.batch, mf.default_options())
    gpu = db.outputs_host()
    inp = db.inputs_host()
    host = engine.fit_host(inp["samples"], inp["pederr"])
    for k in ("amplitudes", "chi2", "intime", "status", "iters"):
        assert np.array_equal(host[k], gpu[k]), k
    assert np.array_equal(host["active_mask"], gpu["active_mask"])


def test_edge_cases(mf, oracle, engine, cuda):
    ecal_engine(mf, engine)
    # empty batch is a no-op
    db0 = DeviceBatch(mf, cuda, 0)
    engine.fit_device(db0.batch, mf.default_options())
    cond, sigma = mf.synth_conditions(mf.SYNTH_ECAL)
    P, R, bxs, _ = mf.conditions_arrays(cond)
    s = np.zeros((6, 10))
    ped = np.full(6, sigma)
    s[1] = P[:, 5] * 50.0          # noiseless single pulse
    s[2, 3] = np.nan                # non-finite sample
    ped[3] = 0.0                    # zero noise: non-PD covariance
    s[3] = P[:, 5]
    s[4] = -P[:, 5] * 10.0          # negative pulse: all amplitudes clamp to 0
    s[5] = P @ np.full(10, 1e6)     # huge amplitudes
    out = engine.fit_host(s, ped)
    ref = oracle.fit_batch(s, ped, P, R, bxs)
    assert_bitwise(out, ref, iters=True)
    assert (out["amplitudes"][0] == 0).all() and out["chi2"][0] == 0.0 and out["status"][0] == 0
    assert abs(out["amplitudes"][1, 5] - 50.0) < 1e-9
    assert out["status"][2] & mf.CH_BADINPUT and out["status"][2] & mf.CH_NONFINITE
    assert out["status"][3] & mf.CH_NONFINITE
    assert (out["amplitudes"][4] == 0).all()
    assert np.isfinite(out["amplitudes"][5]).all()


def test_bad_condition_index(mf, cuda):
    eng = mf.Engine(0)
    ecal_engine(mf, eng)
    n = 4
    s = np.zeros((n, 10))
    ct = np.array([0, 1, 0, 7], dtype=np.uint8)
    # the host cannot see device-side indices: a channel naming a set that was
    # never given is flagged per channel
    out = eng.fit_host(s, np.full(n, 0.044), ctype=ct)
    assert list(out["status"]) == [0, mf.CH_BADINPUT, 0, mf.CH_BADINPUT]
    mixed_engine(mf, eng)
    out = eng.fit_host(s, np.full(n, 0.044), ctype=ct)
    assert out["status"][3] == mf.CH_BADINPUT
    eng.close()


def test_pulsechisq_mirror_matches_oracle(mf, oracle, cuda):
    """The reference-shaped per-channel API: DoFit(samples, samplecor, pederr,
    bxs, fullpulse, fullpulsecov) then X(), ChiSq(), Errors()."""
    cond, sigma = mf.synth_conditions(mf.SYNTH_ECAL)
    P, R, bxs, _ = mf.conditions_arrays(cond)
    # the 12-sample template: two samples before the peak (from the BX 0
    # column) followed by the whole BX -5 column, which starts at its peak
    fullpulse = np.zeros(19)
    fullpulse[7], fullpulse[8] = P[3, 5], P[4, 5]
    fullpulse[9:19] = P[:, 0]
    Pm = mf.build_pulse_matrix(fullpulse, bxs, 10)
    assert np.array_equal(Pm, P)
    data = mf.synth_generate_host(mf.synth_params(21, 16, pileup_mean=0.5), 0, 16)
    ref = oracle.fit_batch(data["samples"], data["pederr"], Pm, R, bxs, compute_errors=True)
    for c in range(16):
        f = mf.PulseChiSqSNNLS()
        assert f.DoFit(data["samples"][c], R, data["pederr"][c], bxs, fullpulse, np.zeros((19, 19)))
        assert np.array_equal(f.X(), ref["amplitudes"][c])
        assert f.ChiSq() == ref["chi2"][c]
        e, r = f.Errors()[5], ref["errors"][c]
        assert e == r or (np.isnan(e) and np.isnan(r))  # the reference start can leave NaN errors
