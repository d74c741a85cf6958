"""The oracle's own seeded generator (oracle/synth_oracle.cpp) makes the same
channels and condition sets as the engine's host generator (mf_synth_generate
with on_device=0, mf_synth_conditions), so the CPU arms of the benchmark can
build the benchmark's workloads without loading the engine library. CPU only."""
import numpy as np
import pytest


@pytest.mark.parametrize("kind", [0, 1])
def test_conditions_equal_the_engine_sets(mf, oracle, kind):
    P, R, bxs, sigma = oracle.synth_conditions(kind)
    c, s = mf.synth_conditions(kind)
    P2, R2, bx2, _ = mf.conditions_arrays(c)
    assert np.array_equal(P, P2)
    assert np.array_equal(R, R2)
    assert np.array_equal(bxs, bx2)
    assert sigma == s


@pytest.mark.parametrize("name,first,count", [
    ("ecal-10k-pu0.5", 0, 3000),
    ("ecal-1m-pu2", 123_456, 2500),
    ("warm-eval-10m", 9_990_000, 10_000),   # multi-threaded path (count >= 4096)
    ("mixed-10m-ecal-hcal", 5_000_000, 6000),
    ("warm-train-5m", 0, 1),
])
def test_channels_bit_identical_to_engine_host_generator(mf, oracle, name, first, count):
    w = oracle.WORKLOADS[name]
    p = mf.WORKLOADS[name]()
    assert (p.seed, p.n) == (w["seed"], w["n"])
    a = oracle.synth_generate(name, first, count, with_truth=True)
    b = mf.synth_generate_host(p, first, count, with_truth=True)
    for k in ("samples", "pederr", "ctype", "truth"):
        assert np.array_equal(a[k], b[k]), k


def test_thread_count_does_not_change_channels(oracle):
    a = oracle.synth_generate("warm-eval-10m", 0, 20_000, nthreads=1)
    b = oracle.synth_generate("warm-eval-10m", 0, 20_000, nthreads=7)
    assert np.array_equal(a["samples"], b["samples"])


def test_bad_arguments_raise(oracle):
    with pytest.raises(ValueError):
        oracle.synth_conditions(7)
    with pytest.raises(ValueError):
        oracle.synth_generate("ecal-10k-pu0.5", 0, 10, stride=9)
