"""mf_fit_noalloc, the allocation-free variant of the mixed-precision fit (its
search-to-judge hand-off lives in a static device array), against mf_fit with
the same options on the same device inputs.

Tolerance: zero. Both entry points run the same kernels on the same inputs and
every channel's arithmetic is independent of the others, so amplitudes, chi2,
active sets, status and iteration counts must agree bit for bit.

Named so that pytest collects it last: it must pass both alone and after the
rest of the suite (the scratch is per device and outlives every context).
"""
import ctypes as C

import numpy as np
import pytest

from _helpers import DeviceBatch

pytestmark = pytest.mark.gpu

AMP_TOL = 0.0  # identical kernels and inputs


def ecal_hcal_engine(mf):
    eng = mf.Engine(0)
    eng.set_conditions(0, mf.synth_conditions(mf.SYNTH_ECAL)[0])
    eng.set_conditions(1, mf.synth_conditions(mf.SYNTH_HCAL)[0])
    return eng


def mixed_options(mf, precision=None):
    return mf.default_options(precision=mf.PREC_MIXED if precision is None else precision, max_iter_nnls=1000)


PRECISIONS = ["mixed", "fp32"]


def precision_of(mf, name):
    return {"mixed": mf.PREC_MIXED, "fp32": mf.PREC_FP32}[name]


def assert_same(a, b):
    for k in ("amplitudes", "chi2", "intime"):
        np.testing.assert_allclose(a[k], b[k], rtol=AMP_TOL, atol=0.0, err_msg=k)
    for k in ("active_mask", "status", "iters"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


@pytest.mark.parametrize("prec", PRECISIONS)
def test_noalloc_matches_mf_fit_two_calls_in_a_row(mf, cuda, prec):
    eng = ecal_hcal_engine(mf)
    opt = mixed_options(mf, precision_of(mf, prec))
    # first call at the size limit, second smaller and with other inputs: what
    # the first call left in the scratch must not leak into the second
    sizes = [(mf.NOALLOC_MAX_CHANNELS, 11), (40_000, 12)]
    batches = []
    for n, seed in sizes:
        db = DeviceBatch(mf, cuda, n, ctype=True)
        db.generate(mf, mf.synth_params(seed, n, intime_log=True, lo=0.1, hi=1000.0, pileup_mean=-8.0,
                                        hcal_fraction=0.4))
        batches.append(db)
    expected = []
    for db in batches:
        eng.fit_device(db.batch, opt)
        expected.append(db.outputs_host())
    for db in batches:
        for v in db.out.values():
            v.fill_(0)
    cuda.cuda.synchronize()
    for db, exp in zip(batches, expected):
        assert eng.fit_noalloc(db.batch, opt) == mf.OK, mf.load_library().mf_last_error()
        got = db.outputs_host()
        assert_same(got, exp)
        assert (got["status"] == 0).all()
        assert set(np.unique(db.inputs_host()["ctype"])) == {0, 1}
    eng.close()


def test_noalloc_rejects_oversize_batch_untouched(mf, cuda):
    eng = ecal_hcal_engine(mf)
    n = mf.NOALLOC_MAX_CHANNELS + 1
    db = DeviceBatch(mf, cuda, n, ctype=True)
    db.generate(mf, mf.synth_params(13, n, pileup_mean=2.0, hcal_fraction=0.4))
    db.out["chi2"].fill_(-1.0)
    cuda.cuda.synchronize()
    assert eng.fit_noalloc(db.batch, mixed_options(mf)) == mf.EINVAL
    msg = mf.load_library().mf_last_error().decode()
    assert "MF_NOALLOC_MAX_CHANNELS" in msg and str(n) in msg
    assert (db.outputs_host()["chi2"] == -1.0).all()  # nothing launched
    eng.close()


def test_noalloc_option_limits(mf, cuda):
    eng = ecal_hcal_engine(mf)
    db = DeviceBatch(mf, cuda, 1000, ctype=True)
    db.generate(mf, mf.synth_params(14, 1000, pileup_mean=2.0, hcal_fraction=0.4))
    assert eng.fit_noalloc(db.batch, mf.default_options()) == mf.EUNSUPPORTED  # plain FP64
    assert eng.fit_noalloc(db.batch, mf.default_options(precision=mf.PREC_MIXED, warm_start=1)) == \
        mf.EUNSUPPORTED
    empty = mf.Engine._batch(0, 10, 10, None, None, None, None, None)
    assert eng.fit_noalloc(empty, mixed_options(mf)) == mf.OK
    eng.close()


@pytest.mark.parametrize("prec", PRECISIONS)
def test_noalloc_allocates_nothing_on_a_side_stream(mf, cuda, prec):
    """What the entry point exists for: after a first call (which resolves the
    scratch address and loads the kernels), further calls on a non-default
    stream leave the device's free memory and torch's allocator untouched, and
    give mf_fit's results."""
    torch = cuda
    eng = ecal_hcal_engine(mf)
    opt = mixed_options(mf, precision_of(mf, prec))
    n = 20_000
    db = DeviceBatch(mf, torch, n, ctype=True)
    db.generate(mf, mf.synth_params(15, n, intime_log=True, lo=0.1, hi=1000.0, pileup_mean=-8.0,
                                    hcal_fraction=0.4))
    eng.fit_device(db.batch, opt)
    expected = db.outputs_host()
    side = torch.cuda.Stream()
    assert eng.fit_noalloc(db.batch, opt, side.cuda_stream) == mf.OK
    side.synchronize()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    alloc0 = torch.cuda.memory_allocated()
    for _ in range(3):
        assert eng.fit_noalloc(db.batch, opt, side.cuda_stream) == mf.OK
    side.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert torch.cuda.memory_allocated() == alloc0
    assert_same(db.outputs_host(), expected)
    eng.close()


def test_noalloc_rejects_a_grid_block_above_128(mf, cuda):
    eng = ecal_hcal_engine(mf)
    db = DeviceBatch(mf, cuda, 1000, ctype=True)
    db.generate(mf, mf.synth_params(16, 1000, pileup_mean=2.0, hcal_fraction=0.4))
    opt = mixed_options(mf)
    opt.block_size = 256
    assert eng.fit_noalloc(db.batch, opt) == mf.EINVAL
    assert "128" in mf.load_library().mf_last_error().decode()
    opt.block_size = 64
    assert eng.fit_noalloc(db.batch, opt) == mf.OK
    eng.close()


def test_noalloc_needs_the_contexts_device_current(mf, cuda):
    if cuda.cuda.device_count() < 2:
        pytest.skip("needs two devices")
    eng = mf.Engine(1)
    eng.set_conditions(0, mf.synth_conditions(mf.SYNTH_ECAL)[0])
    cuda.cuda.set_device(0)
    db = DeviceBatch(mf, cuda, 100)
    assert eng.fit_noalloc(db.batch, mixed_options(mf)) == mf.EINVAL
    assert "current device" in mf.load_library().mf_last_error().decode()
    eng.close()
