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


def mixed_options(mf):
    return mf.default_options(precision=mf.PREC_MIXED, max_iter_nnls=1000)


def assert_same(a, b):
    for k in ("amplitudes", "chi2", "intime"):
        np.testing.assert_allclose(a[k], b[k], rtol=AMP_TOL, atol=0.0, err_msg=k)
    for k in ("active_mask", "status", "iters"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_noalloc_matches_mf_fit_two_calls_in_a_row(mf, cuda):
    eng = ecal_hcal_engine(mf)
    opt = mixed_options(mf)
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
