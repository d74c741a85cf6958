"""The C ABI library: it loads without a GPU, exports every entry point that
include/*.h declares, and the ctypes mirror's structure layouts agree with the
C compiler's. No compute call needs a GPU here."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")]


def declared_functions():
    names = set()
    for h in HEADERS:
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b(mf_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ("mf_create", "mf_destroy", "mf_fit", "mf_fit_host", "mf_set_conditions",
                     "mf_build_pulse_matrix", "mf_synth_generate"):
        assert required in names


def test_library_exports_every_declared_symbol(mf):
    lib = mf.load_library()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.mf_abi_version() == 1


def test_nm_exports_are_c_symbols(mf):
    out = subprocess.run(["nm", "-D", "--defined-only", mf.LIB_PATH], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    for n in declared_functions():
        assert n in exported, n


LAYOUT_PROG = r"""
#include <stdio.h>
#include <stddef.h>
#include "multifit_gb300.h"
int main(void) {
  printf("%zu %zu %zu %zu\n", sizeof(mf_conditions), sizeof(mf_options), sizeof(mf_batch), sizeof(mf_synth_params));
  printf("%zu %zu %zu %zu\n", offsetof(mf_conditions, bxs), offsetof(mf_conditions, fullpulsecov),
         offsetof(mf_options, nnls_start), offsetof(mf_batch, iters));
  return 0;
}
"""


def test_struct_layouts_match_c(mf, tmp_path):
    src = tmp_path / "layout.c"
    src.write_text(LAYOUT_PROG)
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    lines = subprocess.check_output([str(exe)], text=True).split("\n")
    sizes = [int(x) for x in lines[0].split()]
    offs = [int(x) for x in lines[1].split()]
    assert sizes == [C.sizeof(mf.MfConditions), C.sizeof(mf.MfOptions), C.sizeof(mf.MfBatch),
                     C.sizeof(mf.MfSynthParams)]
    assert offs == [mf.MfConditions.bxs.offset, mf.MfConditions.fullpulsecov.offset,
                    mf.MfOptions.nnls_start.offset, mf.MfBatch.iters.offset]


def test_default_options_are_multifit_cpu(mf):
    o = mf.default_options()
    assert (o.max_iter_nnls, o.max_iter_outer, o.dchi2_tol, o.nnls_eps) == (10, 50, 1e-3, 1e-11)
    assert o.nnls_start == mf.START_REFERENCE and o.precision == mf.PREC_FP64


def test_argument_errors_without_gpu(mf):
    lib = mf.load_library()
    assert lib.mf_create(None, 0) == mf.EINVAL
    assert lib.mf_fit(None, None, None, None) == mf.EINVAL
    assert lib.mf_rc_string(mf.EUNSUPPORTED) == b"unsupported option combination"
    c = mf.MfConditions()
    c.nsamples, c.npulses = 11, 10
    with pytest.raises(mf.MultifitError):
        mf._check(lib.mf_synth_conditions(9, C.byref(c), C.byref(C.c_double())), "x")


def test_build_pulse_matrix_reference_rule(mf):
    """P(i,k) = fullpulse(i + 4 - bx_k) for i >= max(0, bx_k + 3), else 0
    (multifit_cpu/src/PulseChiSqSNNLS.cpp:49-62)."""
    fp = np.arange(19, dtype=np.float64) + 1.0
    bxs = np.arange(-5, 5)
    P = mf.build_pulse_matrix(fp, bxs, 10)
    for k, bx in enumerate(bxs):
        first = max(0, bx + 3)
        for i in range(10):
            exp = fp[i + 4 - bx] if i >= first else 0.0
            assert P[i, k] == exp
    with pytest.raises(mf.MultifitError):
        mf.build_pulse_matrix(fp, np.array([-9]), 10)  # reads before fullpulse(0)


@pytest.mark.parametrize("kind", [0, 1])
def test_mixed_tables_are_least_squares_operators(mf, kind):
    """The pseudo-inverse of every passive set equals numpy's least-squares
    solution of the whitened problem (the tables behind the mixed form)."""
    cond, sigma = mf.synth_conditions(kind)
    P, R, bxs, _ = mf.conditions_arrays(cond)
    N, K = P.shape
    Lr = np.linalg.cholesky(R)
    G = np.linalg.solve(Lr, P)
    W, _ = mf.table_operator(cond, 1)
    np.testing.assert_allclose(W, np.linalg.inv(Lr), rtol=1e-12, atol=1e-14)
    rng = np.random.default_rng(kind)
    y = rng.standard_normal(N)
    for mask in list(rng.integers(1, 1 << K, size=40)) + [(1 << K) - 1, 1]:
        cols = [k for k in range(K) if mask >> k & 1]
        _, Pi = mf.table_operator(cond, int(mask))
        x = Pi @ y
        xr = np.linalg.lstsq(G[:, cols], y, rcond=None)[0]
        np.testing.assert_allclose(x, xr, rtol=1e-9, atol=1e-12 * np.abs(xr).max())
