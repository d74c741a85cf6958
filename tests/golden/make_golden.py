"""Generates the golden fixtures of the parity tests (run where the reference
tree is present; the fixtures are committed and nothing reads the reference
at test time).

linalgebra_ref.npz
    Outputs of the reference's OWN linalgebra code (linalgebra/interface/
    cholesky.hpp, substitution.hpp, fused_cholesky_substitution.hpp, compiled
    from the reference sources into oracle/_ref by oracle/build_oracle.py) on
    seeded SPD matrices: the Cholesky factor, forward and backward
    substitution for every view size, the fused rank-1 row addition and the
    in-between removal. They pin the oracle's restatement to the reference.
fits_*.npz
    Seeded channels (the engine's counter-based generator, host path) with
    their conditions and the oracle's outputs for the reference start
    (max_iter 10, the multifit_cpu configuration), the support start at KKT
    convergence (max_iter 1000), and the MINOS-like errors. They pin the
    generator, the oracle and (in the GPU tests) the FP64 kernel bit for bit.

Usage: python tests/golden/make_golden.py
"""
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

spec = importlib.util.spec_from_file_location("multifit_gb300", os.path.join(ROOT, "test-regression_gb300",
                                                                             "__init__.py"))
mf = importlib.util.module_from_spec(spec)
sys.modules["multifit_gb300"] = mf
spec.loader.exec_module(mf)

N = 10


def spd(rng, n, cond):
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    ev = np.geomspace(1.0, cond, n)
    M = (Q * ev) @ Q.T
    return (M + M.T) / 2


def linalgebra_fixture(cases=8):
    ref = oracle.ref()
    if ref is None:
        raise SystemExit("the reference tree is needed to build oracle/_ref")
    rng = np.random.default_rng(2024)
    out = {k: [] for k in ("M", "b", "L", "y", "x", "add_view", "add_L0", "add_y0", "add_L", "add_y",
                           "rm_pos", "rm_M", "rm_b", "rm_L", "rm_y")}
    for _ in range(cases):
        M = spd(rng, N, 10 ** rng.uniform(0, 6)) * 10 ** rng.uniform(-2, 2)
        Mf = np.ascontiguousarray(M).ravel()
        b = rng.standard_normal(N) * 10 ** rng.uniform(-1, 3)
        Ls, ys, xs = [], [], []
        for view in range(1, N + 1):
            L = np.zeros(N * N)
            ref.ref_cholesky_decomp(Mf.copy(), L, N, view)
            y = np.zeros(N)
            ref.ref_forward(L.copy(), b.copy(), y, N, view)
            x = np.zeros(N)
            ref.ref_backward(L.copy(), y.copy(), x, N, view)
            y[view:] = 0.0
            x[view:] = 0.0
            Ls.append(L)
            ys.append(y)
            xs.append(x)
        out["M"].append(Mf)
        out["b"].append(b)
        out["L"].append(np.array(Ls))
        out["y"].append(np.array(ys))
        out["x"].append(np.array(xs))
        # fused rank-1 row addition: factor of view-1, add row view-1
        view = int(rng.integers(2, N + 1))
        L0 = np.zeros(N * N)
        ref.ref_cholesky_decomp(Mf.copy(), L0, N, view - 1)
        y0 = np.zeros(N)
        ref.ref_forward(L0.copy(), b.copy(), y0, N, view - 1)
        y0[view - 1:] = 0.0
        La, ya = L0.copy(), y0.copy()
        ref.ref_rc_addition(Mf.copy(), La, b.copy(), ya, N, view)
        ya[view:] = 0.0
        out["add_view"].append(view)
        out["add_L0"].append(L0)
        out["add_y0"].append(y0)
        out["add_L"].append(La)
        out["add_y"].append(ya)
        # in-between removal of position pos from the full factor, the removed
        # row/column swapped to the end first (symmetric swap, as the caller does)
        pos = int(rng.integers(0, N - 1))
        Lf = np.zeros(N * N)
        ref.ref_cholesky_decomp(Mf.copy(), Lf, N, N)
        yf = np.zeros(N)
        ref.ref_forward(Lf.copy(), b.copy(), yf, N, N)
        Ms = M.copy()
        perm = np.arange(N)
        perm[[pos, N - 1]] = perm[[N - 1, pos]]
        Ms = np.ascontiguousarray(Ms[np.ix_(perm, perm)]).ravel()
        bs = b[perm].copy()
        Lr, yr = Lf.copy(), yf.copy()
        ref.ref_inbetween_removal(Ms.copy(), Lr, bs.copy(), yr, pos, N, N - 1)
        yr[N - 1:] = 0.0
        out["rm_pos"].append(pos)
        out["rm_M"].append(Ms)
        out["rm_b"].append(bs)
        out["rm_L"].append(Lr)
        out["rm_y"].append(yr)
        out.setdefault("rm_L0", []).append(Lf)
        out.setdefault("rm_y0", []).append(yf)
    np.savez_compressed(os.path.join(HERE, "linalgebra_ref.npz"), **{k: np.array(v) for k, v in out.items()})


def fits_fixture(name, cond, inputs, fpc=None):
    P, R, bxs, _ = mf.conditions_arrays(cond)
    s, pe = inputs["samples"], inputs["pederr"]
    res = {"samples": s, "pederr": pe, "P": P, "R": R, "bxs": bxs}
    if fpc is not None:
        res["fullpulsecov"] = fpc
    for tag, kw in (("ref", dict(start=0, max_iter_nnls=10)), ("kkt", dict(start=1, max_iter_nnls=1000)),
                    ("err", dict(start=1, max_iter_nnls=1000, compute_errors=True))):
        o = oracle.fit_batch(s, pe, P, R, bxs, fullpulsecov=fpc, **kw)
        for k in ("amplitudes", "chi2", "active_mask", "status", "iters"):
            res[f"{tag}_{k}"] = o[k]
        if tag == "err":
            res["err_errors"] = o["errors"]
    np.savez_compressed(os.path.join(HERE, f"fits_{name}.npz"), **res)


def edge_inputs():
    """Hand-made channels: zero, negative, huge, tiny-noise, pure-pileup and
    saturating samples (the cases the reference driver can meet)."""
    ecal, _ = mf.synth_conditions(mf.SYNTH_ECAL)
    P, _, _, _ = mf.conditions_arrays(ecal)
    rows, ped = [], []
    rows.append(np.zeros(N)); ped.append(0.044)
    rows.append(-0.1 * np.ones(N)); ped.append(0.044)
    rows.append(1e4 * P[:, 5]); ped.append(0.044)
    rows.append(50.0 * P[:, 5] + 3.0 * P[:, 2]); ped.append(1e-6)
    rows.append(7.0 * P[:, 0] + 2.0 * P[:, 9]); ped.append(0.044)
    rows.append(np.full(N, 4095.0)); ped.append(0.044)
    rows.append(np.linspace(-1, 1, N)); ped.append(10.0)
    rows.append(1e-300 * np.ones(N)); ped.append(0.044)
    return {"samples": np.array(rows), "pederr": np.array(ped)}


def main():
    linalgebra_fixture()
    ecal, _ = mf.synth_conditions(mf.SYNTH_ECAL)
    hcal, _ = mf.synth_conditions(mf.SYNTH_HCAL)
    # ECAL c0 generator (10,000-channel workload, seed 1): its first 256 channels
    fits_fixture("ecal_c0", ecal, mf.synth_generate_host(mf.WORKLOADS["ecal-10k-pu0.5"](), 0, 256, with_truth=False))
    # log-uniform [0.1, 1000] GeV, pileup 4 (the mixed-precision workload, seed 3)
    fits_fixture("ecal_logamp", ecal,
                 mf.synth_generate_host(mf.WORKLOADS["ecal-10m-logamp-pu4"](), 0, 256, with_truth=False))
    # HCAL 8x8 channels (pileup per channel U[0,8])
    fits_fixture("hcal", hcal, mf.synth_generate_host(mf.synth_params(4, 256, pileup_mean=-8.0, hcal_fraction=1.0),
                                                      0, 256, with_truth=False))
    # ECAL with a non-zero pulse covariance (the outer chi2 loop iterates)
    F = np.zeros((19, 19))
    idx = np.arange(7, 19)
    F[np.ix_(idx, idx)] = 1e-4 * np.exp(-np.abs(np.subtract.outer(idx, idx)) / 3.0)
    fits_fixture("ecal_fpc", mf.make_conditions(*mf.conditions_arrays(ecal)[:3], fullpulsecov=F),
                 mf.synth_generate_host(mf.synth_params(8, 128, pileup_mean=2.0), 0, 128, with_truth=False), fpc=F)
    fits_fixture("edge", ecal, edge_inputs())


if __name__ == "__main__":
    main()
