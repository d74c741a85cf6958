"""Checks of the oracle's FNNLS (nnls/src/inplace_fnnls.cu:72-233 and
nnls/src/inplace_fnnls_test_cholesky.cu:35-227) against independent solvers.

The reference ships no golden NNLS outputs (its tests only print), so the
restatement is cross-checked instead:
* fresh-LLT variant == incremental-Cholesky variant, bit for bit;
* run to convergence, it matches exhaustive passive-set enumeration, the
  Lawson-Hanson solver (the algorithm of nnls/src/nnls.cpp) and
  scipy.optimize.nnls, and satisfies KKT;
* a second, pure-Python restatement of the same loop (numpy solves) takes the
  same passive-set path on small cases, including the reference's warm start
  with stale amplitudes outside the passive set.
"""
import numpy as np
import pytest
import scipy.optimize


def random_problem(rng, N=10, K=10, cond_exp=2.0):
    A = rng.standard_normal((N, K)) * 10 ** rng.uniform(-1, 1, size=K)
    U, S, Vt = np.linalg.svd(A, full_matrices=False)
    S = np.geomspace(1, 10 ** -cond_exp, K) * S[0]
    A = (U * S) @ Vt
    xt = np.where(rng.random(K) < 0.5, rng.exponential(1.0, K), 0.0)
    b = A @ xt + 0.05 * rng.standard_normal(N) * np.abs(A).max()
    return A, b


def py_inplace_fnnls(A, b, x, eps, max_iter):
    """Pure-Python restatement of nnls/src/inplace_fnnls.cu:72-233 (numpy LLT solves)."""
    A = np.asarray(A, float)
    K = A.shape[1]
    AtA = A.T @ A
    Atb = A.T @ b
    x = np.array(x, float)
    perm = list(range(K))
    nP = 0
    path = []

    def swap(i, j):
        AtA[[i, j], :] = AtA[[j, i], :]
        AtA[:, [i, j]] = AtA[:, [j, i]]
        Atb[[i, j]] = Atb[[j, i]]
        x[[i, j]] = x[[j, i]]
        perm[i], perm[j] = perm[j], perm[i]

    for _ in range(max_iter):
        if nP == K:
            break
        w = Atb[nP:] - (AtA @ x)[nP:]
        imax = int(np.argmax(w))
        if w[imax] < eps:
            break
        swap(nP, nP + imax)
        path.append(("add", perm[nP]))
        nP += 1
        while nP > 0:
            Lc = np.linalg.cholesky(AtA[:nP, :nP])
            s = np.linalg.solve(Lc.T, np.linalg.solve(Lc, Atb[:nP]))
            if s.min() > 0:
                x[:nP] = s
                break
            alpha, ai = np.inf, 0
            for i in range(nP):
                if s[i] <= 0:
                    r = x[i] / (x[i] - s[i])
                    if r < alpha:
                        alpha, ai = r, i
            if not np.isfinite(alpha):
                x[:nP] = s
                break
            x[:nP] += alpha * (s - x[:nP])
            x[ai] = 0
            nP -= 1
            path.append(("remove", perm[ai]))
            swap(nP, ai)
    out = np.zeros(K)
    out[perm] = x
    return out, path, sorted(perm[:nP])


@pytest.mark.parametrize("seed", range(60))
def test_fresh_equals_incremental_bitwise(oracle, seed):
    rng = np.random.default_rng(seed)
    A, b = random_problem(rng, cond_exp=rng.uniform(0, 4))
    x0 = np.where(rng.random(10) < 0.3, rng.exponential(1.0, 10), 0.0)
    for max_iter in (10, 1000):
        xa, sa = oracle.inplace_fnnls(A, b, x0, max_iter=max_iter, variant=0)
        xb, sb = oracle.inplace_fnnls(A, b, x0, max_iter=max_iter, variant=1)
        assert np.array_equal(xa, xb)
        assert sa == sb


@pytest.mark.parametrize("seed", range(60))
def test_converged_matches_independent_solvers(oracle, seed):
    rng = np.random.default_rng(100 + seed)
    A, b = random_problem(rng, cond_exp=rng.uniform(0, 3))
    x, st = oracle.inplace_fnnls(A, b, None, eps=1e-11, max_iter=1000, variant=1)
    assert st["converged"] == 1
    xb, _ = oracle.nnls_bruteforce(A, b)
    xl = oracle.nnls_lawson_hanson(A, b)
    xs, _ = scipy.optimize.nnls(A, b)
    scale = max(np.abs(xb).max(), 1e-30)
    for other in (xb, xl, xs):
        np.testing.assert_allclose(x, other, rtol=0, atol=1e-8 * scale)
    assert ((x > 0) == (xb > 0)).all()
    g = oracle.kkt_violation(A, b, x)
    assert g <= 1e-9 * np.abs(A.T @ b).max()


@pytest.mark.parametrize("seed", range(40))
def test_python_restatement_same_path(oracle, seed):
    rng = np.random.default_rng(200 + seed)
    A, b = random_problem(rng, cond_exp=1.0)
    x0 = np.where(rng.random(10) < 0.4, rng.exponential(1.0, 10), 0.0)  # stale warm start
    xo, st = oracle.inplace_fnnls(A, b, x0, eps=1e-11, max_iter=1000, variant=0)
    xp, path, passive = py_inplace_fnnls(A, b, x0, 1e-11, 1000)
    mask = sum(1 << k for k in passive)
    assert st["mask"] == mask
    assert st["outer"] == sum(1 for p in path if p[0] == "add")
    np.testing.assert_allclose(xo, xp, rtol=1e-9, atol=1e-12 * np.abs(xp).max())


def test_warm_start_keeps_stale_entries(oracle):
    """The reference starts each FNNLS with an empty passive set but x = the
    previous amplitudes (multifit_cpu/src/PulseChiSqSNNLS.cpp:258): entries
    outside the final passive set keep their stale values."""
    A = np.eye(3)
    b = np.array([1.0, -1.0, 2.0])
    x0 = np.array([0.0, 5.0, 0.0])  # stale positive value in a column whose LS value is negative
    x, st = oracle.inplace_fnnls(A, b, x0, eps=1e-11, max_iter=1000, variant=1)
    # w = Atb - AtA x = (1, -6, 2): adds 2 then 0; column 1 never enters and keeps 5.0
    assert st["mask"] == 0b101
    np.testing.assert_array_equal(x, [1.0, 5.0, 2.0])


def test_max_iter_truncates(oracle):
    rng = np.random.default_rng(7)
    A, b = random_problem(rng, cond_exp=0.5)
    b = A @ np.ones(10)  # all ten columns active at the optimum: ten additions needed
    x1, s1 = oracle.inplace_fnnls(A, b, None, max_iter=3, variant=1)
    assert s1["converged"] == 0 and s1["outer"] == 3
    x2, s2 = oracle.inplace_fnnls(A, b, None, max_iter=1000, variant=1)
    assert s2["converged"] == 1
    np.testing.assert_allclose(x2, np.ones(10), rtol=1e-8)
