"""Pins the oracle's linear-algebra restatement.

* Known answers of the reference's own linalgebra tests: the 3x3 matrix
  [[4,-1,2],[-1,6,0],[2,0,5]] (linalgebra/tests/test_cholesky.cpp:25-27) and
  b = (3,3,4) (linalgebra/tests/test_cholesky_with_solvers.cpp:33-39).
* Bit-for-bit agreement with the reference's header-only primitives
  (linalgebra/interface/*.hpp) compiled in place (oracle/_ref), on seeded SPD
  matrices: Cholesky, forward/backward substitution, the fused row addition
  and the in-between removal.
* The reference's incremental scenarios (linalgebra/tests/
  generate_and_test_fused_impl.cpp:66-119): a 9x9 factor extended by one
  row/column equals the 10x10 factor; removing position 6 (swap with the last,
  refactor rows >= 6) equals the factor of the swapped 9x9 block.
"""
import math

import numpy as np
import pytest

KMAX = 10


def spd(rng, n, cond=1e3):
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    ev = np.geomspace(1.0, cond, n)
    M = (Q * ev) @ Q.T
    return 0.5 * (M + M.T)  # exactly symmetric


def test_cholesky_known_answer_3x3(oracle):
    M = np.array([[4.0, -1, 2], [-1, 6, 0], [2, 0, 5]])
    L = np.zeros(9)
    oracle.lib().oracle_cholesky(np.ascontiguousarray(M).ravel(), L, 3, 3)
    L = L.reshape(3, 3)
    l11 = math.sqrt(5.75)
    l21 = 0.5 / l11
    exp = np.array([[2.0, 0, 0], [-0.5, l11, 0], [1.0, l21, math.sqrt(4.0 - l21 * l21)]])
    np.testing.assert_allclose(L, exp, rtol=0, atol=4e-16)
    np.testing.assert_allclose(L @ L.T, M, rtol=0, atol=1e-14)


def test_solve_known_answer_3x3(oracle):
    M = np.array([[4.0, -1, 2], [-1, 6, 0], [2, 0, 5]])
    b = np.array([3.0, 3, 4])
    L = np.zeros(9)
    o = oracle.lib()
    o.oracle_cholesky(M.ravel().copy(), L, 3, 3)
    y = np.zeros(3)
    x = np.zeros(3)
    o.oracle_forward(L, 3, b, y, 3)
    o.oracle_backward(L, 3, y, x, 3)
    # exact solution: det(M) = 94; x = adj(M) b / det
    exact = np.linalg.solve(M.astype(np.longdouble).astype(np.float64), b)
    np.testing.assert_allclose(x, exact, rtol=1e-15, atol=1e-15)
    np.testing.assert_allclose(M @ x, b, rtol=0, atol=1e-14)


def _ref_or_skip(oracle):
    r = oracle.ref()
    if r is None:
        pytest.skip("reference tree absent: oracle/_ref not built")
    return r


@pytest.mark.parametrize("seed", range(40))
def test_bitwise_vs_reference_linalgebra(oracle, seed):
    ref = _ref_or_skip(oracle)
    o = oracle.lib()
    rng = np.random.default_rng(seed)
    n = KMAX
    M = spd(rng, n, cond=10 ** rng.uniform(0, 8)) * 10 ** rng.uniform(-3, 3)
    Mf = np.ascontiguousarray(M).ravel()
    b = rng.standard_normal(n) * 10 ** rng.uniform(-2, 4)
    for view in range(1, n + 1):
        L1 = np.zeros(n * n)
        L2 = np.zeros(n * n)
        o.oracle_cholesky(Mf.copy(), L1, n, view)
        ref.ref_cholesky_decomp(Mf.copy(), L2, n, view)
        assert np.array_equal(L1, L2), f"cholesky view={view}"
        y1, y2 = np.zeros(n), np.zeros(n)
        o.oracle_forward(L1, n, b, y1, view)
        ref.ref_forward(L2.copy(), b.copy(), y2, n, view)
        assert np.array_equal(y1[:view], y2[:view]), f"forward view={view}"
        x1, x2 = np.zeros(n), np.zeros(n)
        o.oracle_backward(L1, n, y1, x1, view)
        ref.ref_backward(L2.copy(), y2.copy(), x2, n, view)
        assert np.array_equal(x1[:view], x2[:view]), f"backward view={view}"


@pytest.mark.parametrize("seed", range(40))
def test_bitwise_incremental_vs_reference(oracle, seed):
    ref = _ref_or_skip(oracle)
    o = oracle.lib()
    rng = np.random.default_rng(1000 + seed)
    n = KMAX
    M = spd(rng, n, cond=10 ** rng.uniform(0, 6))
    Mf = np.ascontiguousarray(M).ravel()
    b = rng.standard_normal(n)
    view = int(rng.integers(2, n + 1))
    # factor of view-1, then fused addition of the last row
    L1 = np.zeros(n * n)
    o.oracle_cholesky(Mf.copy(), L1, n, view - 1)
    y1 = np.zeros(n)
    o.oracle_forward(L1, n, b, y1, view - 1)
    L2, y2, L3, y3 = L1.copy(), y1.copy(), L1.copy(), y1.copy()
    o.oracle_rc_addition(Mf.copy(), L1, n, b, y1, view)
    ref.ref_rc_addition(Mf.copy(), L2, b.copy(), y2, n, view)
    ref.ref_eigen_rc_addition(Mf.copy(), L3, b.copy(), y3, n, view)
    assert np.array_equal(L1, L2) and np.array_equal(y1[:view], y2[:view])
    assert np.array_equal(L1, L3) and np.array_equal(y1[:view], y3[:view])
    # in-between removal at a random position after a symmetric swap with the last row
    pos = int(rng.integers(0, view))
    Ms = Mf.copy()
    if pos < view - 1:
        # view_size = j keeps the reference swap clear of its elem == j defect
        ref.ref_swap_row_column(Ms, pos, view - 1, n, view - 1)
    Mo = Mf.copy()
    o.oracle_swap_sym(Mo, n, n, pos, view - 1)
    assert np.array_equal(Ms.reshape(n, n)[:view, :view], Mo.reshape(n, n)[:view, :view])
    Ms = Mo.copy()
    bs = b.copy()
    bs[[pos, view - 1]] = bs[[view - 1, pos]]
    La, ya, Lb, yb = L1.copy(), y1.copy(), L1.copy(), y1.copy()
    o.oracle_inbetween_removal(Mo, La, n, bs, ya, pos, view - 1)
    ref.ref_inbetween_removal(Ms.copy(), Lb, bs.copy(), yb, pos, n, view - 1)
    assert np.array_equal(La, Lb) and np.array_equal(ya[: view - 1], yb[: view - 1])
    Lc, yc = L1.copy(), y1.copy()
    ref.ref_eigen_inbetween_removal(Ms.copy(), Lc, bs.copy(), yc, pos, n, view - 1)
    assert np.array_equal(La, Lc) and np.array_equal(ya[: view - 1], yc[: view - 1])


@pytest.mark.parametrize("seed", range(20))
def test_rank1_addition_equals_full_factor(oracle, seed):
    """generate_and_test_fused_impl.cpp:66-86: 9x9 factor + added row == 10x10 factor (bitwise)."""
    o = oracle.lib()
    rng = np.random.default_rng(2000 + seed)
    n = KMAX
    M = spd(rng, n)
    Mf = M.ravel().copy()
    b = rng.standard_normal(n)
    L9 = np.zeros(n * n)
    o.oracle_cholesky(Mf, L9, n, n - 1)
    y = np.zeros(n)
    o.oracle_forward(L9, n, b, y, n - 1)
    o.oracle_rc_addition(Mf, L9, n, b, y, n)
    L10 = np.zeros(n * n)
    o.oracle_cholesky(Mf, L10, n, n)
    y10 = np.zeros(n)
    o.oracle_forward(L10, n, b, y10, n)
    assert np.array_equal(L9, L10)
    assert np.array_equal(y, y10)
    x = np.zeros(n)
    o.oracle_backward(L10, n, y10, x, n)
    np.testing.assert_allclose(x, np.linalg.solve(M, b), rtol=1e-9)


@pytest.mark.parametrize("seed", range(20))
def test_inbetween_removal_equals_fresh_factor(oracle, seed):
    """generate_and_test_fused_impl.cpp:90-119: remove position 6 of a 10x10."""
    o = oracle.lib()
    rng = np.random.default_rng(3000 + seed)
    n, pos = KMAX, 6
    M = spd(rng, n)
    b = rng.standard_normal(n)
    Mf = M.ravel().copy()
    L = np.zeros(n * n)
    o.oracle_cholesky(Mf, L, n, n)
    y = np.zeros(n)
    o.oracle_forward(L, n, b, y, n)
    o.oracle_swap_sym(Mf, n, n, pos, n - 1)
    bs = b.copy()
    bs[[pos, n - 1]] = bs[[n - 1, pos]]
    o.oracle_inbetween_removal(Mf, L, n, bs, y, pos, n - 1)
    Lf = np.zeros(n * n)
    o.oracle_cholesky(Mf, Lf, n, n - 1)
    Lr = L.reshape(n, n)[: n - 1, : n - 1]
    assert np.array_equal(Lr, Lf.reshape(n, n)[: n - 1, : n - 1])
    x = np.zeros(n)
    o.oracle_backward(L, n, y, x, n - 1)
    Ms = Mf.reshape(n, n)[: n - 1, : n - 1]
    np.testing.assert_allclose(x[: n - 1], np.linalg.solve(Ms, bs[: n - 1]), rtol=1e-9)


def test_reference_swap_row_column_defect(oracle):
    """linalgebra/interface/common.hpp:11-42 swaps the diagonal first and then
    runs its second loop over elem = i+1 .. view_size-1; when elem reaches j it
    overwrites M[i][j] with the new M[j][j] and M[j][j] with the old M[i][j].
    The reference's own test calls it that way (linalgebra/tests/
    generate_and_test_fused_impl.cpp:110). The FNNLS hot path swaps with Eigen
    (nnls/src/inplace_fnnls.cu:157-158) and never calls it; the oracle and the
    engine use a correct symmetric exchange."""
    ref = _ref_or_skip(oracle)
    n, i, j = 4, 1, 3
    M = np.arange(n * n, dtype=np.float64).reshape(n, n)
    M = M + M.T  # symmetric
    good = M.copy()
    good[[i, j], :] = good[[j, i], :]
    good[:, [i, j]] = good[:, [j, i]]
    Mr = M.ravel().copy()
    ref.ref_swap_row_column(Mr, i, j, n, n)
    Mr = Mr.reshape(n, n)
    assert Mr[j, j] == M[i, j] and good[j, j] == M[i, i]
    Mo = M.ravel().copy()
    oracle.lib().oracle_swap_sym(Mo, n, n, i, j)
    assert np.array_equal(Mo.reshape(n, n), good)
