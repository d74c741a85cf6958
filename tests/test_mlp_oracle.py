"""The CPU FP64 MLP checker itself: its exact backward matches central finite
differences of its loss, so it can judge the GPU kernels' gradients."""
import numpy as np
import pytest

from oracle import mlp_oracle as mo


def random_params(rng, scale=0.3):
    p = {}
    for name, shape in mo.LAYOUT:
        p[name] = rng.standard_normal(shape) * scale
    p["W3"][20:] = 0.0
    p["b3"][20:] = 0.0
    return p


@pytest.mark.parametrize("seed", [0, 1])
def test_fp64_backward_matches_finite_differences(seed):
    rng = np.random.default_rng(seed)
    p = random_params(rng)
    B = 16
    X = rng.standard_normal((B, 16)) * 0.5
    X[:, 12:] = 0.0
    T = np.concatenate([(rng.random((B, 10)) < 0.5).astype(float), rng.random((B, 10))], axis=1)
    loss, g = mo.loss_and_grad(p, X, T, amp_weight=0.7, quantized=False)
    flat = mo.flatten(p)
    gflat = mo.flatten(g)
    idx = rng.choice(flat.size, 60, replace=False)
    h = 1e-6
    for i in idx:
        fp, fm = flat.copy(), flat.copy()
        fp[i] += h
        fm[i] -= h
        num = (mo.loss_only(mo.unflatten(fp), X, T, 0.7) - mo.loss_only(mo.unflatten(fm), X, T, 0.7)) / (2 * h)
        assert abs(num - gflat[i]) <= 1e-6 + 1e-5 * abs(num), (i, num, gflat[i])


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7 + 2 ** -9, -3.14159, 0.0])
    r = mo.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # tie to even
    assert r[2] == 1.0 + 2 ** -6 or r[2] == 1.0 + 2 ** -7
    assert abs(r[3] - -3.140625) < 1e-12 and r[4] == 0.0
