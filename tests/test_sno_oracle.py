"""CPU checks of the surrogate network's restatement (oracle/sno_oracle.py)."""

import numpy as np

from oracle import sno_oracle as so


def _setup(seed=0, B=2, N=32, cin=4, W=6, K=3, L=2, H=5):
    rng = np.random.default_rng(seed)
    p = so.init_params(cin, W, K, L, H, rng)
    for k in p:
        if k.startswith("b"):
            p[k] = 0.1 * rng.standard_normal(p[k].shape)
    feat = rng.standard_normal((B, N, cin))
    resid = rng.standard_normal((B, N, 2))
    target = resid + 0.3 * rng.standard_normal((B, N, 2))
    F, G = so.dft_mats(N, K)
    return p, feat, resid, target, F, G


def test_truncated_dft_pair_is_the_real_fourier_projection():
    n, k = 32, 5
    F, G = so.dft_mats(n, k)
    x = np.random.default_rng(1).standard_normal(n)
    xh = np.fft.fft(x)
    np.testing.assert_allclose(F @ x, np.stack([xh[:k].real, xh[:k].imag], 1).ravel(), atol=1e-12)
    # G F projects onto the lowest k Fourier modes (a real low-pass filter)
    xl = np.fft.ifft(np.where(np.minimum(np.arange(n), n - np.arange(n)) < k, xh, 0)).real
    np.testing.assert_allclose(G @ (F @ x), xl, atol=1e-12)


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -3.14159, 1e-30, 65504.0])
    r = so.bf16(x)
    np.testing.assert_array_equal(r[:3], [1.0, 1.0, 1.0 + 2 ** -6])  # ties to even
    assert abs(r[3] + 3.14159) < 2 ** -7 * 4
    assert np.all(np.abs(r - x) <= np.abs(x) * 2 ** -8)


def test_backward_matches_finite_differences():
    so.ROUND_BF16 = False
    try:
        p, feat, resid, target, F, G = _setup()
        out, cache = so.forward(p, feat, resid, F, G)
        err, dout = so.loss(out, target)
        g = so.backward(p, cache, dout, F, G)
        rng = np.random.default_rng(7)
        eps = 1e-6
        for name in p:
            idx = tuple(rng.integers(0, s) for s in p[name].shape)
            q = {k: v.copy() for k, v in p.items()}
            q[name][idx] += eps
            lp = so.loss(so.forward(q, feat, resid, F, G)[0], target)[0].mean()
            q[name][idx] -= 2 * eps
            lm = so.loss(so.forward(q, feat, resid, F, G)[0], target)[0].mean()
            fd = (lp - lm) / (2 * eps)
            assert abs(fd - g[name][idx]) <= 1e-6 + 1e-5 * abs(fd), (name, fd, g[name][idx])
    finally:
        so.ROUND_BF16 = True
