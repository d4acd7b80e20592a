"""The four-sub-sequence form of the pruned row transforms (RowPass::quarter in
csrc/step_kernels.cuh), checked as identities in numpy, independent of the
kernels.

With only kx <= K = N/4 carried (the 1/2 rule), a real row x(n) of length N
is band-limited, and each sub-sequence x_s(m) = x(4m + s) is the real inverse
transform of length K of
    Y_s(c) = X(c) om^{cs} + conj(X(K - c) om^{(K - c)s}),   0 < c < K,
    Y_s(0) = Re X(0) + 2 Re(X(K) i^s),                      om = exp(2 pi i / N).
The kernel pairs the outputs: Z_h = Y_{2h} + i Y_{2h+1}, written for both
halves as Z_h = om^{2hc} (x + s xb) + i om^{(2h+1)c} (x - s i xb) with
x = X(c), xb = conj X(K - c), s = 1 - 2h; its inverse transform of length K
is x(4m + 2h) + i x(4m + 2h + 1).  Forward, with Z_h the transform of
p(4m + 2h) + i p(4m + 2h + 1), S_h = Z_h(k) + conj Z_h(K - k) and
D_h = Z_h(k) - conj Z_h(K - k):
    X(k) = (S_0 + om^{-k} D_0 / i + om^{-2k} S_1 + om^{-3k} D_1 / i) / 2,  k < K,
    X(K) = (S_0 - D_0 - S_1 + D_1) / 2  (at k = 0).
Transforms are unnormalised, as the kernels' (C2R: x(n) = sum_k X(k) e^{+2 pi
i k n / N} over the Hermitian extension, imaginary part of X(0) dropped)."""
import numpy as np
import pytest


def c2r_unnormalised(X, n):
    """Real inverse of the half spectrum X[0..n/2] (entries past len(X) zero),
    unnormalised, imaginary part of X(0) dropped."""
    full = np.zeros(n // 2 + 1, complex)
    full[: len(X)] = X
    full[0] = full[0].real
    return np.fft.irfft(full, n) * n


def quarter_inverse(X, n, mean=0.0):
    """x(n) from X[0..K] by the kernel's sub-sequence form; `mean` is added
    to Re X(0) as the row pass adds the mean velocity."""
    K = n // 4
    om = np.exp(2j * np.pi / n)
    c = np.arange(K)
    x = X[c].copy()
    x[0] = x[0].real + mean
    xb = np.conj(X[K - c])
    out = np.empty(n)
    for h in (0, 1):
        s = 1 - 2 * h
        Z = om ** (2 * h * c) * (x + s * xb) + 1j * om ** ((2 * h + 1) * c) * (x - s * 1j * xb)
        # c = 0: Y_s(0) = Re X(0) + 2 Re(X(K) i^s)
        x0, bx, by = x[0].real, 2 * X[K].real, 2 * X[K].imag
        Z[0] = complex(x0 + s * bx, x0 - s * by)
        z = np.fft.ifft(Z) * K
        out[2 * h::4] = z.real
        out[2 * h + 1::4] = z.imag
    return out


def quarter_forward(p):
    """X[0..K] of the real row p by the kernel's sub-sequence form."""
    n = len(p)
    K = n // 4
    om = np.exp(2j * np.pi / n)
    Z = [np.fft.fft(p[2 * h::4] + 1j * p[2 * h + 1::4]) for h in (0, 1)]
    k = np.arange(K)
    kr = (K - k) % K
    S = [Z[h][k] + np.conj(Z[h][kr]) for h in (0, 1)]
    D = [Z[h][k] - np.conj(Z[h][kr]) for h in (0, 1)]
    X = np.empty(K + 1, complex)
    X[:K] = (S[0] + om ** (-k) * D[0] / 1j + om ** (-2 * k) * S[1] + om ** (-3 * k) * D[1] / 1j) / 2
    X[K] = (S[0][0] - D[0][0] - S[1][0] + D[1][0]) / 2
    return X


@pytest.mark.parametrize("n", [32, 256, 2048])
def test_inverse_sub_sequences(n):
    rng = np.random.default_rng(n)
    K = n // 4
    X = rng.standard_normal(K + 1) + 1j * rng.standard_normal(K + 1)   # Im X(0) is dropped by both
    ref = c2r_unnormalised(X, n)
    got = quarter_inverse(X, n)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("n", [32, 256, 2048])
def test_mean_as_the_k0_mode(n):
    """Adding the mean to Re X(0) adds it to every real-space value."""
    rng = np.random.default_rng(n + 1)
    K = n // 4
    X = rng.standard_normal(K + 1) + 1j * rng.standard_normal(K + 1)
    got = quarter_inverse(X, n, mean=3.25)
    ref = c2r_unnormalised(X, n) + 3.25
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("n", [32, 256, 2048])
def test_forward_carried_outputs(n):
    rng = np.random.default_rng(n + 2)
    p = rng.standard_normal(n)
    ref = np.fft.rfft(p)[: n // 4 + 1]
    got = quarter_forward(p)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
