"""Pins the oracle (CPU restatement of the reference step) before it is trusted.

Golden vectors come from the reference program itself (ActFlow_V3-2.cu built
for sm_103a and run on a GB300 by tests/golden/make_reference_golden.py from
seeded fields injected through ``initial_condition: continue``).  The reference
writes six significant digits, so agreement is bounded by ~1e-6 relative.
"""
import math

import numpy as np
import pytest

from refformat import read_energy


def _golden(name):
    import os
    return np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))


def _params(orc, d, dealias="reference"):
    return orc.make_params(int(d["nx"]), int(d["ny"]), float(d["lx"]), float(d["ly"]),
                           float(d["dt"]), float(d["lam"]), float(d["alpha"]),
                           float(d["beta"]), dealias=dealias)


def _snap_indices(d):
    return sorted(int(k[4:]) for k in d.keys()
                  if k.startswith("snap") and k[4:].isdigit())


@pytest.mark.parametrize("n", [(8, 8), (64, 32), (32, 64), (128, 128)])
@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_oracle_fft_matches_numpy(orc, n, prec):
    nx, ny = n
    rng = np.random.default_rng(nx * 7 + ny)
    x = rng.standard_normal((ny, nx))
    X = orc.rfft2(x, prec)
    tol = 2e-5 if prec == "f32" else 1e-12
    ref = np.fft.rfft2(x)
    assert np.abs(X - ref).max() <= tol * np.abs(ref).max()
    y = orc.irfft2(ref, nx, prec) / (nx * ny)
    assert np.abs(y - x).max() <= tol * np.abs(x).max() * 4


@pytest.mark.parametrize("name", ["format8", "small64", "rect64x32", "rect32x64"])
@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_oracle_matches_reference_golden(orc, name, prec):
    d = _golden(name)
    p = _params(orc, d)
    snap = int(d["snap"])
    w, m, done = d["w0"], d["mean0"], 0
    for i in _snap_indices(d):
        target = i * snap + 1
        w, m, _ = orc.run(p, w, m, target - done, prec)
        done = target
        ref = d[f"snap{i}"]
        rel = np.linalg.norm(w - ref) / np.linalg.norm(ref)
        assert rel < 5e-6, (name, i, rel)
        mref = d[f"snap{i}_mean"]
        assert np.abs(m - mref).max() <= 1e-5 * np.abs(mref).max()
    _, _, e = orc.run(p, d["w0"], d["mean0"], int(d["steps"]), prec)
    eref = d["energy"]
    assert np.abs(e - eref).max() <= 1e-5 * np.abs(eref).max()


def test_oracle_matches_reference_config0_short_horizon(orc):
    """256^2 benchmark field (reference units), 51 and 201 steps."""
    d = _golden("config0_256")
    p = _params(orc, d)
    w, m, e = orc.run(p, d["w0"], d["mean0"], 51, "f32")
    assert np.linalg.norm(w - d["snap1"]) / np.linalg.norm(d["snap1"]) < 1e-5
    w, m, e2 = orc.run(p, w, m, 150, "f32")
    assert np.linalg.norm(w - d["snap4"]) / np.linalg.norm(d["snap4"]) < 5e-5
    eref = d["energy"][:201]
    e_all = np.concatenate([e, e2])
    assert np.abs(e_all - eref).max() <= 5e-5 * np.abs(eref).max()


def test_oracle_mask512_reference_quirk(orc):
    """At 512^2 the reference's mask keeps only k=0 of the nonlinear term."""
    d = _golden("mask512")
    p = _params(orc, d)
    w, m, _ = orc.run(p, d["w0"], d["mean0"], int(d["last_index"]) + 1, "f32")
    sup = (d["support_iy"], d["support_ix"])
    ref = d["last_on_support"]
    assert np.abs(w[sup] - ref).max() <= 2e-6 * np.abs(ref).max()
    off = np.ones(w.shape, bool)
    off[sup] = False
    assert np.abs(w[off]).max() == 0.0 == float(d["last_max_off_support"])
    assert np.abs(m - d["last_mean"]).max() <= 1e-5 * np.abs(d["last_mean"]).max()


def test_mask_table(orc):
    """int32 wrap of the dealias radius (ActFlow_V3-2.cu:911): which grids keep what."""
    for n in (64, 128, 256, 384, 768):
        assert orc.mask(n, n, "reference").all(), n
    for n in (512, 1024, 2048):
        m = orc.mask(n, n, "reference")
        assert m[0, 0] == 1 and m.sum() == 1, n
    # 1/2 rule: isotropic, ix <= Nx/4, |ky| <= Ny/4
    m = orc.mask(64, 64, "half")
    assert m[0, 16] == 1 and m[0, 17] == 0 and m[16, 0] == 1 and m[17, 0] == 0
    assert m[48, 0] == 1 and m[47, 0] == 0 and m[11, 11] == 1 and m[12, 12] == 0


def test_linear_only_known_answer(orc):
    """lambda = beta = 0: w(n) = lin^n w(0) exactly, and the mean does not move."""
    nx = ny = 32
    L = 8 * math.pi
    dt = 0.01
    p = orc.make_params(nx, ny, L, L, dt, 0.0, -0.8, 0.0)
    rng = np.random.default_rng(1)
    w0 = np.fft.rfft2(rng.standard_normal((ny, nx)))
    w0[0, 0] = 0
    m0 = np.array([3.0, -2.0])
    w, m, _ = orc.run(p, w0, m0, 25, "f64")
    ky = np.fft.fftfreq(ny, 1.0 / ny)[:, None] * 2 * np.pi / L
    kx = np.arange(nx // 2 + 1)[None, :] * 2 * np.pi / L
    k2 = kx ** 2 + ky ** 2
    lin = np.exp((-(1 - k2) ** 2 + 0.8) * dt)
    assert np.allclose(w, lin ** 25 * w0, rtol=1e-12, atol=1e-12 * np.abs(w0).max())
    # The reference never multiplies the accumulated mean by exp(L(0) dt)
    # (ActFlow_V3-2.cu:729-732 copy it unchanged), so with beta = 0 it stays put.
    assert np.array_equal(m, m0)


def _mean_recurrence(m, n_pts, alpha, beta, dt, steps):
    """The reference's scalar stage pattern for the scaled mean velocity
    (ActFlow_V3-2.cu:729-732, 756-759, 778-781, 799-802, 820-821) with w = 0:
    N(a) = -beta' sum_x |a|^2 a = -beta |a|^2 a / N^2 (beta' = beta/N^3)."""
    lv = math.exp(-(1 + alpha) * dt)
    l2v = math.exp(-(1 + alpha) * dt / 2)

    def rhs(a):
        return -beta * (a[0] ** 2 + a[1] ** 2) * a / n_pts ** 2

    m = np.array(m, dtype=float)
    for _ in range(steps):
        old = m.copy()
        k1 = rhs(old)
        new = old + dt / 6 * lv * k1
        a = l2v * (old + dt / 2 * k1)
        k2 = rhs(a)
        new = new + dt / 3 * l2v * k2
        a = l2v * (old + dt / 2 * k2)
        k3 = rhs(a)
        new = new + dt / 3 * l2v * k3
        a = lv * (old + dt * k3)
        k4 = rhs(a)
        m = new + dt / 6 * k4
    return m


def test_mean_flow_only_known_answer(orc):
    """w = 0, mean != 0: w stays 0 and the mean follows the reference's scalar recurrence."""
    nx = ny = 16
    alpha, beta, dt, steps = -0.5, 0.05, 0.01, 200
    p = orc.make_params(nx, ny, 20.0, 20.0, dt, 7.0, alpha, beta)
    N = nx * ny
    m0 = np.array([1.2, -0.5]) * N
    w, m, _ = orc.run(p, np.zeros((ny, nx // 2 + 1), complex), m0, steps, "f64")
    assert np.abs(w).max() == 0.0
    ref = _mean_recurrence(m0, N, alpha, beta, dt, steps)
    assert np.allclose(m, ref, rtol=1e-12)
    assert np.linalg.norm(ref) < np.linalg.norm(m0)


def test_reference_example_is_zero_field():
    """The shipped 1024^2 example: the mask erases the random field (ActFlow_V3-2.cu:671)."""
    d = _golden("example1024")
    assert str(d["energy_txt"]) == "0.005 0\n0.01 0\n"
    assert float(d["snap0_max_abs"]) == 0.0


def test_golden_energy_text_parses():
    import os
    t, e = read_energy(os.path.join(os.path.dirname(__file__), "golden", "format8_energy.txt"))
    assert len(t) == 3 and t[0] == 0.0 and abs(t[1] - 0.01) < 1e-12
