"""Parity at the exact benchmark configuration, and the two ways of forming the
integrating factors.

The benchmark step: a 2048^2 grid on the [0, 2 pi)^2 box, the dimensional
operator (Gamma0 = -0.045, Gamma2 = 2.5e-5), lambda = 3.5, alpha = -0.8,
beta = 0.01, dt = 1e-4, the isotropic 1/2 rule with pruned transforms (the
state is band-limited, so the passes carry kx <= Nx/4), the wide column-pass
shape, seeded band-limited field (seed 7, rms 0.01).  Ten steps in FP32, FP64
and double-float against the FP64 oracle.

Tolerances: FP64 and double-float 1e-10 relative (the same arithmetic,
different summation order; double-float carries about 48 bits); FP32 2e-5
relative, the short-horizon bound the parity tests use.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 2048
L = 2 * math.pi
DT, LAM, ALPHA, BETA, G0, G2 = 1e-4, 3.5, -0.8, 0.01, -0.045, 2.5e-5


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def oracle_10(orc, am):
    w0 = am.ic_bandlimited(N, N, seed=7)
    p = orc.make_params(N, N, L, L, DT, LAM, ALPHA, BETA, G0, G2, dealias="half")
    return w0, orc.run(p, w0, (0.0, 0.0), 10, "f64")


@pytest.mark.parametrize("prec", ["fp32", "fp64", "df64"])
def test_headline_configuration_vs_oracle(am, oracle_10, prec):
    w0, (wo, mo, eo) = oracle_10
    before = am.column_shape(prec, N)
    am.set_column_shape(prec, N, "wide")
    try:
        sim = am.Solver(N, N, L, L, DT, LAM, ALPHA, BETA, gamma0=G0, gamma2=G2, dealias="half", precision=prec)
        sim.set_state(w0 if prec != "fp32" else w0.astype(np.complex64))
        assert sim.kx_carried == N // 4   # pruned transforms, as benchmarked
        e = sim.step(10)
        w, m = sim.get_state()
        sim.close()
    finally:
        am.set_column_shape(prec, N, before)
    tol = 1e-10 if prec != "fp32" else 2e-5
    assert rel(w, wo) < tol
    assert np.abs(e - eo).max() <= tol * np.abs(eo).max()
    # the mean starts at zero and stays near it: compare it on the scale of the
    # rms velocity (the stored mean is Nx*Ny*<u>; the energy is <|u|^2>/2)
    assert np.abs(m - mo).max() <= tol * N * N * math.sqrt(2 * eo[0])


@pytest.mark.parametrize("if_factors", ["float", "double"])
def test_fp32_integrating_factor_forms(am, orc, if_factors):
    """FP32 with the exponentials per value (lin_func's float exp) and from the
    table computed in double: each against the FP32 oracle that forms them the
    same way, on a strongly nonlinear 256^2 field over 40 steps."""
    n = 256
    w0 = am.ic_bandlimited(n, n, seed=12, kmin=1, kmax=20, rms=30.0)
    mean0 = (0.05 * n * n, -0.02 * n * n)
    sim = am.Solver(n, n, L, L, 2e-4, LAM, ALPHA, BETA, gamma0=G0, gamma2=G2, dealias="half",
                    if_factors=if_factors)
    sim.set_state(w0.astype(np.complex64), mean0)
    e = sim.step(40)
    w, m = sim.get_state()
    sim.close()
    p = orc.make_params(n, n, L, L, 2e-4, LAM, ALPHA, BETA, G0, G2, dealias="half",
                        if_double=if_factors == "double")
    wo, mo, eo = orc.run(p, w0.astype(np.complex64), mean0, 40, "f32")
    w64, _, _ = orc.run(orc.make_params(n, n, L, L, 2e-4, LAM, ALPHA, BETA, G0, G2, dealias="half"), w0,
                        mean0, 40, "f64")
    assert rel(wo, w64) > 1e-7   # FP32 rounding is visible at this horizon
    assert rel(w, wo) < 2e-5
    assert np.abs(e - eo).max() <= 2e-5 * np.abs(eo).max()
    assert np.abs(m - mo).max() <= 2e-5 * np.abs(mo).max()
    assert rel(w, w64) < 2e-5


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_pruned_rows_match_full_transforms(am, prec):
    """At 2048^2 the pruned rows run as four interleaved sub-sequences (two
    512-point transforms per field), the full transforms as one 1024-point
    transform per field.  The same band-limited state through both (the full
    path forced by one 1e-30 mode outside the 1/2-rule ellipse) differs by the
    rounding of the nonlinear term alone, measured against the nonlinear part
    of the step (the state minus a run without lambda and beta): an error of
    1e-5 (FP32) or 1e-11 (FP64) in the nonlinear term would fail this."""
    w0 = am.ic_bandlimited(N, N, seed=7, kmax=60.0, rms=2.0)
    if prec == "fp32":
        w0 = w0.astype(np.complex64)
    w0f = w0.copy()
    w0f[N // 2, 3 * N // 8] = 1e-30

    def run(w, lam, beta):
        sim = am.Solver(N, N, L, L, DT, lam, ALPHA, beta, gamma0=G0, gamma2=G2, dealias="half", precision=prec)
        sim.set_state(w)
        kc = sim.kx_carried
        sim.step(5)
        out = sim.get_state()[0]
        sim.close()
        return out, kc

    wp, kp = run(w0, LAM, BETA)
    wf, kf = run(w0f, LAM, BETA)
    wl, _ = run(w0, 0.0, 0.0)
    assert kp == N // 4 and kf == N // 2
    nl = np.linalg.norm(wp - wl)
    assert nl > 1e-3 * np.linalg.norm(wp)   # the nonlinear term matters
    assert np.linalg.norm(wp - wf) < (1e-5 if prec == "fp32" else 1e-11) * nl, np.linalg.norm(wp - wf) / nl
