"""Column-pass launch shapes and the autotuner: both shapes compute the same
step (the per-column arithmetic is identical; only the CTA-level sum of the
row sums runs in a different order), and am_autotune keeps the faster one."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(am, nx, ny, prec, shape, nsteps=4):
    am.set_column_shape(prec, ny, shape)
    L = 2 * math.pi
    sim = am.Solver(nx, ny, L, L, 2e-4, 3.5, -0.8, 0.01, gamma0=-0.045, gamma2=2.5e-5, dealias="half",
                    precision=prec)
    w0 = am.ic_bandlimited(nx, ny, seed=nx + ny, rms=0.5)
    sim.set_state(w0 if prec == "fp64" else w0.astype(np.complex64), (0.01 * nx * ny, -0.02 * nx * ny))
    e = sim.step(nsteps)
    w, m = sim.get_state()
    sim.close()
    return w, m, e


@pytest.mark.parametrize("nx,ny,prec", [(256, 256, "fp32"), (2048, 2048, "fp32"), (128, 512, "fp64"),
                                        (64, 4096, "fp32"), (64, 2048, "fp64")])
def test_column_shapes_agree(am, nx, ny, prec):
    old = am.column_shape(prec, ny)
    try:
        ww, mw, ew = _run(am, nx, ny, prec, "wide")
        wn, mn, en = _run(am, nx, ny, prec, "narrow")
    finally:
        am.set_column_shape(prec, ny, old)
    tol = 1e-12 if prec == "fp64" else 1e-6
    assert np.linalg.norm(ww - wn) / np.linalg.norm(ww) < tol
    assert np.abs(ew - en).max() <= tol * np.abs(ew).max()
    assert np.abs(mw - mn).max() <= tol * np.abs(mw).max()


def test_autotune_keeps_the_faster_shape(am):
    p = am.make_params(512, 512, 2 * math.pi, 2 * math.pi, 2e-4, 3.5, -0.8, 0.01, gamma0=-0.045, gamma2=2.5e-5,
                       dealias="half")
    old = am.column_shape("fp32", 512)
    try:
        wide, narrow, chosen = am.autotune(p, nsteps=10)
        assert wide > 0 and narrow > 0
        assert chosen == ("wide" if wide < narrow else "narrow")
        # a batch created now uses the chosen shape and still matches a lone handle
        b = am.Batch([p, p])
        w0 = am.ic_bandlimited(512, 512, 5, rms=0.5).astype(np.complex64)
        b.set_state(0, w0)
        b.set_state(1, w0)
        b.step(3)
        wb, _ = b.get_state(1)
        b.close()
        sim = am.Solver(512, 512, p.lx, p.ly, p.dt, p.lam, p.alpha, p.beta, gamma0=p.gamma0, gamma2=p.gamma2,
                        dealias="half")
        sim.set_state(w0)
        sim.step(3)
        ws, _ = sim.get_state()
        sim.close()
        assert np.array_equal(wb, ws)
    finally:
        am.set_column_shape("fp32", 512, old)
