"""GPU parity: the sm_103a solver (through the C ABI) against the oracle and
against the reference program's own outputs (golden fixtures).

Tolerances: FP64 runs must agree with the FP64 oracle to 1e-11 relative (both
compute the same arithmetic; only summation order differs), and so must
double-float runs (AM_DF64: about 48 significant bits, agreement near 1e-14).  FP32 runs agree
with the FP32/FP64 oracle to a few 1e-6 relative over short horizons (FP32
rounding of two different FFT algorithms), and with the reference's six-digit
text outputs to the same level.
"""
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _golden(name):
    return np.load(os.path.join(GOLD, name + ".npz"))


def _solver(am, d, prec, dealias="reference"):
    return am.Solver(int(d["nx"]), int(d["ny"]), float(d["lx"]), float(d["ly"]), float(d["dt"]),
                     float(d["lam"]), float(d["alpha"]), float(d["beta"]), dealias=dealias, precision=prec)


def _oparams(orc, d, dealias="reference"):
    return orc.make_params(int(d["nx"]), int(d["ny"]), float(d["lx"]), float(d["ly"]), float(d["dt"]),
                           float(d["lam"]), float(d["alpha"]), float(d["beta"]), dealias=dealias)


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("name", ["format8", "small64", "rect64x32", "rect32x64"])
@pytest.mark.parametrize("prec", ["fp32", "fp64", "df64"])
def test_gpu_matches_oracle(am, orc, name, prec):
    d = _golden(name)
    n = int(d["steps"])
    sim = _solver(am, d, prec)
    sim.set_state(d["w0"], d["mean0"])
    e = sim.step(n)
    w, m = sim.get_state()
    sim.close()
    wo, mo, eo = orc.run(_oparams(orc, d), d["w0"], d["mean0"], n, "f64" if prec != "fp32" else "f32")
    tol = 1e-11 if prec != "fp32" else 5e-6
    assert rel(w, wo) < tol
    assert np.abs(m - mo).max() <= tol * np.abs(mo).max()
    assert np.abs(e - eo).max() <= tol * np.abs(eo).max()


@pytest.mark.parametrize("name", ["format8", "small64", "rect64x32", "rect32x64"])
def test_gpu_matches_reference_golden(am, name):
    """FP32 solver against the reference program's snapshots and energy file."""
    d = _golden(name)
    snap = int(d["snap"])
    sim = _solver(am, d, "fp32")
    sim.set_state(d["w0"], d["mean0"])
    done = 0
    energies = []
    idx = sorted(int(k[4:]) for k in d.keys() if k.startswith("snap") and k[4:].isdigit())
    for i in idx:
        target = i * snap + 1
        energies.append(sim.step(target - done))
        done = target
        w, m = sim.get_state()
        ref = d[f"snap{i}"]
        assert rel(w, ref) < 5e-6, (i, rel(w, ref))
        mref = d[f"snap{i}_mean"]
        assert np.abs(m - mref).max() <= 1e-5 * np.abs(mref).max()
    e = np.concatenate(energies)
    eref = d["energy"][: len(e)]
    assert np.abs(e - eref).max() <= 1e-5 * np.abs(eref).max()
    sim.close()


def test_gpu_config0_short_horizon_vs_reference(am):
    """256^2 benchmark field in reference units: 51 and 201 steps against the
    reference's snapshots; the energy series over 201 steps."""
    d = _golden("config0_256")
    sim = _solver(am, d, "fp32")
    sim.set_state(d["w0"], d["mean0"])
    e1 = sim.step(51)
    w, _ = sim.get_state()
    assert rel(w, d["snap1"]) < 1e-5
    e2 = sim.step(150)
    w, _ = sim.get_state()
    assert rel(w, d["snap4"]) < 5e-5
    e = np.concatenate([e1, e2])
    eref = d["energy"][:201]
    assert np.abs(e - eref).max() <= 5e-5 * np.abs(eref).max()
    sim.close()


def test_gpu_mask512_reference_quirk(am):
    """512^2 with the reference mask: only k=0 of the nonlinear term survives."""
    d = _golden("mask512")
    sim = _solver(am, d, "fp32")
    sim.set_state(d["w0"], d["mean0"])
    sim.step(int(d["last_index"]) + 1)
    w, m = sim.get_state()
    sup = (d["support_iy"], d["support_ix"])
    ref = d["last_on_support"]
    assert np.abs(w[sup] - ref).max() <= 2e-6 * np.abs(ref).max()
    off = np.ones(w.shape, bool)
    off[sup] = False
    assert np.abs(w[off]).max() == 0.0
    assert np.abs(m - d["last_mean"]).max() <= 1e-5 * np.abs(d["last_mean"]).max()
    sim.close()


@pytest.mark.parametrize("n", [(256, 256), (512, 128), (128, 512), (1024, 1024), (2048, 64), (64, 2048),
                               (4096, 64), (64, 4096)])
@pytest.mark.parametrize("prec", ["fp32", "fp64", "df64"])
@pytest.mark.parametrize("dealias", ["reference", "half"])
def test_gpu_sizes_vs_oracle(am, orc, n, prec, dealias):
    nx, ny = n
    L = 2 * math.pi * nx / 16
    w0 = am.ic_bandlimited(nx, ny, seed=nx + ny, kmin=1, kmax=8, rms=1.0)
    mean0 = (0.1 * nx * ny, 0.05 * nx * ny)
    sim = am.Solver(nx, ny, L, L * ny / nx, 0.005, 7.0, -0.8, 0.01, dealias=dealias, precision=prec)
    sim.set_state(w0, mean0)
    e = sim.step(3)
    w, m = sim.get_state()
    sim.close()
    p = orc.make_params(nx, ny, L, L * ny / nx, 0.005, 7.0, -0.8, 0.01, dealias=dealias)
    wo, mo, eo = orc.run(p, w0, mean0, 3, "f64")
    tol = 1e-10 if prec != "fp32" else 2e-5
    assert rel(w, wo) < tol
    assert np.abs(e - eo).max() <= tol * np.abs(eo).max()
    assert np.abs(m - mo).max() <= tol * np.abs(mo).max()


@pytest.mark.parametrize("prec", ["fp32", "fp64", "df64"])
def test_gpu_general_operator_vs_oracle(am, orc, prec):
    """Dimensional form L(k) = -alpha - Gamma0 k^2 - Gamma2 k^4 on the 2 pi box."""
    nx = ny = 256
    L = 2 * math.pi
    w0 = am.ic_bandlimited(nx, ny, seed=42)
    kw = dict(gamma0=-0.045, gamma2=2.5e-5)
    sim = am.Solver(nx, ny, L, L, 5e-4, 3.5, -0.8, 0.01, dealias="half", precision=prec, **kw)
    sim.set_state(w0, (0.0, 0.0))
    e = sim.step(20)
    w, m = sim.get_state()
    sim.close()
    p = orc.make_params(nx, ny, L, L, 5e-4, 3.5, -0.8, 0.01, dealias="half", **kw)
    wo, mo, eo = orc.run(p, w0, (0.0, 0.0), 20, "f64")
    tol = 1e-10 if prec != "fp32" else 2e-5
    assert rel(w, wo) < tol
    assert np.abs(e - eo).max() <= tol * np.abs(eo).max()


@pytest.mark.parametrize("prec", ["fp32", "fp64", "df64"])
def test_gpu_set_state_real_matches_numpy(am, prec):
    """Fresh-start processing: R2C, mask and w(0,0) = 0 (ActFlow_V3-2.cu:660-679)."""
    nx, ny = 128, 64
    x = np.random.default_rng(3).uniform(-1, 1, (ny, nx))
    sim = am.Solver(nx, ny, 30.0, 15.0, 0.01, 7.0, -0.8, 0.01, precision=prec)
    sim.set_state_real(x, (0.0, 0.0), True)
    w, m = sim.get_state()
    sim.close()
    ref = np.fft.rfft2(x)
    ref[0, 0] = 0
    tol = 1e-12 if prec != "fp32" else 3e-6
    assert np.abs(w - ref).max() <= tol * np.abs(ref).max()


def test_gpu_reference_mask_erases_1024_random_field(am):
    """The reference example: at 1024^2 the mask keeps only k=0, so a random
    field becomes zero and stays zero, energy exactly 0."""
    sim = am.Solver(1024, 1024, 628.3185307, 628.3185307, 0.005, 7.0, -0.8, 0.01, precision="fp32")
    x = np.random.default_rng(1).uniform(-1, 1, (1024, 1024))
    sim.set_state_real(x, (0.0, 0.0), True)
    w, _ = sim.get_state()
    assert np.abs(w).max() == 0.0
    e = sim.step(2)
    assert np.all(e == 0.0)
    sim.close()


def test_gpu_nan_is_reported(am):
    """A NaN in w(0,0) stops the run with AM_ERR_NAN and the step index."""
    nx = ny = 32
    w0 = am.ic_bandlimited(nx, ny, seed=1, kmax=4.0, rms=1.0).astype(np.complex64)
    w0[0, 0] = np.nan
    sim = am.Solver(nx, ny, 30.0, 30.0, 0.01, 7.0, -0.8, 0.01)
    sim.set_state(w0, (0.0, 0.0))
    with pytest.raises(am.ActflowError) as ei:
        sim.step(5)
    assert ei.value.status == am.AM_ERR_NAN
    assert "step 0" in str(ei.value)
    sim.close()


def test_gpu_step_async_matches_step(am):
    nx = ny = 128
    w0 = am.ic_bandlimited(nx, ny, seed=5, rms=1.0)
    a = am.Solver(nx, ny, 50.0, 50.0, 0.005, 7.0, -0.8, 0.01)
    b = am.Solver(nx, ny, 50.0, 50.0, 0.005, 7.0, -0.8, 0.01)
    a.set_state(w0)
    b.set_state(w0)
    a.step(10)
    b.step_async(10)
    b.sync()
    wa, ma = a.get_state()
    wb, mb = b.get_state()
    assert np.array_equal(wa, wb) and np.array_equal(ma, mb)
    a.close()
    b.close()


@pytest.mark.parametrize("prec", ["fp32", "fp64", "df64"])
def test_gpu_half_rule_state_outside_ellipse(am, orc, prec):
    """A state with modes outside the 1/2-rule ellipse runs the full transforms
    (the pruned path needs zeros there) and still matches the oracle; the modes
    outside decay by the integrating factor alone."""
    nx, ny = 128, 64
    w0 = np.fft.rfft2(np.random.default_rng(8).standard_normal((ny, nx)))
    w0[0, 0] = 0
    sim = am.Solver(nx, ny, 40.0, 20.0, 0.004, 7.0, -0.8, 0.01, dealias="half", precision=prec)
    sim.set_state(w0, (20.0, -5.0))
    e = sim.step(4)
    w, m = sim.get_state()
    sim.close()
    p = orc.make_params(nx, ny, 40.0, 20.0, 0.004, 7.0, -0.8, 0.01, dealias="half")
    wo, mo, eo = orc.run(p, w0, (20.0, -5.0), 4, "f64")
    tol = 1e-10 if prec != "fp32" else 2e-5
    assert rel(w, wo) < tol
    assert np.abs(e - eo).max() <= tol * np.abs(eo).max()


def test_gpu_pruned_state_stays_inside_ellipse(am):
    """Pruned transforms: a band-limited state under the 1/2 rule keeps exact
    zeros outside the ellipse after many steps."""
    nx = ny = 256
    w0 = am.ic_bandlimited(nx, ny, seed=4, kmax=30.0, rms=0.5)
    sim = am.Solver(nx, ny, 2 * math.pi, 2 * math.pi, 2e-4, 3.5, -0.8, 0.01, gamma0=-0.045, gamma2=2.5e-5,
                    dealias="half")
    sim.set_state(w0)
    sim.step(50)
    w, _ = sim.get_state()
    sim.close()
    mask = np.array([[am.mask_value(nx, ny, "half", ix, iy) for ix in range(nx // 2 + 1)] for iy in range(ny)])
    assert np.abs(w[mask == 0]).max() == 0.0
    assert np.abs(w[mask == 1]).max() > 0.0


@pytest.mark.parametrize("prec", ["fp32", "fp64", "df64"])
def test_gpu_largest_grid_vs_oracle(am, orc, prec):
    """The largest supported grid, 4096^2, both passes at full length, 2 steps
    of the 1/2-rule step against the FP64 oracle."""
    n = 4096
    L = 2 * math.pi
    w0 = am.ic_bandlimited(n, n, seed=5, kmin=1, kmax=8, rms=0.5)
    mean0 = (0.01 * n * n, -0.02 * n * n)
    sim = am.Solver(n, n, L, L, 1e-4, 3.5, -0.8, 0.01, gamma0=-0.045, gamma2=2.5e-5, dealias="half", precision=prec)
    sim.set_state(w0 if prec != "fp32" else w0.astype(np.complex64), mean0)
    e = sim.step(2)
    w, m = sim.get_state()
    sim.close()
    p = orc.make_params(n, n, L, L, 1e-4, 3.5, -0.8, 0.01, -0.045, 2.5e-5, dealias="half")
    wo, mo, eo = orc.run(p, w0, mean0, 2, "f64")
    tol = 1e-10 if prec != "fp32" else 2e-5
    assert rel(w, wo) < tol
    assert np.abs(e - eo).max() <= tol * np.abs(eo).max()
    assert np.abs(m - mo).max() <= tol * np.abs(mo).max()


def test_gpu_zero_steps_leave_the_state(am):
    """nsteps = 0 through every entry point: nothing advances, nothing fails."""
    n = 64
    w0 = am.ic_bandlimited(n, n, seed=3, rms=0.5).astype(np.complex64)
    sim = am.Solver(n, n, 2 * math.pi, 2 * math.pi, 1e-3, 3.5, -0.8, 0.01, dealias="half")
    sim.set_state(w0, (1.0, 2.0))
    assert len(sim.step(0)) == 0
    w, m = sim.get_state()
    sim.close()
    assert np.array_equal(w, w0) and np.array_equal(m, [1.0, 2.0])
    p = am.make_params(128, 128, 2 * math.pi, 2 * math.pi, 1e-3, 3.5, -0.8, 0.01, dealias="half")
    r = am.Ragged([p, p], [0, 3])
    wr = am.ic_bandlimited(128, 128, seed=4, rms=0.5).astype(np.complex64)
    r.set_state(0, wr)
    r.set_state(1, wr)
    energies, gps = r.run()
    assert gps == 3 * 128 * 128 and len(energies[0]) == 0 and len(energies[1]) == 3
    assert np.array_equal(r.get_state(0)[0], wr) and not np.array_equal(r.get_state(1)[0], wr)
    r.close()
    srv = am.Server()
    res = srv.wait(srv.submit(p, 0, seed=9), timeout=60)
    srv.close()
    assert res["status"] == am.AM_OK and res["steps_done"] == 0
    w9 = am.ic_bandlimited(128, 128, 9, 1.0, 8.0, 0.01).astype(np.complex64)
    assert np.array_equal(res["state"], w9)


@pytest.mark.parametrize("prec", ["fp32", "fp64", "df64"])
def test_gpu_pruning_choice_on_the_device(am, prec):
    """set_state checks on the device, in the tile kernel, whether the state
    is zero outside the 1/2-rule ellipse (pruned transforms) -- the same
    decision as the host check: a negative zero outside still counts as zero,
    one nonzero mode outside (or a NaN) turns pruning off."""
    nx, ny = 256, 128
    w0 = am.ic_bandlimited(nx, ny, seed=3, kmax=10.0, rms=1.0)
    w0 = w0 if prec != "fp32" else w0.astype(np.complex64)
    sim = am.Solver(nx, ny, 2 * math.pi, 2 * math.pi, 1e-4, 3.5, -0.8, 0.01, gamma0=-0.045, gamma2=2.5e-5,
                    dealias="half", precision=prec)
    sim.set_state(w0)
    assert sim.kx_carried == nx // 4
    w = w0.copy()
    w[5, nx // 2 - 3] = complex(-0.0, -0.0)
    sim.set_state(w)
    assert sim.kx_carried == nx // 4
    for val in (1e-30, complex(0.0, 2.0), complex(float("nan"), 0.0)):
        w = w0.copy()
        w[ny // 2, 3 * nx // 8] = val
        sim.set_state(w)
        assert sim.kx_carried == nx // 2, val
    sim.close()


@pytest.mark.parametrize("if_factors", ["float", "double"])
def test_gpu_double_float_integrating_factor_forms(am, orc, if_factors):
    """Double-float with the integrating factors per value (exp in double on
    the device, split once) and from the double table: both against the FP64
    oracle, which forms them in double."""
    n = 128
    w0 = am.ic_bandlimited(n, n, seed=31, kmin=1, kmax=20, rms=5.0)
    mean0 = (0.05 * n * n, -0.02 * n * n)
    sim = am.Solver(n, n, 2 * math.pi, 2 * math.pi, 2e-4, 3.5, -0.8, 0.01, gamma0=-0.045, gamma2=2.5e-5,
                    dealias="half", precision="df64", if_factors=if_factors)
    sim.set_state(w0, mean0)
    e = sim.step(20)
    w, m = sim.get_state()
    sim.close()
    p = orc.make_params(n, n, 2 * math.pi, 2 * math.pi, 2e-4, 3.5, -0.8, 0.01, -0.045, 2.5e-5, dealias="half",
                        if_double=if_factors == "double")
    wo, mo, eo = orc.run(p, w0, mean0, 20, "f64")
    assert rel(w, wo) < 1e-11
    assert np.abs(e - eo).max() <= 1e-11 * np.abs(eo).max()
    assert np.abs(m - mo).max() <= 1e-11 * np.abs(mo).max()
