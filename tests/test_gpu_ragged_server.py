"""Ragged batches (am_ragged) and the serving engine (am_server).

Both run the same kernels as a lone handle, so every run / request must give
exactly what a lone handle with its parameters gives -- alone or in the mix,
whatever else shares the GPU."""
import math
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TWO_PI = 2 * math.pi


def _run_params(am, nx, ny, rng, dealias="half"):
    """Parameters drawn like the ragged-batch workload: alpha in [-1, -0.3],
    lambda in [2, 5], beta = 0.01, Gamma0 = -0.045, Gamma2 = 2.5e-5 on the 2 pi box,
    dt = 0.1 dx / sqrt(-alpha / beta)."""
    alpha = float(rng.uniform(-1.0, -0.3))
    lam = float(rng.uniform(2.0, 5.0))
    dt = 0.1 * (TWO_PI / max(nx, ny)) / math.sqrt(-alpha / 0.01)
    return am.make_params(nx, ny, TWO_PI, TWO_PI, dt, lam, alpha, 0.01, gamma0=-0.045, gamma2=2.5e-5,
                          dealias=dealias)


def _solo(am, p, w0, m0, nsteps, precision="fp32"):
    sim = am.Solver(p.nx, p.ny, p.lx, p.ly, p.dt, p.lam, p.alpha, p.beta, gamma0=p.gamma0, gamma2=p.gamma2,
                    dealias=p.dealias, precision=precision)
    sim.set_state(w0, m0)
    e = sim.step(nsteps)
    w, m = sim.get_state()
    sim.close()
    return w, m, e


@pytest.mark.parametrize("mode", ["worklist", "per_class"])
def test_ragged_runs_equal_solo_runs(am, mode):
    """Every run equals a lone handle bit for bit, in both modes: one launch per
    pass over the size-sorted work list, and one launch per size class."""
    rng = np.random.default_rng(3)
    shapes = [(128, 128), (256, 256), (128, 128), (512, 512), (256, 128), (1024, 1024), (256, 256)]
    steps = [7, 12, 3, 12, 5, 4, 9]
    params = [_run_params(am, nx, ny, rng) for nx, ny in shapes]
    r = am.Ragged(params, steps)
    r.set_mode(mode)
    assert r.classes == 5
    ics = []
    for i, p in enumerate(params):
        w0 = am.ic_bandlimited(p.nx, p.ny, 2000 + i, rms=0.5).astype(np.complex64)
        m0 = (0.01 * i * p.nx * p.ny, -0.02 * p.nx * p.ny)
        ics.append((w0, m0))
        r.set_state(i, w0, m0)
    energies, gps = r.run()
    assert gps == sum(p.nx * p.ny * k for p, k in zip(params, steps))
    for i, p in enumerate(params):
        wr, mr = r.get_state(i)
        ws, ms, es = _solo(am, p, ics[i][0], ics[i][1], steps[i])
        assert np.array_equal(wr, ws), i
        assert np.array_equal(mr, ms), i
        assert np.array_equal(energies[i], es), i
    # a second run() has nothing left to do
    _, gps2 = r.run()
    assert gps2 == 0
    r.close()


def test_ragged_runs_against_oracle(am, orc):
    """The batched kernels of a ragged batch checked directly against the
    oracle: one run of each of three size classes (256^2, 128^2, 256x128), each
    with its own parameters, dt and step count, FP32 against the FP64 oracle
    (2e-5, the short-horizon bound of the parity tests)."""
    rng = np.random.default_rng(11)
    shapes = [(256, 256), (128, 128), (256, 128)]
    steps = [15, 20, 10]
    params = [_run_params(am, nx, ny, rng) for nx, ny in shapes]
    r = am.Ragged(params, steps)
    ics = []
    for i, p in enumerate(params):
        w0 = am.ic_bandlimited(p.nx, p.ny, 3000 + i, rms=0.5).astype(np.complex64)
        m0 = (0.02 * p.nx * p.ny, 0.01 * (i + 1) * p.nx * p.ny)
        ics.append((w0, m0))
        r.set_state(i, w0, m0)
    energies, _ = r.run()
    for i, p in enumerate(params):
        wr, mr = r.get_state(i)
        op = orc.make_params(p.nx, p.ny, p.lx, p.ly, p.dt, p.lam, p.alpha, p.beta, p.gamma0, p.gamma2,
                             dealias="half")
        wo, mo, eo = orc.run(op, ics[i][0].astype(np.complex128), ics[i][1], steps[i], "f64")
        assert np.linalg.norm(wr - wo) / np.linalg.norm(wo) < 2e-5, i
        assert np.abs(mr - mo).max() <= 2e-5 * np.abs(mo).max(), i
        assert np.abs(energies[i] - eo).max() <= 2e-5 * np.abs(eo).max(), i
    r.close()


def test_ragged_class_with_full_spectrum_run(am):
    """A run with modes outside the 1/2-rule ellipse makes its size class run
    the full transforms; every run still matches its lone handle."""
    rng = np.random.default_rng(5)
    shapes = [(128, 128), (128, 128), (256, 256)]
    steps = [6, 4, 5]
    params = [_run_params(am, nx, ny, rng) for nx, ny in shapes]
    full = np.fft.rfft2(0.3 * np.random.default_rng(9).standard_normal((128, 128))).astype(np.complex64)
    full[0, 0] = 0
    ics = [full, am.ic_bandlimited(128, 128, 11, rms=0.5).astype(np.complex64),
           am.ic_bandlimited(256, 256, 12, rms=0.5).astype(np.complex64)]
    r = am.Ragged(params, steps)
    for i in range(3):
        r.set_state(i, ics[i])
    r.run(energy=False)
    for i, p in enumerate(params):
        wr, _ = r.get_state(i)
        ws, _, _ = _solo(am, p, ics[i], (0.0, 0.0), steps[i])
        assert np.linalg.norm(wr - ws) / np.linalg.norm(ws) < 1e-6, i
    r.close()


def test_ragged_rejects_unsupported(am):
    p = am.make_params(2048, 2048, 1.0, 1.0, 1e-3, 1.0, -0.8, 0.01)
    with pytest.raises(am.ActflowError):
        am.Ragged([p], [3])
    for prec in ("fp64", "df64"):
        p = am.make_params(256, 256, 1.0, 1.0, 1e-3, 1.0, -0.8, 0.01, precision=prec)
        with pytest.raises(am.ActflowError):
            am.Ragged([p], [3])


def test_footprint_matches_handle(am):
    for nx, ny, prec in ((64, 64, "fp32"), (256, 128, "fp64"), (2048, 2048, "fp32"), (128, 512, "df64")):
        p = am.make_params(nx, ny, 1.0, 1.0, 1e-3, 1.0, -0.8, 0.01, precision=prec)
        sim = am.Solver(nx, ny, 1.0, 1.0, 1e-3, 1.0, -0.8, 0.01, precision=prec)
        assert am.footprint_bytes(p) == sim.device_bytes
        sim.close()


def _requests(am, rng, n):
    out = []
    for i in range(n):
        nx = int(rng.choice([64, 128, 256, 512]))
        prec = "fp64" if i % 8 == 3 else "df64" if i % 8 == 7 else "fp32"
        p = _run_params(am, nx, nx, rng)
        p.precision = am.PRECISIONS[prec]
        out.append((p, int(rng.integers(10, 120)), 4000 + i, prec))
    return out


def _check_against_solo(am, res, p, nsteps, seed, prec):
    w0 = am.ic_bandlimited(p.nx, p.ny, seed, 1.0, 8.0, 0.01)
    if prec == "fp32":
        w0 = w0.astype(np.complex64)
    ws, ms, es = _solo(am, p, w0, (0.0, 0.0), nsteps, precision=prec)
    assert res["status"] == am.AM_OK, res["error"]
    assert res["steps_done"] == nsteps
    assert np.array_equal(res["state"], ws)
    assert np.array_equal(res["mean"], ms)
    assert np.array_equal(res["energy"], es)


def test_server_results_equal_solo_alone_and_in_mix(am):
    """Requests of mixed grids and precisions, some submitted while others
    run, small chunks so that every request crosses chunk boundaries: each
    result equals a lone handle's, and the same request alone gives the same."""
    rng = np.random.default_rng(21)
    reqs = _requests(am, rng, 10)
    srv = am.Server(max_active=4, chunk_steps=16)
    ids = [srv.submit(p, k, seed=s) for p, k, s, _ in reqs[:6]]
    time.sleep(0.05)
    ids += [srv.submit(p, k, seed=s) for p, k, s, _ in reqs[6:]]
    results = [srv.wait(i, timeout=300) for i in ids]
    st = srv.stats()
    srv.close()
    assert st["jobs_done"] == len(reqs)
    assert st["peak_active"] <= 4
    for res, (p, k, s, prec) in zip(results, reqs):
        _check_against_solo(am, res, p, k, s, prec)
        assert res["t_submit"] <= res["t_admit"] <= res["t_done"]
    # the same request alone on a fresh server
    p, k, s, prec = reqs[3]
    srv = am.Server()
    alone = srv.wait(srv.submit(p, k, seed=s), timeout=300)
    srv.close()
    assert np.array_equal(alone["state"], results[3]["state"])
    assert np.array_equal(alone["energy"], results[3]["energy"])


def test_server_budget_serialises_admission(am):
    """A budget as large as the biggest request: admission never holds more
    than the budget (shortest first here), and every result is exact."""
    rng = np.random.default_rng(8)
    reqs = _requests(am, rng, 5)
    biggest = max(am.footprint_bytes(p) for p, _, _, _ in reqs)
    srv = am.Server(hbm_budget_bytes=biggest, max_active=8, chunk_steps=32, order="shortest")
    ids = [srv.submit(p, k, seed=s) for p, k, s, _ in reqs]
    results = [srv.wait(i, timeout=300) for i in ids]
    st = srv.stats()
    srv.close()
    assert st["peak_device_bytes"] <= biggest
    for res, (p, k, s, prec) in zip(results, reqs):
        _check_against_solo(am, res, p, k, s, prec)


def test_server_rejects_and_times_out(am):
    srv = am.Server(hbm_budget_bytes=1 << 20)
    big = am.make_params(1024, 1024, TWO_PI, TWO_PI, 1e-4, 3.5, -0.8, 0.01)
    with pytest.raises(am.ActflowError) as ei:
        srv.submit(big, 10)
    assert ei.value.status == am.AM_ERR_OOM
    odd = am.make_params(96, 96, TWO_PI, TWO_PI, 1e-4, 3.5, -0.8, 0.01)
    with pytest.raises(am.ActflowError) as ei:
        srv.submit(odd, 10)
    assert ei.value.status == am.AM_ERR_UNSUPPORTED
    srv.close()
    srv = am.Server()
    p = am.make_params(256, 256, TWO_PI, TWO_PI, 1e-4, 3.5, -0.8, 0.01, gamma0=-0.045, gamma2=2.5e-5,
                       dealias="half")
    jid = srv.submit(p, 3000, seed=1, want_state=False)
    with pytest.raises(am.ActflowError) as ei:
        srv.wait(jid, timeout=1e-4)
    assert ei.value.status == am.AM_ERR_TIMEOUT
    res = srv.wait(jid, timeout=300)
    assert res["status"] == am.AM_OK and res["steps_done"] == 3000 and res["state"] is None
    srv.close()


def test_server_reports_nan(am):
    p = am.make_params(64, 64, TWO_PI, TWO_PI, 1e-4, 3.5, -0.8, 0.01)
    w = am.ic_bandlimited(64, 64, 3, rms=0.5).astype(np.complex64)
    w[0, 0] = np.nan
    srv = am.Server(chunk_steps=8)
    res = srv.wait(srv.submit(p, 40, w_hat=w), timeout=300)
    srv.close()
    assert res["status"] == am.AM_ERR_NAN
    assert "NaN" in res["error"]


def test_server_small_request_overtakes_large_one(am):
    """Continuous batching: a small request submitted while a large one runs
    is admitted into a free slot and, on a higher-priority stream, finishes
    first instead of queueing behind it."""
    big = am.make_params(2048, 2048, TWO_PI, TWO_PI, 1e-4, 3.5, -0.8, 0.01, gamma0=-0.045, gamma2=2.5e-5,
                         dealias="half")
    small = am.make_params(64, 64, TWO_PI, TWO_PI, 1e-3, 3.5, -0.8, 0.01, gamma0=-0.045, gamma2=2.5e-5,
                           dealias="half")
    srv = am.Server(max_active=4)
    jb = srv.submit(big, 3000, seed=1, want_state=False, want_energy=False)
    time.sleep(0.2)
    js = srv.submit(small, 20, seed=2)
    rs = srv.wait(js, timeout=300)
    rb = srv.wait(jb, timeout=300)
    srv.close()
    assert rs["status"] == am.AM_OK and rb["status"] == am.AM_OK
    assert rs["t_done"] < rb["t_done"]
    assert rs["t_admit"] < rb["t_done"]


def test_server_fp64_lane(am):
    """FP64 requests have a lane of their own: with one FP64 slot, the second
    and third FP64 requests wait for the first to finish, while an FP32 request
    submitted after them is admitted at once; every result is exact."""
    p64 = am.make_params(512, 512, TWO_PI, TWO_PI, 1e-4, 3.5, -0.8, 0.01, gamma0=-0.045, gamma2=2.5e-5,
                         dealias="half", precision="fp64")
    p32 = am.make_params(256, 256, TWO_PI, TWO_PI, 1e-4, 3.5, -0.8, 0.01, gamma0=-0.045, gamma2=2.5e-5,
                         dealias="half")
    srv = am.Server(max_active=8, max_active_fp64=1, chunk_steps=32)
    j64 = [srv.submit(p64, 300, seed=10 + i) for i in range(3)]
    j32 = srv.submit(p32, 50, seed=20)
    r64 = [srv.wait(j, timeout=300) for j in j64]
    r32 = srv.wait(j32, timeout=300)
    st = srv.stats()
    srv.close()
    assert all(r["status"] == am.AM_OK for r in r64) and r32["status"] == am.AM_OK
    # one FP64 request at a time
    assert r64[1]["t_admit"] >= r64[0]["t_done"] - 1e-3
    assert r64[2]["t_admit"] >= r64[1]["t_done"] - 1e-3
    # the FP32 request did not queue behind the waiting FP64 ones
    assert r32["t_admit"] < r64[0]["t_done"]
    assert st["peak_active"] <= 2
    _check_against_solo(am, r32, p32, 50, 20, "fp32")
    _check_against_solo(am, r64[2], p64, 300, 12, "fp64")
