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
                                        (64, 4096, "fp32"), (64, 2048, "fp64"), (128, 1024, "fp32"),
                                        (32, 128, "fp32")])
def test_column_shapes_agree(am, nx, ny, prec):
    """Every candidate the autotuner may pick gives the same step: 1e-6 in FP32
    (different radices round differently), 1e-12 in FP64."""
    old = am.column_shape(prec, ny)
    shapes = ["wide", "narrow"] + (["wide8"] if prec == "fp32" else [])
    try:
        res = {s: _run(am, nx, ny, prec, s) for s in shapes}
    finally:
        am.set_column_shape(prec, ny, old)
    tol = 1e-12 if prec == "fp64" else 1e-6
    ww, mw, ew = res["wide"]
    for s in shapes[1:]:
        wn, mn, en = res[s]
        assert np.linalg.norm(ww - wn) / np.linalg.norm(ww) < tol, s
        assert np.abs(ew - en).max() <= tol * np.abs(ew).max(), s
        assert np.abs(mw - mn).max() <= tol * np.abs(mw).max(), s


@pytest.mark.parametrize("nx,ny", [(1024, 64), (2048, 2048), (4096, 32)])
def test_row_shapes_agree(am, nx, ny):
    """Both row-pass shapes give the same step (FP32, 1e-6)."""
    old = am.row_shape("fp32", nx)
    try:
        am.set_row_shape("fp32", nx, "lockstep")
        w8, m8, e8 = _run(am, nx, ny, "fp32", am.column_shape("fp32", ny))
        am.set_row_shape("fp32", nx, "sequence")
        w16, m16, e16 = _run(am, nx, ny, "fp32", am.column_shape("fp32", ny))
    finally:
        am.set_row_shape("fp32", nx, old)
    assert np.linalg.norm(w8 - w16) / np.linalg.norm(w8) < 1e-6
    assert np.abs(e8 - e16).max() <= 1e-6 * np.abs(e8).max()
    assert np.abs(m8 - m16).max() <= 1e-6 * np.abs(m8).max()


def test_autotune_row_shape_at_2048(am):
    p = am.make_params(2048, 256, 2 * math.pi, 2 * math.pi, 2e-4, 3.5, -0.8, 0.01, gamma0=-0.045,
                       gamma2=2.5e-5, dealias="half")
    oc, orr = am.column_shape("fp32", 256), am.row_shape("fp32", 2048)
    try:
        _, _, rtimes, rchosen = am.autotune(p, nsteps=5)
        assert set(rtimes) == {"lockstep", "sequence", "lockstep-tma"} and rchosen == min(rtimes, key=rtimes.get)
    finally:
        am.set_column_shape("fp32", 256, oc)
        am.set_row_shape("fp32", 2048, orr)


def test_fp64_has_no_radix8_shape(am):
    with pytest.raises(am.ActflowError):
        am.set_column_shape("fp64", 2048, "wide8")


def test_autotune_keeps_the_faster_shape(am):
    p = am.make_params(512, 512, 2 * math.pi, 2 * math.pi, 2e-4, 3.5, -0.8, 0.01, gamma0=-0.045, gamma2=2.5e-5,
                       dealias="half")
    old = am.column_shape("fp32", 512)
    try:
        times, chosen, rtimes, rchosen = am.autotune(p, nsteps=10)
        assert set(times) == {"wide", "narrow", "wide8"} and min(times.values()) > 0
        assert chosen == min(times, key=times.get)
        # the sequence shape is built from Nx = 1024
        assert set(rtimes) == {"lockstep", "lockstep-tma"} and rchosen == min(rtimes, key=rtimes.get)
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
        if chosen == "wide8":
            # the batched and single radix-8 kernels are compiled separately under a
            # 64-register limit and may round the last bit differently
            assert np.linalg.norm(wb - ws) / np.linalg.norm(ws) < 1e-6
        else:
            assert np.array_equal(wb, ws)
    finally:
        am.set_column_shape("fp32", 512, old)


def test_double_float_shapes(am):
    """Double-float builds the seeded column shape of each length only
    (narrow below Ny = 2048, wide from it) and both row shapes from Nx = 1024
    (seeded with the sequence shape there); the autotuner times what is
    built, and the two row shapes agree."""
    with pytest.raises(am.ActflowError):
        am.set_column_shape("df64", 2048, "narrow")
    with pytest.raises(am.ActflowError):
        am.set_row_shape("df64", 512, "sequence")
    assert am.row_shape("df64", 2048) == "sequence" and am.row_shape("df64", 512) == "lockstep"
    p = am.make_params(2048, 2048, 2 * math.pi, 2 * math.pi, 2e-4, 3.5, -0.8, 0.01, gamma0=-0.045,
                       gamma2=2.5e-5, dealias="half", precision="df64")
    old = am.row_shape("df64", 2048)
    try:
        times, chosen, rtimes, rchosen = am.autotune(p, nsteps=3)
        assert set(times) == {"wide"} and chosen == "wide" and times["wide"] > 0
        assert set(rtimes) == {"lockstep", "sequence"} and rchosen == min(rtimes, key=rtimes.get)
        w0 = am.ic_bandlimited(2048, 2048, 5, rms=0.5)
        res = {}
        for shape in ("lockstep", "sequence"):
            am.set_row_shape("df64", 2048, shape)
            sim = am.Solver(2048, 2048, p.lx, p.ly, p.dt, p.lam, p.alpha, p.beta, gamma0=p.gamma0,
                            gamma2=p.gamma2, dealias="half", precision="df64")
            sim.set_state(w0)
            sim.step(4)
            res[shape] = sim.get_state()[0]
            sim.close()
        assert np.linalg.norm(res["sequence"] - res["lockstep"]) / np.linalg.norm(res["lockstep"]) < 1e-13
    finally:
        am.set_row_shape("df64", 2048, old)


@pytest.mark.parametrize("nx,ny,kind", [(2048, 2048, "pruned"), (4096, 64, "pruned"), (2048, 128, "full"),
                                        (1024, 256, "pruned"), (256, 512, "pruned"), (128, 64, "full")])
def test_tensor_map_row_fetch_is_exact(am, nx, ny, kind):
    """Row shape 2 fetches each row's inputs by tensor-map copies into shared
    memory and reads them from there (one row per CTA at 2048 and 4096,
    several below); the arithmetic is shape 0's, so the steps are bit for bit
    shape 0's.  With full transforms at 2048 the carried tiles do not fit one
    exchange buffer and shape 2 runs as shape 0; at 128 they do."""
    old = am.row_shape("fp32", nx)
    w0 = am.ic_bandlimited(nx, ny, 9, 1.0, 8.0, 0.5)
    if kind == "full":
        w0[ny // 2, 3 * nx // 8] = 1e-3   # a mode outside the 1/2-rule ellipse: no pruning
    res = {}
    try:
        for shape in ("lockstep", "lockstep-tma"):
            am.set_row_shape("fp32", nx, shape)
            sim = am.Solver(nx, ny, 2 * math.pi, 2 * math.pi * ny / nx, 1e-4, 3.5, -0.8, 0.01, gamma0=-0.045,
                            gamma2=2.5e-5, dealias="half")
            sim.set_state(w0.astype(np.complex64), (0.02 * nx * ny, -0.01 * nx * ny))
            assert sim.kx_carried == (nx // 4 if kind == "pruned" else nx // 2)
            e = sim.step(5)
            w, m = sim.get_state()
            sim.close()
            res[shape] = (w, m, e)
    finally:
        am.set_row_shape("fp32", nx, old)
    for a, b in zip(res["lockstep"], res["lockstep-tma"]):
        assert np.array_equal(a, b)
