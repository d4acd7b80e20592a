"""The CUDA kernel bodies executed on the CPU (tests/kernel_emu/emu.cpp: one
std::thread per CUDA thread, std::barrier for __syncthreads) against the
oracle.  Checks index arithmetic, shared-memory exchanges and the fused stage
logic without a GPU; the GPU tests then check the compiled kernels."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EMU_DIR = os.path.join(ROOT, "tests", "kernel_emu")
EMU_LIB = os.path.join(EMU_DIR, "_build", "libemu.so")
GOLD = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="session")
def emu(am):
    src = os.path.join(EMU_DIR, "emu.cpp")
    csrc = os.path.join(ROOT, "2d_active_matter_simulation_gb300", "csrc")
    deps = [src] + [os.path.join(csrc, f) for f in os.listdir(csrc) if f.endswith((".cuh", ".h"))]
    if not os.path.exists(EMU_LIB) or any(os.path.getmtime(d) > os.path.getmtime(EMU_LIB) for d in deps):
        # the harness compiles as seven translation units in parallel: the entry
        # points, five groups of row lengths and the double-float kernels (see
        # emu.cpp)
        bdir = os.path.dirname(EMU_LIB)
        os.makedirs(bdir, exist_ok=True)
        flags = ["g++", "-std=c++20", "-O2", "-pthread", "-fPIC", "-ffp-contract=off",
                 "-I" + os.path.join(ROOT, "include"), "-I" + csrc, "-c", src]
        objs, procs = [], []
        for g in [None, 0, 1, 2, 3, 4, 5]:
            obj = os.path.join(bdir, f"emu_{'main' if g is None else g}.o")
            objs.append(obj)
            procs.append(subprocess.Popen(flags + ([] if g is None else [f"-DEMU_GROUP={g}"]) + ["-o", obj]))
        assert all(p.wait() == 0 for p in procs), "emulator build failed"
        subprocess.run(["g++", "-shared", "-pthread", "-o", EMU_LIB] + objs, check=True)
    L = ctypes.CDLL(EMU_LIB)
    L.emu_run.argtypes = [ctypes.POINTER(am.Params), ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                          ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_int]
    L.emu_forward.argtypes = [ctypes.POINTER(am.Params), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    L.emu_inside_half.argtypes = [ctypes.POINTER(am.Params), ctypes.c_void_p]
    return L


def _emu_run(am, emu, p, w0, mean0, n, colvar=-1, rowvar=0):
    w = np.ascontiguousarray(w0, dtype=np.complex128 if p.precision else np.complex64).copy()
    m = np.array(mean0, dtype=np.float64)
    e = np.zeros(max(n, 1))
    r = emu.emu_run(ctypes.byref(p), w.ctypes.data, m.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n,
                    e.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), colvar, rowvar)
    assert r == -1
    return w, m, e[:n]


@pytest.mark.parametrize("name", ["format8", "small64", "rect64x32", "rect32x64"])
@pytest.mark.parametrize("prec", [0, 1])
def test_emulated_kernels_match_oracle(am, orc, emu, name, prec):
    d = np.load(os.path.join(GOLD, name + ".npz"))
    nx, ny = int(d["nx"]), int(d["ny"])
    p = am.Params(nx, ny, float(d["lx"]), float(d["ly"]), float(d["dt"]), float(d["lam"]), float(d["alpha"]),
                  float(d["beta"]), 0.0, 0.0, 0, 0, prec)
    w, m, e = _emu_run(am, emu, p, d["w0"], d["mean0"], 3)
    op = orc.make_params(nx, ny, float(d["lx"]), float(d["ly"]), float(d["dt"]), float(d["lam"]),
                         float(d["alpha"]), float(d["beta"]))
    wo, mo, eo = orc.run(op, d["w0"], d["mean0"], 3, "f64")
    tol = 1e-13 if prec else 1e-6
    assert np.linalg.norm(w - wo) / np.linalg.norm(wo) < tol
    assert np.abs(m - mo).max() <= tol * np.abs(mo).max()
    assert np.abs(e - eo).max() <= tol * np.abs(eo).max()


@pytest.mark.parametrize("dealias", ["reference", "half", "none"])
def test_emulated_general_form_and_masks(am, orc, emu, dealias):
    nx, ny = 128, 64
    w0 = am.ic_bandlimited(nx, ny, seed=9, kmax=10.0, rms=3.0)
    p = am.Params(nx, ny, 6.283185307179586, 3.141592653589793, 1e-3, 3.5, -0.8, 0.01, -0.045, 2.5e-5, 1,
                  am.DEALIAS[dealias], 1)
    w, m, e = _emu_run(am, emu, p, w0, (50.0, -20.0), 2)
    op = orc.make_params(nx, ny, 6.283185307179586, 3.141592653589793, 1e-3, 3.5, -0.8, 0.01, -0.045, 2.5e-5,
                         dealias=dealias)
    wo, mo, eo = orc.run(op, w0, (50.0, -20.0), 2, "f64")
    assert np.linalg.norm(w - wo) / np.linalg.norm(wo) < 1e-13
    assert np.abs(m - mo).max() <= 1e-13 * np.abs(mo).max()


@pytest.mark.parametrize("n", [(8, 8), (64, 32), (16, 128), (128, 128)])
@pytest.mark.parametrize("prec", [0, 1])
def test_emulated_forward_transform(am, emu, n, prec):
    nx, ny = n
    p = am.Params(nx, ny, 1.0, 1.0, 0.1, 1.0, 1.0, 1.0, 0.0, 0.0, 0, 2, prec)
    x = np.random.default_rng(nx * ny).standard_normal((ny, nx)).astype(np.float64 if prec else np.float32)
    w = np.zeros((ny, nx // 2 + 1), np.complex128 if prec else np.complex64)
    emu.emu_forward(ctypes.byref(p), x.ctypes.data, w.ctypes.data, 0)
    ref = np.fft.rfft2(x.astype(np.float64))
    assert np.abs(w - ref).max() <= (1e-14 if prec else 5e-7) * np.abs(ref).max()


@pytest.mark.parametrize("n", [(64, 64), (128, 32), (32, 128)])
@pytest.mark.parametrize("prec", [0, 1])
def test_emulated_pruned_half_rule(am, orc, emu, n, prec):
    """1/2 rule with a state inside the ellipse: the kernels skip kx > Nx/4
    (pruned transforms) and must reproduce the full-transform oracle."""
    nx, ny = n
    w0 = am.ic_bandlimited(nx, ny, seed=17, kmax=min(nx, ny) / 8.0, rms=2.0)
    kw = dict(gamma0=-0.045, gamma2=2.5e-5)
    p = am.Params(nx, ny, 6.283185307179586, 6.283185307179586, 2e-3, 3.5, -0.8, 0.01, kw["gamma0"],
                  kw["gamma2"], 1, 1, prec)
    w, m, e = _emu_run(am, emu, p, w0, (30.0, 10.0), 3)
    op = orc.make_params(nx, ny, 6.283185307179586, 6.283185307179586, 2e-3, 3.5, -0.8, 0.01, dealias="half", **kw)
    wo, mo, eo = orc.run(op, w0, (30.0, 10.0), 3, "f64")
    tol = 1e-13 if prec else 1e-6
    assert np.linalg.norm(w - wo) / np.linalg.norm(wo) < tol
    assert np.abs(e - eo).max() <= tol * np.abs(eo).max()
    mask = orc.mask(nx, ny, "half")
    assert np.abs(w[mask == 0]).max() == 0.0


@pytest.mark.parametrize("n,kind", [((2048, 16), "full"), ((2048, 16), "pruned"), ((16, 2048), "full"),
                                    ((16, 2048), "pruned"), ((4096, 8), "full"), ((8, 4096), "full"),
                                    ((512, 8), "pruned"), ((1024, 8), "full")])
@pytest.mark.parametrize("prec", [0, 1])
def test_emulated_production_lengths(am, orc, emu, n, prec, kind):
    """The row kernel at Nx = 2048 and the column kernel at Ny = 2048 (the
    benchmark's transform lengths) and at 4096 (the largest grid: the FP64 row
    pass there reuses one exchange buffer per transform, and the column pass
    runs its transforms one at a time), with few rows or columns so that the
    emulation stays quick.  A unit-variance white-noise field and dt = 1e-3
    make the nonlinear term about 1e-3 of the result, so FP64 agreement to
    1e-13 pins the nonlinear term to about 1e-10.  "pruned": the state is
    zeroed outside the 1/2-rule ellipse, so the kernels carry kx <= Nx/4 only."""
    nx, ny = n
    w0 = np.fft.rfft2(np.random.default_rng(nx + 7 * ny).standard_normal((ny, nx)))
    dealias = "half"
    if kind == "pruned":
        w0 = w0 * orc.mask(nx, ny, "half")
    p = am.Params(nx, ny, 10.0, 12.0, 1e-3, 7.0, -0.8, 0.01, 0.0, 0.0, 0, am.DEALIAS[dealias], prec)
    w, m, e = _emu_run(am, emu, p, w0, (3.0, 1.0), 3)
    op = orc.make_params(nx, ny, 10.0, 12.0, 1e-3, 7.0, -0.8, 0.01, dealias=dealias)
    wo, mo, eo = orc.run(op, w0, (3.0, 1.0), 3, "f64")
    w_lin, _, _ = orc.run(orc.make_params(nx, ny, 10.0, 12.0, 1e-3, 0.0, -0.8, 0.0, dealias=dealias), w0,
                          (3.0, 1.0), 3, "f64")
    assert np.linalg.norm(wo - w_lin) / np.linalg.norm(wo) > 1e-4   # the nonlinear term matters
    tol = 1e-13 if prec else 2e-6
    assert np.linalg.norm(w - wo) / np.linalg.norm(wo) < tol
    assert np.abs(m - mo).max() <= tol * np.abs(mo).max()
    assert np.abs(e - eo).max() <= tol * np.abs(eo).max()


@pytest.mark.parametrize("n", [(2048, 16), (2048, 8), (512, 8)])
@pytest.mark.parametrize("prec", [0, 1])
def test_emulated_pruned_rows_match_full_transforms(am, orc, emu, n, prec):
    """One band-limited state through the pruned passes and through the full
    transforms (forced by one 1e-30 mode outside the 1/2-rule ellipse).  At
    Nx = 2048 the pruned rows run as four interleaved sub-sequences (two
    512-point transforms per field) instead of one 1024-point transform, so
    the two runs differ by the rounding of the nonlinear term alone (the
    linear part is computed the same way): measured about 1e-6 of the
    nonlinear part of the step in FP32 and 1e-15 in FP64, where a 1e-4 change
    of lambda shows as 1e-4.  Nx = 512 has no such form and serves as the
    control."""
    nx, ny = n
    w0 = np.fft.rfft2(np.random.default_rng(nx + 7 * ny).standard_normal((ny, nx))) * orc.mask(nx, ny, "half")
    w0f = w0.copy()
    w0f[ny // 2, 3 * nx // 8] = 1e-30
    p = am.Params(nx, ny, 10.0, 12.0, 1e-3, 7.0, -0.8, 0.01, 0.0, 0.0, 0, am.DEALIAS["half"], prec)
    wp, _, _ = _emu_run(am, emu, p, w0, (3.0, 1.0), 3)
    wf, _, _ = _emu_run(am, emu, p, w0f, (3.0, 1.0), 3)
    wo, _, _ = orc.run(orc.make_params(nx, ny, 10.0, 12.0, 1e-3, 7.0, -0.8, 0.01, dealias="half"), w0,
                       (3.0, 1.0), 3, "f64")
    wl, _, _ = orc.run(orc.make_params(nx, ny, 10.0, 12.0, 1e-3, 0.0, -0.8, 0.0, dealias="half"), w0,
                       (3.0, 1.0), 3, "f64")
    nl = np.linalg.norm(wo - wl)
    assert nl > 1e-4 * np.linalg.norm(wo)   # the nonlinear term matters
    assert np.linalg.norm(wp - wf) < (1e-11 if prec else 1e-5) * nl


@pytest.mark.parametrize("if_factors", ["float", "double"])
@pytest.mark.parametrize("prec", [0, 1])
def test_emulated_integrating_factor_modes(am, orc, emu, if_factors, prec):
    """Both ways of forming exp(L dt) and exp(L dt / 2): per value in the
    state's precision (lin_func) and the table computed in double and rounded
    once (the precision form), each against the oracle that forms them the
    same way."""
    nx, ny = 64, 128
    w0 = am.ic_bandlimited(nx, ny, seed=23, kmax=10.0, rms=2.0)
    p = am.Params(nx, ny, 6.283185307179586, 6.283185307179586, 2e-3, 3.5, -0.8, 0.01, -0.045, 2.5e-5, 1,
                  am.DEALIAS["half"], prec, am.IF_FACTORS[if_factors])
    w, m, e = _emu_run(am, emu, p, w0, (20.0, -5.0), 3)
    op = orc.make_params(nx, ny, 6.283185307179586, 6.283185307179586, 2e-3, 3.5, -0.8, 0.01, -0.045, 2.5e-5,
                         dealias="half", if_double=if_factors == "double")
    wo, mo, eo = orc.run(op, w0 if prec else w0.astype(np.complex64), (20.0, -5.0), 3, "f64" if prec else "f32")
    tol = 1e-13 if prec else 2e-6
    assert np.linalg.norm(w - wo) / np.linalg.norm(wo) < tol
    assert np.abs(m - mo).max() <= tol * np.abs(mo).max()
    assert np.abs(e - eo).max() <= tol * np.abs(eo).max()


@pytest.mark.parametrize("n,kind", [((16, 2048), "pruned"), ((64, 128), "full"), ((16, 1024), "pruned")])
def test_emulated_radix8_column_shape(am, orc, emu, n, kind):
    """The third column-pass launch shape (wide tiles, radix-8 passes, up to
    1024 threads per CTA), FP32, at the benchmark's column length and at
    smaller ones, against the FP64 oracle."""
    nx, ny = n
    w0 = np.fft.rfft2(np.random.default_rng(nx + 5 * ny).standard_normal((ny, nx)))
    if kind == "pruned":
        w0 = w0 * orc.mask(nx, ny, "half")
    p = am.Params(nx, ny, 10.0, 12.0, 1e-3, 7.0, -0.8, 0.01, 0.0, 0.0, 0, am.DEALIAS["half"], 0)
    w, m, e = _emu_run(am, emu, p, w0, (3.0, 1.0), 3, colvar=2)
    op = orc.make_params(nx, ny, 10.0, 12.0, 1e-3, 7.0, -0.8, 0.01, dealias="half", if_double=True)
    wo, mo, eo = orc.run(op, w0, (3.0, 1.0), 3, "f64")
    assert np.linalg.norm(w - wo) / np.linalg.norm(wo) < 2e-6
    assert np.abs(m - mo).max() <= 2e-6 * np.abs(mo).max()
    assert np.abs(e - eo).max() <= 2e-6 * np.abs(eo).max()


@pytest.mark.parametrize("n,kind", [((2048, 8), "pruned"), ((1024, 8), "full"), ((4096, 8), "pruned")])
def test_emulated_radix16_row_shape(am, orc, emu, n, kind):
    """The second row-pass launch shape (radix-16 passes, transforms one after
    another with shared-memory stashes), FP32, at the benchmark's row length and
    at 1024 and 4096, against the FP64 oracle."""
    nx, ny = n
    w0 = np.fft.rfft2(np.random.default_rng(3 * nx + ny).standard_normal((ny, nx)))
    if kind == "pruned":
        w0 = w0 * orc.mask(nx, ny, "half")
    p = am.Params(nx, ny, 10.0, 12.0, 1e-3, 7.0, -0.8, 0.01, 0.0, 0.0, 0, am.DEALIAS["half"], 0)
    w, m, e = _emu_run(am, emu, p, w0, (3.0, 1.0), 3, rowvar=1)
    op = orc.make_params(nx, ny, 10.0, 12.0, 1e-3, 7.0, -0.8, 0.01, dealias="half", if_double=True)
    wo, mo, eo = orc.run(op, w0, (3.0, 1.0), 3, "f64")
    assert np.linalg.norm(w - wo) / np.linalg.norm(wo) < 2e-6
    assert np.abs(m - mo).max() <= 2e-6 * np.abs(mo).max()
    assert np.abs(e - eo).max() <= 2e-6 * np.abs(eo).max()


@pytest.mark.parametrize("n", [(8, 8), (64, 32), (128, 256), (2048, 16), (16, 2048)])
@pytest.mark.parametrize("prec", [0, 1])
def test_inside_half_mask_check(am, emu, n, prec):
    """The host check that selects pruned transforms (a per-row limit instead of
    the mask formula at every mode) against the mask itself: zero outside the
    ellipse -> inside; one nonzero value anywhere outside -> not inside."""
    nx, ny = n
    mask = np.array([[am.mask_value(nx, ny, "half", ix, iy) for ix in range(nx // 2 + 1)] for iy in range(ny)])
    p = am.Params(nx, ny, 1.0, 1.0, 0.1, 1.0, 1.0, 1.0, 0.0, 0.0, 0, 1, prec)
    dt = np.complex128 if prec else np.complex64
    rng = np.random.default_rng(nx * 7 + ny)
    w = ((rng.standard_normal(mask.shape) + 1j * rng.standard_normal(mask.shape)) * mask).astype(dt)
    assert emu.emu_inside_half(ctypes.byref(p), w.ctypes.data) == 1
    outside = np.argwhere(mask == 0)
    for iy, ix in outside[rng.choice(len(outside), size=min(20, len(outside)), replace=False)]:
        v = w.copy()
        v[iy, ix] = 1e-30 if rng.uniform() < 0.5 else 1e-30j
        assert emu.emu_inside_half(ctypes.byref(p), v.ctypes.data) == 0, (iy, ix)


@pytest.mark.parametrize("n,dealias,rowvar", [((32, 32), "reference", 0), ((64, 64), "half", 0),
                                              ((128, 32), "none", 0), ((2048, 8), "half", 0),
                                              ((2048, 8), "half", 1), ((8, 2048), "half", 0)])
def test_emulated_double_float(am, orc, emu, n, dealias, rowvar):
    """The double-float kernels (AM_DF64: two floats per real, FP32 arithmetic
    only) against the FP64 oracle, with both row shapes at Nx = 2048 (rowvar 1:
    the transforms in sequence, radix 8).  Double-float carries about 48 bits
    against double's 53; the state agrees to about 5e-15 of its norm (FP32
    would be off by 1e-7)."""
    nx, ny = n
    w0 = np.fft.rfft2(np.random.default_rng(nx + 3 * ny).standard_normal((ny, nx)))
    p = am.Params(nx, ny, 10.0, 12.0, 1e-3, 7.0, -0.8, 0.01, -0.045, 2.5e-5, 1, am.DEALIAS[dealias], am.DF64)
    w, m, e = _emu_run(am, emu, p, w0, (3.0, 1.0), 3, rowvar=rowvar)
    op = orc.make_params(nx, ny, 10.0, 12.0, 1e-3, 7.0, -0.8, 0.01, -0.045, 2.5e-5, dealias=dealias,
                         if_double=True)
    wo, mo, eo = orc.run(op, w0, (3.0, 1.0), 3, "f64")
    assert np.linalg.norm(w - wo) / np.linalg.norm(wo) < 1e-13
    assert np.abs(m - mo).max() <= 1e-13 * np.abs(mo).max()
    assert np.abs(e - eo).max() <= 1e-13 * np.abs(eo).max()
