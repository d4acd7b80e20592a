"""am_step_noalloc: the step for callers that may not allocate device memory.

Such callers (a plug-in inside a host application that owns the GPU memory
budget, a real-time loop that cannot afford cudaMalloc's synchronisation) pass
their own device buffers for the state, the mean velocity and the energies; the
library takes every intermediate buffer from one fixed device array.  These
tests call it through the C ABI twice in a row, on buffers owned by the caller,
and check it against the ordinary handle path (am_create / am_step) within the
tolerances the other GPU tests use.  The file sorts last so that a run that
stops at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(am, params, w_dev, m_dev, nsteps, e_dev, stream):
    return am.lib.am_step_noalloc(ctypes.byref(params), ctypes.c_void_p(w_dev.data_ptr()),
                                  ctypes.c_void_p(m_dev.data_ptr()), nsteps,
                                  ctypes.c_void_p(e_dev.data_ptr()) if e_dev is not None else None,
                                  ctypes.c_void_p(stream))


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("prec,nx,ny", [("fp32", 256, 128), ("fp64", 256, 128),
                                        # the largest FP32 size class, non-square (Nx*Ny = 2^18)
                                        ("fp32", 1024, 256)])
@pytest.mark.parametrize("dealias", ["reference", "half"])
def test_noalloc_matches_handle_path_two_calls(am, prec, nx, ny, dealias):
    torch = pytest.importorskip("torch")
    lx, ly, dt, lam, alpha, beta = 40.0, 20.0, 0.004, 7.0, -0.8, 0.01
    w0 = am.ic_bandlimited(nx, ny, seed=21, kmax=12.0, rms=1.0)
    mean0 = np.array([0.2 * nx * ny, -0.1 * nx * ny])
    npdt = np.complex64 if prec == "fp32" else np.complex128
    tol = 2e-5 if prec == "fp32" else 1e-10

    # the ordinary entry points
    sim = am.Solver(nx, ny, lx, ly, dt, lam, alpha, beta, dealias=dealias, precision=prec)
    sim.set_state(w0.astype(npdt), mean0)
    e1 = sim.step(7)
    w1, m1 = sim.get_state()
    e2 = sim.step(5)
    w2, m2 = sim.get_state()
    sim.close()

    # the allocation-free entry point on caller-owned device buffers
    params = am.Params(nx, ny, lx, ly, dt, lam, alpha, beta, 0.0, 0.0, am.FORM_REFERENCE, am.DEALIAS[dealias],
                       am.FP32 if prec == "fp32" else am.FP64)
    w_dev = torch.from_numpy(np.ascontiguousarray(w0.astype(npdt))).cuda()
    m_dev = torch.from_numpy(mean0.copy()).cuda()
    e_dev = torch.zeros(7, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    assert _call(am, params, w_dev, m_dev, 7, e_dev, stream) == am.AM_OK
    torch.cuda.synchronize()
    assert _rel(w_dev.cpu().numpy(), w1) < tol
    assert np.abs(m_dev.cpu().numpy() - m1).max() <= tol * np.abs(m1).max()
    assert np.abs(e_dev.cpu().numpy() - e1).max() <= tol * np.abs(e1).max()

    e_dev2 = torch.zeros(5, dtype=torch.float64, device="cuda")
    assert _call(am, params, w_dev, m_dev, 5, e_dev2, stream) == am.AM_OK
    torch.cuda.synchronize()
    assert _rel(w_dev.cpu().numpy(), w2) < tol
    assert np.abs(m_dev.cpu().numpy() - m2).max() <= tol * np.abs(m2).max()
    assert np.abs(e_dev2.cpu().numpy() - e2).max() <= tol * np.abs(e2).max()


def test_noalloc_energy_optional_and_size_limit(am):
    torch = pytest.importorskip("torch")
    nx = ny = 64
    w0 = am.ic_bandlimited(nx, ny, seed=2, kmax=6.0, rms=1.0).astype(np.complex64)
    params = am.Params(nx, ny, 16 * np.pi, 16 * np.pi, 0.005, 7.0, -0.8, 0.01, 0.0, 0.0, am.FORM_REFERENCE, 0,
                       am.FP32)
    w_dev = torch.from_numpy(w0).cuda()
    m_dev = torch.zeros(2, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    assert _call(am, params, w_dev, m_dev, 3, None, stream) == am.AM_OK
    torch.cuda.synchronize()
    sim = am.Solver(nx, ny, 16 * np.pi, 16 * np.pi, 0.005, 7.0, -0.8, 0.01)
    sim.set_state(w0)
    sim.step(3)
    w, _ = sim.get_state()
    sim.close()
    assert _rel(w_dev.cpu().numpy(), w) < 2e-5
    # a grid whose scratch exceeds the fixed array is refused, nothing is touched
    big = am.Params(1024, 1024, 1.0, 1.0, 0.01, 1.0, -0.8, 0.01, 0.0, 0.0, am.FORM_REFERENCE, 0, am.FP32)
    before = w_dev.clone()
    assert _call(am, big, w_dev, m_dev, 1, None, stream) == am.AM_ERR_UNSUPPORTED
    torch.cuda.synchronize()
    assert torch.equal(before, w_dev)


def test_noalloc_rejects_bad_parameters(am):
    """The checks of am_create: a non-positive box length or a non-finite dt is
    refused before anything is enqueued, and the caller's buffers stay as they were."""
    torch = pytest.importorskip("torch")
    nx = ny = 64
    w0 = am.ic_bandlimited(nx, ny, seed=4, kmax=6.0, rms=1.0).astype(np.complex64)
    w_dev = torch.from_numpy(w0).cuda()
    m_dev = torch.tensor([1.0, 2.0], dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for lx, ly, dt in ((0.0, 10.0, 0.005), (10.0, -1.0, 0.005), (10.0, 10.0, float("nan")),
                       (10.0, 10.0, float("inf"))):
        params = am.Params(nx, ny, lx, ly, dt, 7.0, -0.8, 0.01, 0.0, 0.0, am.FORM_REFERENCE, 0, am.FP32)
        before_w, before_m = w_dev.clone(), m_dev.clone()
        assert _call(am, params, w_dev, m_dev, 2, None, stream) == am.AM_ERR_ARG
        torch.cuda.synchronize()
        assert torch.equal(before_w, w_dev) and torch.equal(before_m, m_dev)
