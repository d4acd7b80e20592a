"""Ensembles (am_batch): every member must compute exactly what a lone handle
with its own parameters computes -- same kernels, same arguments."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _members(am, n, nb, dealias, seed0):
    rng = np.random.default_rng(seed0)
    out = []
    for i in range(nb):
        alpha = float(rng.uniform(-1.0, -0.3))
        lam = float(rng.uniform(2.0, 5.0))
        p = am.make_params(n, n, 2 * math.pi, 2 * math.pi, 2.5e-4, lam, alpha, 0.01, gamma0=-0.045,
                           gamma2=2.5e-5, dealias=dealias)
        w0 = am.ic_bandlimited(n, n, 1000 + i, rms=0.5).astype(np.complex64)
        out.append((p, w0, (0.01 * i * n * n, -0.02 * n * n)))
    return out


@pytest.mark.parametrize("n,nb,dealias", [(128, 5, "half"), (128, 3, "reference"), (512, 8, "half"),
                                          (256, 4, "none")])
def test_batch_members_equal_solo_runs(am, n, nb, dealias):
    mem = _members(am, n, nb, dealias, seed0=n + nb)
    batch = am.Batch([p for p, _, _ in mem])
    for i, (_, w0, m0) in enumerate(mem):
        batch.set_state(i, w0, m0)
    e = batch.step(12)
    for i, (p, w0, m0) in enumerate(mem):
        wb, mb = batch.get_state(i)
        sim = am.Solver(n, n, p.lx, p.ly, p.dt, p.lam, p.alpha, p.beta, gamma0=p.gamma0, gamma2=p.gamma2,
                        dealias=dealias)
        sim.set_state(w0, m0)
        es = sim.step(12)
        ws, ms = sim.get_state()
        sim.close()
        assert np.array_equal(wb, ws), i
        assert np.array_equal(mb, ms), i
        assert np.array_equal(e[:, i], es), i
    batch.close()


def test_batch_mixed_pruning_and_restate(am):
    """One member with modes outside the 1/2-rule ellipse makes the whole batch
    run the full transforms; reloading it with a band-limited state prunes again.
    Results stay equal to lone handles either way."""
    n, nb = 128, 3
    mem = _members(am, n, nb, "half", seed0=7)
    full = np.fft.rfft2(np.random.default_rng(3).standard_normal((n, n))).astype(np.complex64)
    full[0, 0] = 0
    batch = am.Batch([p for p, _, _ in mem])
    states = [mem[0][1], full, mem[2][1]]
    for i in range(nb):
        batch.set_state(i, states[i], mem[i][2])
    batch.step(4)
    for rnd in range(2):
        for i, (p, _, m0) in enumerate(mem):
            wb, mb = batch.get_state(i)
            sim = am.Solver(n, n, p.lx, p.ly, p.dt, p.lam, p.alpha, p.beta, gamma0=p.gamma0, gamma2=p.gamma2,
                            dealias="half")
            sim.set_state(states[i], m0)
            sim.step(4)
            ws, _ = sim.get_state()
            sim.close()
            assert np.linalg.norm(wb - ws) / np.linalg.norm(ws) < 1e-6, (rnd, i)
        states[1] = mem[1][1]
        batch.set_state(1, states[1], mem[1][2])
        for i in (0, 2):
            batch.set_state(i, states[i], mem[i][2])
        batch.step(4)
    batch.close()


def test_batch_rejects_mismatched_grids(am):
    p1 = am.make_params(128, 128, 1.0, 1.0, 0.01, 1.0, -0.8, 0.01)
    p2 = am.make_params(256, 256, 1.0, 1.0, 0.01, 1.0, -0.8, 0.01)
    with pytest.raises(am.ActflowError):
        am.Batch([p1, p2])


@pytest.mark.parametrize("dealias", ["half", "reference"])
def test_batch_members_against_oracle(am, orc, dealias):
    """The batched kernels (blockIdx.y = member) checked directly against the
    oracle, not only against lone handles: each member of a 256^2 ensemble with
    its own lambda and alpha, 20 steps, FP32 against the FP64 oracle (2e-5, the
    short-horizon bound of the parity tests)."""
    n, nb = 256, 3
    mem = _members(am, n, nb, dealias, seed0=41)
    batch = am.Batch([p for p, _, _ in mem])
    for i, (_, w0, m0) in enumerate(mem):
        batch.set_state(i, w0, m0)
    e = batch.step(20)
    for i, (p, w0, m0) in enumerate(mem):
        wb, mb = batch.get_state(i)
        op = orc.make_params(n, n, p.lx, p.ly, p.dt, p.lam, p.alpha, p.beta, p.gamma0, p.gamma2, dealias=dealias)
        wo, mo, eo = orc.run(op, w0.astype(np.complex128), m0, 20, "f64")
        assert np.linalg.norm(wb - wo) / np.linalg.norm(wo) < 2e-5, i
        assert np.abs(mb - mo).max() <= 2e-5 * np.abs(mo).max(), i
        assert np.abs(e[:, i] - eo).max() <= 2e-5 * np.abs(eo).max(), i
    batch.close()
