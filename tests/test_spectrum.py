"""The spectrum/statistics tool against the solver's own energy (oracle) and
the reference's file formats."""
import importlib
import os

import numpy as np

spec = importlib.import_module("2d_active_matter_simulation_gb300.spectrum")
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_spectrum_sums_to_solver_energy(orc):
    d = np.load(os.path.join(GOLD, "small64.npz"))
    nx, ny = int(d["nx"]), int(d["ny"])
    p = orc.make_params(nx, ny, float(d["lx"]), float(d["ly"]), float(d["dt"]), float(d["lam"]),
                        float(d["alpha"]), float(d["beta"]))
    w, m, e = orc.run(p, d["w0"], d["mean0"], 1, "f64")
    k, E = spec.energy_spectrum(d["w0"], d["mean0"], nx, ny, float(d["lx"]), float(d["ly"]))
    assert abs(E.sum() - e[0]) <= 1e-12 * e[0]
    # the mean flow sits in the k = 0 shell
    n = nx * ny
    assert abs(E[0] - 0.5 * ((d["mean0"][0] / n) ** 2 + (d["mean0"][1] / n) ** 2)) <= 1e-12 * E.sum()


def test_spectrum_reads_reference_snapshot():
    w, m = spec.read_snapshot(os.path.join(GOLD, "format8_snap0.txt"), 8, 8)
    g = np.load(os.path.join(GOLD, "format8.npz"))
    assert np.allclose(w, g["snap0"], rtol=1e-6, atol=1e-12)
    k, E = spec.energy_spectrum(w, m, 8, 8, float(g["lx"]), float(g["ly"]))
    assert np.all(E >= 0) and k[0] == 0


def test_time_mean_energy_of_reference_file():
    t, E = spec.read_energy(os.path.join(GOLD, "format8_energy.txt"))
    assert spec.time_mean_energy(t, E) == np.mean(E)
    assert spec.time_mean_energy(t, E, t_start=0.01) == np.mean(E[1:])


def test_spectrum_rel_error():
    a = np.array([1.0, 2.0, 3.0])
    assert spec.spectrum_rel_error(a, a) == 0.0
    assert abs(spec.spectrum_rel_error(a * 1.01, a) - 0.01) < 1e-12
