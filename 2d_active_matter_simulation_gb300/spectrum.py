"""Spectrum and statistics of the solver's output files (CPU, numpy).

Reads the reference program's formats -- snapshots ``ActTurb_snap{i}.bin``
(text: ``Ny*(Nx/2+1)`` pairs ``re,im,`` then the two scaled mean-velocity
components, written by save_func, ActFlow_V3-2.cu:1245-1266, read the same way
as image.py:49-52) and ``energy.txt`` (``t E`` lines, ActFlow_V3-2.cu:1268-1278)
-- and computes

* the shell-summed kinetic-energy spectrum E(k) of a snapshot, with
  E = sum_k E(k) equal to the energy the solver writes
  (sum(ux^2 + uy^2) / (2 N^3) for the scaled fields, ActFlow_V3-2.cu:1118-1127);
* the time-mean energy of an ``energy.txt`` (optionally after a start time);
* relative differences of two spectra (for precision and long-horizon checks).

Usage:
    python -m 2d_active_matter_simulation_gb300.spectrum SNAPSHOT NX NY LX LY
    (prints "k E(k)" lines)
"""
import sys

import numpy as np


def read_snapshot(path, nx, ny):
    """Return (w_hat [ny][nx//2+1] complex128, mean[2]) from a text snapshot."""
    vals = np.fromfile(path, sep=",")
    nxh = nx // 2 + 1
    n = ny * nxh
    if vals.size != 2 * n + 2:
        raise ValueError(f"{path}: {vals.size} numbers, expected {2 * n + 2}")
    w = vals[: 2 * n].view(np.complex128).reshape(ny, nxh)
    return w, vals[2 * n:].copy()


def read_energy(path):
    """Return (t, E) arrays from energy.txt."""
    d = np.loadtxt(path, ndmin=2)
    return d[:, 0], d[:, 1]


def velocity_spectra(w_hat, mean, nx, ny, lx, ly):
    """ux_hat, uy_hat (unnormalised, N-scaled as the solver stores them)."""
    nxh = nx // 2 + 1
    kx = 2 * np.pi / lx * np.arange(nxh)[None, :]
    ky = 2 * np.pi / ly * np.fft.fftfreq(ny, 1.0 / ny)[:, None]
    k2 = kx * kx + ky * ky
    k2[0, 0] = 1.0
    ux = 1j * ky * w_hat / k2
    uy = -1j * kx * w_hat / k2
    ux[0, 0] = mean[0]
    uy[0, 0] = mean[1]
    return ux, uy


def energy_spectrum(w_hat, mean, nx, ny, lx, ly, nbins=None):
    """Shell-summed energy spectrum.

    Shells are integer multiples of dk = 2 pi / max(lx, ly); bin i collects
    |k| in [(i - 1/2) dk, (i + 1/2) dk).  Returns (k_centres, E_k) with
    sum(E_k) = E (the solver's energy of this state, mean flow in bin 0)."""
    ux, uy = velocity_spectra(w_hat, mean, nx, ny, lx, ly)
    nxh = nx // 2 + 1
    n = float(nx) * ny
    # full-plane weights of the half plane (kx = 0 and the Nyquist column once)
    wt = np.full((ny, nxh), 2.0)
    wt[:, 0] = 1.0
    if nx % 2 == 0:
        wt[:, -1] = 1.0
    # The stored spectra are the unnormalised DFTs of the physical fields, so by
    # Parseval <u^2> = sum_k |u_hat|^2 / N^2 and E = <|u|^2> / 2.
    dens = wt * (np.abs(ux) ** 2 + np.abs(uy) ** 2) / (2.0 * n * n)
    kx = 2 * np.pi / lx * np.arange(nxh)[None, :]
    ky = 2 * np.pi / ly * np.fft.fftfreq(ny, 1.0 / ny)[:, None]
    kk = np.sqrt(kx * kx + ky * ky)
    dk = 2 * np.pi / max(lx, ly)
    idx = np.rint(kk / dk).astype(int)
    if nbins is None:
        nbins = int(idx.max()) + 1
    E = np.bincount(idx.ravel(), weights=dens.ravel(), minlength=nbins)[:nbins]
    return dk * np.arange(nbins), E


def time_mean_energy(t, E, t_start=None):
    sel = np.ones_like(t, bool) if t_start is None else t >= t_start
    return float(np.mean(E[sel]))


def spectrum_rel_error(Ea, Eb, kmax_bin=None):
    """max over shells of |Ea - Eb| / max(Eb) (shells up to kmax_bin)."""
    n = min(len(Ea), len(Eb)) if kmax_bin is None else kmax_bin + 1
    return float(np.max(np.abs(Ea[:n] - Eb[:n])) / np.max(np.abs(Eb[:n])))


def main(argv):
    if len(argv) != 6:
        print(__doc__)
        return 1
    path, nx, ny, lx, ly = argv[1], int(argv[2]), int(argv[3]), float(argv[4]), float(argv[5])
    w, m = read_snapshot(path, nx, ny)
    k, E = energy_spectrum(w, m, nx, ny, lx, ly)
    for a, b in zip(k, E):
        print(f"{a:.6g} {b:.6g}")
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
