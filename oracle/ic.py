"""Oracle-side restatement of the seeded initial vorticity fields.

TEST INFRASTRUCTURE ONLY: this module is the checker's copy of the initial-field
generators.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py`` may import it; the product generates its initial fields in C++
(``am_ic_bandlimited`` in ``csrc/actflow_api.cu``) and this file exists to
check that code.

Two generators are restated here.

* ``mt19937_64`` -- the 64-bit Mersenne Twister of Matsumoto and Nishimura
  (the engine behind ``std::mt19937_64``), written from the published
  recurrence.  The reference seeds one of these for its ``random`` initial
  condition (ActFlow_V3-2.cu:539-546).
* ``bandlimited`` -- the seeded, band-limited vorticity field used for the
  benchmark workloads (the reference's own ``random`` field is seeded from the
  wall clock, ActFlow_V3-2.cu:539-545, so it cannot be reproduced).  Modes with
  integer index vector ``(ix, iy)`` and ``kmin <= |(ix, iy)| <= kmax`` get a
  Gaussian amplitude and a uniform phase; the field is Hermitian, has zero mean
  and is scaled to a prescribed real-space rms.  Draw order: ``iy`` from
  ``-kmax`` to ``kmax`` (outer), ``ix`` from 0 to ``kmax`` (inner); on the
  ``ix == 0`` column only ``iy > 0`` is drawn and ``iy < 0`` is its conjugate.
  Per mode three 64-bit draws are taken: ``u1, u2`` give the amplitude by the
  Box-Muller transform ``sqrt(-2 ln(1-u1)) cos(2 pi u2)`` and ``u3`` the phase
  ``2 pi u3``; a draw ``x`` maps to ``u = (x >> 11) * 2**-53``.

The spectrum is stored as unnormalised DFT coefficients on the half plane,
``w_hat[iy mod Ny, ix]`` with ``ix in [0, Nx/2]`` -- the layout of the
reference's state array (cuFFT R2C output, ActFlow_V3-2.cu:507, 665) and of its
snapshot files (ActFlow_V3-2.cu:1261-1262).
"""
import math

import numpy as np

_MASK64 = (1 << 64) - 1


class MT19937_64:
    """64-bit Mersenne Twister (Matsumoto & Nishimura, 2004 reference recurrence)."""

    NN = 312
    MM = 156
    MATRIX_A = 0xB5026F5AA96619E9
    UM = 0xFFFFFFFF80000000
    LM = 0x7FFFFFFF

    def __init__(self, seed=5489):
        self.mt = [0] * self.NN
        self.mt[0] = seed & _MASK64
        for i in range(1, self.NN):
            prev = self.mt[i - 1]
            self.mt[i] = (6364136223846793005 * (prev ^ (prev >> 62)) + i) & _MASK64
        self.mti = self.NN

    def _twist(self):
        mt = self.mt
        nn, mm = self.NN, self.MM
        for i in range(nn):
            x = (mt[i] & self.UM) | (mt[(i + 1) % nn] & self.LM)
            xa = x >> 1
            if x & 1:
                xa ^= self.MATRIX_A
            mt[i] = mt[(i + mm) % nn] ^ xa
        self.mti = 0

    def __call__(self):
        if self.mti >= self.NN:
            self._twist()
        x = self.mt[self.mti]
        self.mti += 1
        x ^= (x >> 29) & 0x5555555555555555
        x ^= (x << 17) & 0x71D67FFFEDA60000
        x ^= (x << 37) & 0xFFF7EEE000000000
        x ^= x >> 43
        return x & _MASK64


def unit_draw(gen):
    """One draw in [0, 1): the top 53 bits of a 64-bit output."""
    return (gen() >> 11) * (1.0 / 9007199254740992.0)


def bandlimited(nx, ny, seed, kmin=1.0, kmax=8.0, rms=0.01, dtype=np.float64):
    """Seeded band-limited vorticity spectrum (see module docstring).

    Returns a complex array of shape ``(ny, nx//2 + 1)`` holding the
    unnormalised DFT of a real field whose real-space rms is ``rms``.
    ``dtype`` is the precision of the stored state (float32 states are
    rounded after scaling).
    """
    nxh = nx // 2 + 1
    w = np.zeros((ny, nxh), dtype=np.complex128)
    gen = MT19937_64(seed)
    km = int(math.floor(kmax))
    kmin2, kmax2 = kmin * kmin, kmax * kmax
    for iy in range(-km, km + 1):
        for ix in range(0, km + 1):
            if ix == 0 and iy <= 0:
                continue
            r2 = ix * ix + iy * iy
            if r2 < kmin2 or r2 > kmax2:
                continue
            u1 = unit_draw(gen)
            u2 = unit_draw(gen)
            u3 = unit_draw(gen)
            amp = math.sqrt(-2.0 * math.log(1.0 - u1)) * math.cos(2.0 * math.pi * u2)
            ph = 2.0 * math.pi * u3
            c = complex(amp * math.cos(ph), amp * math.sin(ph))
            w[iy % ny, ix] = c
            if ix == 0:
                w[(-iy) % ny, 0] = c.conjugate()
    # Parseval on the full plane: sum_x w^2 = (1/N) sum_k |w_hat|^2.
    n = nx * ny
    full = np.sum(np.abs(w[:, 0]) ** 2) + 2.0 * np.sum(np.abs(w[:, 1:]) ** 2)
    cur_rms = math.sqrt(full) / n
    if cur_rms > 0:
        w *= rms / cur_rms
    if dtype == np.float32:
        return w.astype(np.complex64)
    return w
