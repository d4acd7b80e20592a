"""Time the reference program itself (its cuFFT build, ``_ref/bin/ActFlow_ref``)
on the benchmark's grid, and the cuFFT floor (``_ref/bin/cufft_floor``).

The reference has no API but its command line: ``ActFlow_ref <dir>`` reads
``<dir>/specifications.txt``, and with ``initial_condition: continue`` resumes
from the text snapshot ``ActTurb_snap0.bin`` (ActFlow_V3-2.cu:567-647).  Its own
clock spans the time loop including the snapshots it writes and its clean-up
(ActFlow_V3-2.cu:713, 873-876).  Two runs of different lengths from the same
field (30 and 30 + K steps, snapshots only at the start and the end of each)
cancel every fixed cost; the difference of their loop times over K is the
reference's time per step, energy file writes included as in the reference.

The initial field is a seeded band-limited vorticity field (modes
1 <= |k| <= 8, rms 0.01 on the 2 pi box) mapped onto the reference's
normalised units (length l = sqrt(-2 Gamma2 / Gamma0), time tau = l^4 / Gamma2;
omega_ref = tau omega).  The reference's 2048^2 dealias radius wraps to 0 in
32-bit arithmetic (ActFlow_V3-2.cu:911), so it advances the field linearly, but
it does all of its work: the timing does not depend on the mask.
"""
import json
import math
import os
import shutil
import subprocess
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BIN = os.path.join(HERE, "_ref", "bin")
REF_BIN = os.path.join(BIN, "ActFlow_ref")
FLOOR_BIN = os.path.join(BIN, "cufft_floor")

GAMMA0, GAMMA2 = -0.045, 2.5e-5
ELL = math.sqrt(-2.0 * GAMMA2 / GAMMA0)
TAU = ELL ** 4 / GAMMA2


def reference_units(alpha, beta, dt):
    """(alpha, beta, box length, dt) of the reference's normalised equation."""
    return TAU * alpha - 1.0, beta * ELL * ELL / TAU, 2.0 * math.pi / ELL, dt / TAU


def seeded_field(n, seed=7, kmax=8, rms=0.01):
    """Band-limited Hermitian half-plane spectrum [n][n/2+1] with real-space rms `rms`."""
    rng = np.random.default_rng(seed)
    nxh = n // 2 + 1
    w = np.zeros((n, nxh), np.complex128)
    for iy in range(-kmax, kmax + 1):
        for ix in range(0, kmax + 1):
            if (ix == 0 and iy <= 0) or not (1 <= ix * ix + iy * iy <= kmax * kmax):
                continue
            v = rng.standard_normal() * np.exp(2j * np.pi * rng.uniform())
            w[iy % n, ix] = v
            if ix == 0:
                w[(-iy) % n, 0] = np.conj(v)
    full = np.sum(np.abs(w) ** 2) * 2 - np.sum(np.abs(w[:, 0]) ** 2)
    return w * (rms / (math.sqrt(full) / (n * n)))


def _write_inputs(d, n, steps, lam=3.5, alpha=-0.8, beta=0.01, dt=1e-4):
    a_r, b_r, L_r, dt_r = reference_units(alpha, beta, dt)
    T = (steps - 1) * dt_r   # resuming at m = 0 runs m = 0..M, M + 1 steps
    spec = [("T", "%.9g" % T), ("dt", "%.9g" % dt_r), ("Lx", "%.9g" % L_r), ("Ly", "%.9g" % L_r), ("Nx", n),
            ("Ny", n), ("lambda", "%.9g" % lam), ("alpha", "%.9g" % a_r), ("beta", "%.9g" % b_r),
            ("dt_snap", "%.9g" % T), ("initial_condition", "continue"), ("save_directory", d)]
    with open(os.path.join(d, "specifications.txt"), "w") as f:
        f.write("\n".join(f"{k}:\n{v}" for k, v in spec) + "\n")


def _write_snapshot(path, w):
    """Text snapshot: re,im, pairs in [iy][ix] order, then the mean (0,0);
    nine significant digits so that the float values round-trip exactly."""
    v = np.asarray(w, np.complex64).reshape(-1)
    flat = np.empty(2 * v.size, np.float64)
    flat[0::2], flat[1::2] = v.real, v.imag
    with open(path, "w") as f:
        f.write(",".join(np.char.mod("%.9g", flat).tolist()))
        f.write(",0,0")


def _run(d, n, steps, w, timeout):
    for name in os.listdir(d):
        os.remove(os.path.join(d, name))
    _write_inputs(d, n, steps)
    _write_snapshot(os.path.join(d, "ActTurb_snap0.bin"), w)
    t0 = time.perf_counter()
    p = subprocess.run([REF_BIN, d], capture_output=True, text=True, timeout=timeout)
    wall = time.perf_counter() - t0
    if p.returncode != 0:
        raise RuntimeError(f"reference exited {p.returncode}: {(p.stdout + p.stderr)[-500:]}")
    for line in p.stdout.splitlines():
        if "finished successfully after" in line:
            return float(line.split("after")[1].strip().rstrip(".").rstrip("s")), wall
    raise RuntimeError("reference printed no loop time")


def time_reference(n=2048, steps=200, base=30, timeout=900):
    """The reference's seconds per step on an n^2 grid (difference of two runs)."""
    if not os.path.exists(REF_BIN):
        return {"unavailable": "reference program not built (baseline/_ref/bin/ActFlow_ref)"}
    w = seeded_field(n) * TAU
    d = tempfile.mkdtemp(prefix="actflow_ref_")
    try:
        short, _ = _run(d, n, base, w, timeout)
        long_, wall = _run(d, n, base + steps, w, timeout)
    finally:
        shutil.rmtree(d, ignore_errors=True)
    per = (long_ - short) / steps
    return {"value": n * n / per, "unit": "grid-point-steps/s", "ms_per_step": 1e3 * per,
            "steps_timed": steps, "loop_s": [short, long_],
            "how": f"reference program (cuFFT, FP32, unmodified ActFlow_V3-2.cu) on {n}^2 through "
                   f"initial_condition: continue; its own loop clock, ({base}+{steps} steps) - ({base} steps)"}


def time_floor(n=2048, steps=200, warmup=10, timeout=600):
    """The cuFFT floor harness on an n^2 grid."""
    if not os.path.exists(FLOOR_BIN):
        return {"unavailable": "cuFFT floor harness not built (baseline/_ref/bin/cufft_floor)"}
    p = subprocess.run([FLOOR_BIN, str(n), str(n), str(steps), str(warmup)], capture_output=True, text=True,
                       timeout=timeout)
    if p.returncode != 0:
        return {"unavailable": f"cufft_floor exited {p.returncode}: {p.stderr[-300:]}"}
    r = json.loads(p.stdout.strip().splitlines()[-1])
    return {"value": r["grid_point_steps_per_s"], "unit": "grid-point-steps/s", "ms_per_step": r["ms_per_step"],
            "steps_timed": steps, "finite": r["finite"],
            "how": "the reference's 28 cufftExec* (cufftPlan2d R2C/C2R) and 21 pointwise kernels per step in one "
                   "CUDA graph, no host syncs, no host energy loop (baseline/cufft_floor.cu); CUDA events"}
