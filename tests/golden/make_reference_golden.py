"""Run the reference program on seeded inputs and save its outputs as fixtures.

The reference (ActFlow_V3-2.cu) is a single-GPU CUDA program with no tests and
no golden data, and its own ``random`` initial field is seeded from the wall
clock (ActFlow_V3-2.cu:539-545).  This script therefore injects seeded initial
fields through the reference's resume path: it writes ``ActTurb_snap0.bin`` in
the reference's text layout with nine significant digits (an exact float32
round trip), writes a ``specifications.txt`` with ``initial_condition:
continue``, runs the reference binary, and reads back ``energy.txt`` and the
snapshots.

Resume semantics that fix the step numbering (ActFlow_V3-2.cu:567-647, 718-862):
resuming from snapshot 0 sets the step counter ``m`` to 0 and the loop runs
``m = 0 .. M`` with ``M = round(T/dt)``, i.e. ``M + 1`` steps.  ``energy.txt``
line ``m`` holds ``(m*dt, E)`` with ``E`` the energy of the state at the start
of step ``m``; snapshot ``i`` is written after step ``m = i*snap`` and so holds
the state after ``i*snap + 1`` steps (snapshot 0 is overwritten after the first
step).

The reference binary is built by ``oracle/build_ref.sh`` and needs a GPU; run
this script where one is present:

    python tests/golden/make_reference_golden.py oracle/_ref/ActFlow_ref OUTDIR

Each case writes ``OUTDIR/<case>.npz`` (float64 arrays) and, for the tiny
format case, the raw text files.
"""
import math
import os
import shutil
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, HERE)

from ic import bandlimited  # noqa: E402
from refformat import read_energy, read_snapshot, write_snapshot_exact, write_spec  # noqa: E402

# Physical parameters of the benchmark workloads and their exact map onto the
# reference's normalised equation (length l, time tau): L_ref(k) = -(1-k^2)^2 - alpha_ref.
GAMMA0, GAMMA2 = -0.045, 2.5e-5
ELL = math.sqrt(-2.0 * GAMMA2 / GAMMA0)
TAU = ELL ** 4 / GAMMA2


def to_reference_units(alpha, beta, dt):
    return dict(alpha=TAU * alpha - 1.0, beta=beta * ELL * ELL / TAU,
                L=2.0 * math.pi / ELL, dt=dt / TAU)


def _fmt(x):
    return "%.9g" % x


def run_case(ref_bin, workdir, nx, ny, lx, ly, lam, alpha, beta, dt, steps, snap,
             w0, mean0, timeout=1800):
    """Run the reference for ``steps`` steps from (w0, mean0); return outputs."""
    if os.path.isdir(workdir):
        shutil.rmtree(workdir)
    os.makedirs(workdir)
    M = steps - 1
    T = M * dt
    write_spec(os.path.join(workdir, "specifications.txt"), [
        ("T", _fmt(T)), ("dt", _fmt(dt)), ("Lx", _fmt(lx)), ("Ly", _fmt(ly)),
        ("Nx", nx), ("Ny", ny), ("lambda", _fmt(lam)), ("alpha", _fmt(alpha)),
        ("beta", _fmt(beta)), ("dt_snap", _fmt(snap * dt)),
        ("initial_condition", "continue"), ("save_directory", workdir)])
    write_snapshot_exact(os.path.join(workdir, "ActTurb_snap0.bin"), w0, mean0)
    t0 = time.time()
    p = subprocess.run([ref_bin, workdir], capture_output=True, text=True, timeout=timeout)
    wall = time.time() - t0
    if p.returncode != 0:
        raise RuntimeError(f"reference exited {p.returncode}: {p.stderr[-2000:]}")
    # The reference prints "program finished successfully after Xs." (loop + cleanup).
    loop_s = float("nan")
    for line in p.stdout.splitlines():
        if "finished successfully after" in line:
            loop_s = float(line.split("after")[1].strip().rstrip(".").rstrip("s"))
    t, e = read_energy(os.path.join(workdir, "energy.txt"))
    snaps = {}
    i = 0
    while os.path.exists(os.path.join(workdir, f"ActTurb_snap{i}.bin")):
        snaps[i] = os.path.join(workdir, f"ActTurb_snap{i}.bin")
        i += 1
    return dict(t=t, e=e, snaps=snaps, wall=wall, loop_s=loop_s, stdout=p.stdout)


def case_params(name):
    """The golden cases (reference units unless noted)."""
    cases = {
        # Strongly nonlinear small case with a nonzero mean flow.
        "small64": dict(nx=64, ny=64, lx=16 * math.pi, ly=16 * math.pi, lam=7.0,
                        alpha=-0.8, beta=0.01, dt=0.005, steps=21, snap=5,
                        seed=11, kmax=8.0, rms=1.0, mean=(0.3, -0.2)),
        # Rectangular grids, both orientations.
        "rect64x32": dict(nx=64, ny=32, lx=16 * math.pi, ly=8 * math.pi, lam=7.0,
                          alpha=-0.8, beta=0.01, dt=0.005, steps=11, snap=5,
                          seed=12, kmax=6.0, rms=1.0, mean=(-0.1, 0.25)),
        "rect32x64": dict(nx=32, ny=64, lx=8 * math.pi, ly=16 * math.pi, lam=5.0,
                          alpha=-0.6, beta=0.02, dt=0.004, steps=11, snap=5,
                          seed=13, kmax=6.0, rms=1.0, mean=(0.2, 0.05)),
        # 512^2: the reference's dealias radius wraps to 0 in int32, so only the
        # k=0 mode of the nonlinear term survives (ActFlow_V3-2.cu:911-917).
        "mask512": dict(nx=512, ny=512, lx=64 * math.pi, ly=64 * math.pi, lam=7.0,
                        alpha=-0.8, beta=0.01, dt=0.005, steps=3, snap=1,
                        seed=5, kmax=8.0, rms=1.0, mean=(0.5, 0.1)),
        # Tiny grid whose raw text outputs are kept for byte-exact format checks.
        "format8": dict(nx=8, ny=8, lx=2 * math.pi, ly=2 * math.pi, lam=7.0,
                        alpha=-0.8, beta=0.01, dt=0.01, steps=3, snap=1,
                        seed=3, kmax=2.0, rms=1.0, mean=(0.4, -0.3)),
    }
    # The 256^2 benchmark field in physical units (2pi box, rms 0.01), mapped
    # onto the reference's units: omega_ref = tau*omega, u_ref = (tau/l) u.
    r = to_reference_units(alpha=-0.8, beta=0.01, dt=5e-4)
    cases["config0_256"] = dict(nx=256, ny=256, lx=r["L"], ly=r["L"], lam=3.5,
                                alpha=r["alpha"], beta=r["beta"], dt=r["dt"],
                                steps=2001, snap=50, seed=42, kmax=8.0, rms=0.01,
                                mean=(0.0, 0.0), scale=TAU)
    # Timing-only: the 2048^2 benchmark grid (dt = 1e-4 physical), few steps.
    r1 = to_reference_units(alpha=-0.8, beta=0.01, dt=1e-4)
    cases["time2048"] = dict(nx=2048, ny=2048, lx=r1["L"], ly=r1["L"], lam=3.5,
                             alpha=r1["alpha"], beta=r1["beta"], dt=r1["dt"],
                             steps=21, snap=20, seed=7, kmax=8.0, rms=0.01,
                             mean=(0.0, 0.0), scale=TAU)
    return cases[name]


ALL_CASES = ["format8", "small64", "rect64x32", "rect32x64", "mask512", "config0_256", "time2048"]


def make_case(ref_bin, outdir, name):
    p = case_params(name)
    nx, ny = p["nx"], p["ny"]
    w0 = bandlimited(nx, ny, p["seed"], kmax=p["kmax"], rms=p["rms"]) * p.get("scale", 1.0)
    w0 = w0.astype(np.complex64)
    n = nx * ny
    mean0 = (np.float32(p["mean"][0] * n), np.float32(p["mean"][1] * n))
    workdir = os.path.join(outdir, "run_" + name)
    res = run_case(ref_bin, workdir, nx, ny, p["lx"], p["ly"], p["lam"], p["alpha"],
                   p["beta"], p["dt"], p["steps"], p["snap"], w0, mean0)
    out = dict(nx=nx, ny=ny, lx=p["lx"], ly=p["ly"], lam=p["lam"], alpha=p["alpha"],
               beta=p["beta"], dt=p["dt"], steps=p["steps"], snap=p["snap"],
               w0=w0, mean0=np.array(mean0, dtype=np.float64),
               energy_t=res["t"], energy=res["e"], wall_s=res["wall"],
               loop_s=res["loop_s"])
    keep = sorted(res["snaps"])
    if name == "config0_256":
        keep = [1, 4]                     # states after 51 and 201 steps
        w_last, m_last = read_snapshot(res["snaps"][max(res["snaps"])], nx, ny)
        out["last_index"] = max(res["snaps"])
        out["last_mean"] = m_last
        out["last_shell_spectrum"] = shell_spectrum(w_last, nx, ny)
    elif name == "mask512":
        keep = []
        w_last, m_last = read_snapshot(res["snaps"][max(res["snaps"])], nx, ny)
        nz = np.nonzero(w0)
        out["last_index"] = max(res["snaps"])
        out["last_mean"] = m_last
        out["support_iy"], out["support_ix"] = nz[0], nz[1]
        out["last_on_support"] = w_last[nz]
        off = np.ones(w_last.shape, bool)
        off[nz] = False
        out["last_max_off_support"] = np.abs(w_last[off]).max()
    elif name == "time2048":
        keep = []
    for i in keep:
        w, m = read_snapshot(res["snaps"][i], nx, ny)
        out[f"snap{i}"] = w.astype(np.complex64)
        out[f"snap{i}_mean"] = m
    np.savez_compressed(os.path.join(outdir, name + ".npz"), **out)
    if name == "format8":
        for i, path in res["snaps"].items():
            shutil.copy(path, os.path.join(outdir, f"format8_snap{i}.txt"))
        shutil.copy(os.path.join(workdir, "energy.txt"), os.path.join(outdir, "format8_energy.txt"))
    shutil.rmtree(workdir)
    print(f"{name}: steps={p['steps']} wall={res['wall']:.3f}s loop={res['loop_s']}s", flush=True)


def make_example1024(ref_bin, outdir):
    """The reference's shipped example (1024^2, random IC), two steps.

    At 1024^2 the dealias radius wraps to 0 and the mask keeps only k=0, so the
    random initial field is erased and the energy stays exactly 0.
    """
    workdir = os.path.join(outdir, "run_example1024")
    if os.path.isdir(workdir):
        shutil.rmtree(workdir)
    os.makedirs(workdir)
    write_spec(os.path.join(workdir, "specifications.txt"), [
        ("T", "0.01"), ("dt", "0.005"), ("Lx", "628.3185307"), ("Ly", "628.3185307"),
        ("Nx", 1024), ("Ny", 1024), ("alpha", "-0.8"), ("beta", "0.01"), ("lambda", "7"),
        ("dt_snap", "1000"), ("initial_condition", "random 42"), ("save_directory", workdir)])
    p = subprocess.run([ref_bin, workdir], capture_output=True, text=True, timeout=600)
    if p.returncode != 0:
        raise RuntimeError(f"reference exited {p.returncode}: {p.stderr[-2000:]}")
    with open(os.path.join(workdir, "energy.txt")) as f:
        energy_txt = f.read()
    w, m = read_snapshot(os.path.join(workdir, "ActTurb_snap0.bin"), 1024, 1024)
    np.savez_compressed(os.path.join(outdir, "example1024.npz"),
                        energy_txt=np.array(energy_txt), snap0_max_abs=np.abs(w).max(),
                        snap0_mean=m)
    shutil.rmtree(workdir)
    print("example1024:", repr(energy_txt), "max|w|=", np.abs(w).max(), flush=True)


def shell_spectrum(w, nx, ny):
    """Shell-summed |w_hat|^2 over integer |k| shells (index units), full plane."""
    nxh = nx // 2 + 1
    iy = np.fft.fftfreq(ny, 1.0 / ny)[:, None]
    ix = np.arange(nxh)[None, :]
    kk = np.sqrt(ix * ix + iy * iy)
    wt = np.where(ix == 0, 1.0, 2.0)
    if nx % 2 == 0:
        wt = np.where(ix == nx // 2, 1.0, wt)
    shell = np.rint(kk).astype(int)
    return np.bincount(shell.ravel(), weights=(wt * np.abs(w) ** 2).ravel())


def main():
    ref_bin, outdir = sys.argv[1], sys.argv[2]
    names = sys.argv[3:] or ALL_CASES + ["example1024"]
    os.makedirs(outdir, exist_ok=True)
    for name in names:
        if name == "example1024":
            make_example1024(ref_bin, outdir)
        else:
            make_case(ref_bin, outdir, name)


if __name__ == "__main__":
    main()
