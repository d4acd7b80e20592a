"""The drop-in program on the GPU: `actflow <dir>` against the reference's own
outputs for the same specifications.txt (process contract of ActFlow_V3-2.cu:
exit codes, energy.txt, ActTurb_snap{i}.bin)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from refformat import read_energy, read_snapshot, write_snapshot_exact, write_spec

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _run(am, d):
    exe = am.CLI_PATH
    return subprocess.run([exe, d], capture_output=True, text=True, timeout=600)


def test_cli_reference_example_1024(am, tmp_path):
    """The shipped example spec (1024^2, random 42): the reference writes
    energy.txt = '0.005 0\\n0.01 0\\n' and an all-zero snapshot 0."""
    d = str(tmp_path)
    write_spec(os.path.join(d, "specifications.txt"), [
        ("T", "0.01"), ("dt", "0.005"), ("Lx", "628.3185307"), ("Ly", "628.3185307"),
        ("Nx", 1024), ("Ny", 1024), ("alpha", "-0.8"), ("beta", "0.01"), ("lambda", "7"),
        ("dt_snap", "1000"), ("initial_condition", "random 42"), ("save_directory", d)])
    p = _run(am, d)
    assert p.returncode == 0, p.stderr
    gold = np.load(os.path.join(GOLD, "example1024.npz"))
    with open(os.path.join(d, "energy.txt")) as f:
        assert f.read() == str(gold["energy_txt"])
    w, m = read_snapshot(os.path.join(d, "ActTurb_snap0.bin"), 1024, 1024)
    assert np.abs(w).max() == 0.0 and np.all(m == 0)


@pytest.mark.parametrize("name", ["format8", "small64"])
def test_cli_continue_matches_reference_outputs(am, tmp_path, name):
    """Same injected field, same spec: snapshots and energy.txt agree with the
    reference's files to its six printed digits."""
    g = np.load(os.path.join(GOLD, name + ".npz"))
    nx, ny, dt, steps, snap = int(g["nx"]), int(g["ny"]), float(g["dt"]), int(g["steps"]), int(g["snap"])
    d = str(tmp_path)
    write_spec(os.path.join(d, "specifications.txt"), [
        ("T", "%.9g" % ((steps - 1) * dt)), ("dt", "%.9g" % dt), ("Lx", "%.9g" % float(g["lx"])),
        ("Ly", "%.9g" % float(g["ly"])), ("Nx", nx), ("Ny", ny), ("lambda", "%.9g" % float(g["lam"])),
        ("alpha", "%.9g" % float(g["alpha"])), ("beta", "%.9g" % float(g["beta"])),
        ("dt_snap", "%.9g" % (snap * dt)), ("initial_condition", "continue"), ("save_directory", d)])
    write_snapshot_exact(os.path.join(d, "ActTurb_snap0.bin"), g["w0"], g["mean0"])
    p = _run(am, d)
    assert p.returncode == 0, p.stderr
    t, e = read_energy(os.path.join(d, "energy.txt"))
    assert len(e) == steps
    assert np.allclose(t, g["energy_t"], rtol=1e-6, atol=0)
    assert np.abs(e - g["energy"]).max() <= 1e-5 * np.abs(g["energy"]).max()
    idx = sorted(int(k[4:]) for k in g.keys() if k.startswith("snap") and k[4:].isdigit())
    for i in idx:
        w, m = read_snapshot(os.path.join(d, f"ActTurb_snap{i}.bin"), nx, ny)
        ref = g[f"snap{i}"]
        assert np.linalg.norm(w - ref) / np.linalg.norm(ref) < 5e-6
    if name == "format8":
        # Same number of fields and separators as the reference's files.
        for i in idx:
            with open(os.path.join(GOLD, f"format8_snap{i}.txt")) as f:
                ref_txt = f.read()
            with open(os.path.join(d, f"ActTurb_snap{i}.bin")) as f:
                txt = f.read()
            assert txt.count(",") == ref_txt.count(",") and not txt.endswith(",")


def test_cli_nan_exits_1(am, tmp_path):
    d = str(tmp_path)
    nx = ny = 16
    write_spec(os.path.join(d, "specifications.txt"), [
        ("T", "0.05"), ("dt", "0.01"), ("Lx", "20"), ("Ly", "20"), ("Nx", nx), ("Ny", ny),
        ("dt_snap", "0.02"), ("initial_condition", "continue"), ("save_directory", d)])
    w = np.zeros((ny, nx // 2 + 1), np.complex64)
    w[0, 0] = np.nan
    write_snapshot_exact(os.path.join(d, "ActTurb_snap0.bin"), w, (0.0, 0.0))
    p = _run(am, d)
    assert p.returncode == 1
    assert "nan values after 0 timesteps" in p.stderr
    # the reference writes the energy of step 0 and snapshot 0 (0 % snap == 0)
    t, e = read_energy(os.path.join(d, "energy.txt"))
    assert len(t) == 1


def _fresh_bandlimited(am, d, precision):
    write_spec(os.path.join(d, "specifications.txt"), [
        ("T", "0.01"), ("dt", "0.001"), ("Lx", "6.283185307"), ("Ly", "6.283185307"), ("Nx", 64), ("Ny", 64),
        ("lambda", "3.5"), ("alpha", "-0.8"), ("beta", "0.01"), ("dt_snap", "0.005"),
        ("initial_condition", "bandlimited 42"), ("save_directory", d), ("precision", precision),
        ("dealias", "half"), ("Gamma0", "-0.045"), ("Gamma2", "2.5e-5")])
    p = _run(am, d)
    assert p.returncode == 0, p.stderr
    t, e = read_energy(os.path.join(d, "energy.txt"))
    assert len(t) == 10 and abs(t[0] - 0.001) < 1e-9
    assert os.path.exists(os.path.join(d, "ActTurb_snap2.bin"))
    return e, read_snapshot(os.path.join(d, "ActTurb_snap2.bin"), 64, 64)


def test_cli_fresh_bandlimited_fp64(am, tmp_path):
    _fresh_bandlimited(am, str(tmp_path), "fp64")


def test_cli_double_float_matches_fp64(am, tmp_path):
    """`precision: df64` through the drop-in program: the same files as an FP64
    run, with energies and the snapshot (printed to six digits, as the
    reference's text snapshots) equal to the FP64 run's up to rounding of
    the last printed digit."""
    os.makedirs(tmp_path / "a")
    os.makedirs(tmp_path / "b")
    e64, (w64, m64) = _fresh_bandlimited(am, str(tmp_path / "a"), "fp64")
    edf, (wdf, mdf) = _fresh_bandlimited(am, str(tmp_path / "b"), "df64")
    assert np.abs(edf - e64).max() <= 1e-5 * np.abs(e64).max()
    assert np.abs(wdf - w64).max() <= 1e-5 * np.abs(w64).max()


def _raw(path, nx, ny):
    with open(path, "rb") as f:
        b = f.read()
    assert b[:6] == b"AFRAW1"
    hdr = np.frombuffer(b[8:24], dtype=np.int32)
    assert tuple(hdr[:2]) == (nx, ny)
    n = ny * (nx // 2 + 1)
    w = np.frombuffer(b[24:24 + 8 * n], dtype=np.complex64).reshape(ny, nx // 2 + 1)
    m = np.frombuffer(b[24 + 8 * n:], dtype=np.float64)
    return w, m


def test_cli_binary_sidecar_resumes_exactly(am, tmp_path):
    """snapshot_binary: 1 writes ActTurb_snap{i}.raw beside each text snapshot;
    `continue` then resumes from the exact state (the text has six digits)."""
    nx = ny = 64
    d = str(tmp_path)
    spec = [("T", "0.05"), ("dt", "0.005"), ("Lx", "50.26548"), ("Ly", "50.26548"), ("Nx", nx), ("Ny", ny),
            ("lambda", "7"), ("alpha", "-0.8"), ("beta", "0.01"), ("dt_snap", "0.025"),
            ("initial_condition", "bandlimited 5 1 8 1.0"), ("save_directory", d), ("snapshot_binary", "1")]
    write_spec(os.path.join(d, "specifications.txt"), spec)
    p = _run(am, d)
    assert p.returncode == 0, p.stderr
    for i in range(3):
        w_txt, m_txt = read_snapshot(os.path.join(d, f"ActTurb_snap{i}.bin"), nx, ny)
        w_raw, m_raw = _raw(os.path.join(d, f"ActTurb_snap{i}.raw"), nx, ny)
        assert np.allclose(w_txt, w_raw, rtol=1e-5, atol=1e-6 * np.abs(w_raw).max())
    # resume from snapshot 1 (m = 5, steps 5..10 -> 6 steps, the reference's numbering)
    w1, m1 = _raw(os.path.join(d, "ActTurb_snap1.raw"), nx, ny)
    for f in ("ActTurb_snap2.bin", "ActTurb_snap2.raw", "energy.txt"):
        os.remove(os.path.join(d, f))
    spec[10] = ("initial_condition", "continue")
    write_spec(os.path.join(d, "specifications.txt"), spec)
    p = _run(am, d)
    assert p.returncode == 0, p.stderr
    assert "exact binary copy" in p.stdout
    w2, m2 = _raw(os.path.join(d, "ActTurb_snap2.raw"), nx, ny)
    sim = am.Solver(nx, ny, float(np.float32(50.26548)), float(np.float32(50.26548)), float(np.float32(0.005)),
                    7.0, float(np.float32(-0.8)), float(np.float32(0.01)))
    sim.set_state(w1, m1)
    sim.step(6)
    w, m = sim.get_state()
    sim.close()
    assert np.array_equal(w, w2) and np.array_equal(m, m2)


def test_cli_unwritable_snapshot_dir_exits_1(am, tmp_path):
    d = str(tmp_path)
    out = os.path.join(d, "no", "such", "dir")
    write_spec(os.path.join(d, "specifications.txt"), [
        ("T", "0.01"), ("dt", "0.005"), ("Nx", 32), ("Ny", 32), ("Lx", "30"), ("Ly", "30"),
        ("initial_condition", "blank"), ("save_directory", out)])
    p = _run(am, d)
    assert p.returncode == 1 and "unable to create snapshot file" in p.stderr
