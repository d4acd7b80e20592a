"""CPU tests of the host side: the C ABI library loads and exports every
declared symbol, the spec reader, the snapshot/energy formats (byte-exact
against the reference's own files), the initial-field generator, the mask
emulation and the drop-in program's non-GPU paths."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from refformat import read_snapshot, write_spec

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


def test_header_symbols_exported(am):
    with open(os.path.join(ROOT, "include", "actflow.h")) as f:
        hdr = f.read()
    declared = set(re.findall(r"\b(am_[a-z_0-9]+)\s*\(", hdr))
    assert declared == set(am.EXPORTED), declared ^ set(am.EXPORTED)
    lib = ctypes.CDLL(am.LIB_PATH)
    for name in declared:
        assert hasattr(lib, name), name


def test_status_strings(am):
    assert am.status_string(am.AM_OK) == "ok"
    assert "nan" in am.status_string(am.AM_ERR_NAN)


def test_spec_reader_reference_example(am, tmp_path):
    """The reference's shipped specifications.txt layout."""
    d = str(tmp_path)
    write_spec(os.path.join(d, "specifications.txt"), [
        ("T", "5000"), ("dt", "0.005"), ("Lx", "628.3185307"), ("Ly", "628.3185307"), ("Nx", 1024),
        ("Ny", 1024), ("alpha", "-0.8"), ("beta", "0.01"), ("lambda", "7"), ("dt_snap", "1000"),
        ("initial_condition", "random 42"), ("save_directory", "/somewhere/else")])
    s = am.read_spec(d)
    assert s.nx == 1024 and s.ny == 1024
    assert s.T == 5000.0 and s.dt == float(np.float32(0.005))
    assert s.lx == float(np.float32(628.3185307))
    assert s.initial == b"random 42" and s.directory == b"/somewhere/else"
    assert s.precision == am.FP32 and s.dealias == 0 and s.has_gamma == 0


def test_spec_reader_defaults_and_extensions(am, tmp_path):
    d = str(tmp_path)
    write_spec(os.path.join(d, "specifications.txt"), [
        ("precision", "fp64"), ("dealias", "half"), ("Gamma0", "-0.045"), ("Gamma2", "2.5e-5")])
    s = am.read_spec(d)
    # reference defaults (ActFlow_V3-2.cu:183-204)
    assert (s.T, s.nx, s.ny, s.lx) == (100.0, 1024, 1024, 250.0)
    assert s.lam == 7.0 and s.alpha == float(np.float32(-0.8)) and s.initial == b"random"
    assert s.precision == am.FP64 and s.dealias == 1 and s.has_gamma == 1
    assert s.gamma0 == -0.045 and s.gamma2 == 2.5e-5


def test_spec_reader_errors(am, tmp_path):
    d = str(tmp_path)
    with pytest.raises(am.ActflowError) as e:
        am.read_spec(d)
    assert e.value.status == am.AM_ERR_IO
    with open(os.path.join(d, "specifications.txt"), "w") as f:
        f.write("T:\n10\nbogus:\n1\n")
    with pytest.raises(am.ActflowError) as e:
        am.read_spec(d)
    assert e.value.status == am.AM_ERR_SPEC and "bogus" in str(e.value)
    # a blank line is an unknown specification in the reference too
    with open(os.path.join(d, "specifications.txt"), "w") as f:
        f.write("T:\n10\n\ndt:\n0.1\n")
    with pytest.raises(am.ActflowError):
        am.read_spec(d)


@pytest.mark.parametrize("i", [0, 1, 2])
def test_snapshot_writer_byte_exact(am, tmp_path, i):
    """Parse the reference's snapshot text, write it back: identical bytes."""
    src = os.path.join(GOLD, f"format8_snap{i}.txt")
    w, m = am.read_snapshot(src, 8, 8)
    out = str(tmp_path / "s.bin")
    am.write_snapshot(out, w, m)
    with open(src, "rb") as f:
        a = f.read()
    with open(out, "rb") as f:
        b = f.read()
    assert a == b


def test_snapshot_roundtrip_fp64(am, tmp_path):
    w = np.fft.rfft2(np.random.default_rng(2).standard_normal((16, 32)))
    out = str(tmp_path / "s.bin")
    am.write_snapshot(out, w, (1.5, -2.25), precision="fp64")
    w2, m2 = am.read_snapshot(out, 32, 16, precision="fp64")
    assert np.allclose(w2, w, rtol=1e-5) and np.allclose(m2, (1.5, -2.25))
    w3, _ = read_snapshot(out, 32, 16)
    assert np.array_equal(w3, w2)


def test_snapshot_reader_rejects_truncated(am, tmp_path):
    out = str(tmp_path / "s.bin")
    with open(out, "w") as f:
        f.write("1,2,3,4,")
    with pytest.raises(am.ActflowError):
        am.read_snapshot(out, 8, 8)


def test_energy_writer_byte_exact(am, tmp_path):
    with open(os.path.join(GOLD, "format8_energy.txt")) as f:
        ref = f.read()
    vals = [float(line.split()[1]) for line in ref.splitlines()]
    out = str(tmp_path / "energy.txt")
    am.append_energy(out, 0, float(np.float32(0.01)), vals[:1])
    am.append_energy(out, 1, float(np.float32(0.01)), vals[1:])
    with open(out) as f:
        assert f.read() == ref


def test_bandlimited_ic_matches_oracle_restatement(am):
    from oracle.ic import bandlimited
    for nx, ny, seed in [(64, 64, 42), (256, 128, 7), (32, 64, 3)]:
        a = am.ic_bandlimited(nx, ny, seed)
        b = bandlimited(nx, ny, seed)
        assert np.abs(a - b).max() <= 1e-15 * np.abs(b).max()
        x = np.fft.irfft2(a, s=(ny, nx))
        assert abs(np.sqrt((x ** 2).mean()) - 0.01) < 1e-12
        assert abs(x.mean()) < 1e-15


@pytest.mark.parametrize("n", [(64, 64), (384, 384), (512, 512), (1024, 1024), (64, 32), (2048, 2048)])
@pytest.mark.parametrize("mode", ["reference", "half", "none"])
def test_mask_matches_oracle(am, orc, n, mode):
    nx, ny = n
    m = orc.mask(nx, ny, mode)
    rng = np.random.default_rng(nx + ny)
    for _ in range(200):
        ix, iy = int(rng.integers(0, nx // 2 + 1)), int(rng.integers(0, ny))
        assert am.mask_value(nx, ny, mode, ix, iy) == int(m[iy, ix])
    assert am.mask_value(nx, ny, mode, 0, 0) == 1


def test_cli_help_spec_math(am, tmp_path):
    exe = am.CLI_PATH
    p = subprocess.run([exe, "help"], capture_output=True, text=True)
    assert p.returncode == 0 and "specifications.txt" in p.stdout
    p = subprocess.run([exe, "spec"], capture_output=True, text=True, cwd=tmp_path)
    assert p.returncode == 0
    s = am.read_spec(str(tmp_path))
    assert (s.T, s.nx, s.lx, s.initial) == (100.0, 1024, 250.0, b"random")
    with open(tmp_path / "specifications.txt") as f:
        txt = f.read()
    assert txt.startswith("T:\n100\ndt:\n0.002\nLx:\n250\n") and txt.endswith("save_directory:\n./")
    p = subprocess.run([exe, "math"], capture_output=True, text=True, cwd=tmp_path)
    assert p.returncode == 0 and (tmp_path / "theory.tex").exists()


def test_cli_error_exits(am, tmp_path):
    exe = am.CLI_PATH
    assert subprocess.run([exe], capture_output=True).returncode == 1
    assert subprocess.run([exe, "a", "b"], capture_output=True).returncode == 1
    # missing specifications.txt
    assert subprocess.run([exe, str(tmp_path)], capture_output=True).returncode == 1
    # unknown key
    with open(tmp_path / "specifications.txt", "w") as f:
        f.write("T:\n1\nfoo:\n2\n")
    p = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True)
    assert p.returncode == 1 and "foo" in p.stderr
    # dt_snap below dt/2 (undefined behaviour in the reference) is rejected
    with open(tmp_path / "specifications.txt", "w") as f:
        f.write("dt:\n0.1\ndt_snap:\n0.01\n")
    assert subprocess.run([exe, str(tmp_path)], capture_output=True).returncode == 1


def test_column_shape_table(am):
    """The column-pass shape table (no GPU needed): seeded narrow below 2048,
    settable per precision and Ny, sizes outside 8..4096 rejected."""
    assert am.column_shape("fp32", 2048) == "wide" and am.column_shape("fp32", 1024) == "narrow"
    assert am.column_shape("fp64", 4096) == "wide" and am.column_shape("fp64", 256) == "narrow"
    am.set_column_shape("fp32", 512, "wide")
    assert am.column_shape("fp32", 512) == "wide" and am.column_shape("fp64", 512) == "narrow"
    am.set_column_shape("fp32", 512, "narrow")
    assert am.column_shape("fp32", 512) == "narrow"
    assert am.column_shape("fp32", 96) is None
    with pytest.raises(am.ActflowError):
        am.set_column_shape("fp32", 8192, "wide")
