"""Readers and writers for the reference program's on-disk formats (test side).

* ``specifications.txt``: ``key:`` lines each followed by one value line
  (ActFlow_V3-2.cu:326-401).
* Snapshot ``ActTurb_snap{i}.bin``: ASCII despite the suffix -- ``Ny*(Nx/2+1)``
  pairs ``re,im,`` of the half-plane spectrum in row-major ``[iy][ix]`` order,
  then ``mean_x,mean_y`` (the mean velocity scaled by ``Nx*Ny``), each number in
  the default ostream form (``%g``, six significant digits)
  (ActFlow_V3-2.cu:1261-1263; reader ActFlow_V3-2.cu:620-631, image.py:49-52).
* ``energy.txt``: one ``"{m*dt} {E}\\n"`` line per step (ActFlow_V3-2.cu:1275).
"""
import numpy as np


def write_spec(path, entries):
    """Write a specifications file from (key, value) pairs, in order."""
    with open(path, "w") as f:
        lines = []
        for k, v in entries:
            lines.append(f"{k}:")
            lines.append(str(v))
        f.write("\n".join(lines) + "\n")


def write_snapshot_exact(path, w_hat, mean):
    """Write a snapshot with nine significant digits (exact float32 round trip).

    Used to inject a seeded initial field through ``initial_condition:
    continue``; the reference parses it with ``operator>>`` into floats.
    """
    w = np.asarray(w_hat, dtype=np.complex64).reshape(-1)
    parts = []
    for c in w:
        parts.append("%.9g,%.9g," % (float(c.real), float(c.imag)))
    parts.append("%.9g,%.9g" % (float(np.float32(mean[0])), float(np.float32(mean[1]))))
    with open(path, "w") as f:
        f.write("".join(parts))


def read_snapshot(path, nx, ny):
    """Parse a snapshot into (complex128 array [ny, nx//2+1], mean[2])."""
    with open(path) as f:
        txt = f.read()
    vals = np.array([float(t) for t in txt.split(",") if t.strip() != ""], dtype=np.float64)
    nxh = nx // 2 + 1
    n = ny * nxh
    if vals.size != 2 * n + 2:
        raise ValueError(f"{path}: expected {2 * n + 2} numbers, got {vals.size}")
    w = vals[: 2 * n].reshape(ny, nxh, 2)
    return w[..., 0] + 1j * w[..., 1], vals[2 * n:]


def read_energy(path):
    """Parse energy.txt into (times, energies) float64 arrays."""
    t, e = [], []
    with open(path) as f:
        for line in f:
            if not line.strip():
                continue
            a, b = line.split()
            t.append(float(a))
            e.append(float(b))
    return np.array(t), np.array(e)
