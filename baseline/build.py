"""Build the two GPU comparators the benchmark times beside the solver.

* ``_ref/bin/ActFlow_ref`` -- the reference program itself (ActFlow_V3-2.cu
  with its two headers, unmodified), compiled for sm_103a with cuFFT by
  ``oracle/build_ref.sh``.  Its sources are staged into ``_ref/src`` from the
  reference checkout when one is mounted (``stage``); ``_ref/`` is not part of
  the repository's history, but it is carried with the working tree to the
  machine that runs the benchmark, which builds from the staged copy.
* ``_ref/bin/cufft_floor`` -- ``cufft_floor.cu``: the reference's step as its
  28 cuFFT transforms and 21 pointwise kernels in one CUDA graph, with no host
  synchronisation (a lower bound on the reference design's step time).

Neither is part of the solver; failures are recorded in ``_ref/bin/BUILD_LOG``
and leave the benchmark to report the comparator as unavailable.
"""
import os
import platform
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REF = os.path.join(HERE, "_ref")
SRC = os.path.join(REF, "src")
BIN = os.path.join(REF, "bin")
REF_FILES = ("ActFlow_V3-2.cu", "cudaErr.h", "cuComplexBinOp.h")


def stage(ref_dir):
    """Copy the reference program's three source files into _ref/src."""
    if not all(os.path.isfile(os.path.join(ref_dir, f)) for f in REF_FILES):
        return False
    os.makedirs(SRC, exist_ok=True)
    for f in REF_FILES:
        dst = os.path.join(SRC, f)
        if os.path.exists(dst):
            os.remove(dst)   # the copies keep the mount's read-only mode
        shutil.copyfile(os.path.join(ref_dir, f), dst)
    return True


def _nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def build(ref_dir=None):
    """Stage (if ref_dir holds the reference) and compile both comparators."""
    if ref_dir:
        stage(ref_dir)
    os.makedirs(BIN, exist_ok=True)
    stamp = os.path.join(BIN, "BUILD_ARCH")
    arch = platform.machine()
    if not os.path.exists(stamp) or open(stamp).read().strip() != arch:
        for f in ("ActFlow_ref", "cufft_floor"):
            if os.path.exists(os.path.join(BIN, f)):
                os.remove(os.path.join(BIN, f))
        with open(stamp, "w") as fh:
            fh.write(arch + "\n")
    log = []
    jobs = []
    floor_src = os.path.join(HERE, "cufft_floor.cu")
    floor_bin = os.path.join(BIN, "cufft_floor")
    if not os.path.exists(floor_bin) or os.path.getmtime(floor_bin) < os.path.getmtime(floor_src):
        jobs.append(("cufft_floor", [_nvcc(), "-std=c++17", "-O3", "-gencode", "arch=compute_103a,code=sm_103a",
                                     floor_src, "-lcufft", "-o", floor_bin]))
    ref_bin = os.path.join(BIN, "ActFlow_ref")
    if os.path.isfile(os.path.join(SRC, REF_FILES[0])) and not os.path.exists(ref_bin):
        jobs.append(("ActFlow_ref", ["bash", os.path.join(ROOT, "oracle", "build_ref.sh"), SRC, BIN]))
    procs = [(name, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
             for name, cmd in jobs]
    for name, p in procs:
        out, _ = p.communicate()
        log.append(f"{name}: exit {p.returncode}\n{out[-2000:]}")
    if log:
        with open(os.path.join(BIN, "BUILD_LOG"), "w") as fh:
            fh.write("\n".join(log))
    return {"ActFlow_ref": os.path.exists(ref_bin), "cufft_floor": os.path.exists(floor_bin)}


if __name__ == "__main__":
    import sys
    print(build(sys.argv[1] if len(sys.argv) > 1 else None))
