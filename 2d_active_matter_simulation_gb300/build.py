"""In-tree build of libactflow.so (CUDA, sm_103a) and the `actflow` front end.

Translation units are compiled in parallel with nvcc / g++ and linked into
``lib/`` next to this file.  A unit is rebuilt only when one of the sources it
depends on is newer than its object file.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(CSRC, "host")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(HERE, "lib")
OBJ = os.path.join(LIB, "obj")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-diag-suppress", "20013",
              "-I" + INCLUDE, "-I" + CSRC] + ARCH
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-Wall", "-I" + INCLUDE, "-I" + CSRC]

# the kernel tables are split by transform length so that the heavy units
# compile in parallel (the 2048- and 4096-point ones take the longest)
CUDA_UNITS = ["kernels_df_12.cu", "kernels_df_11.cu", "kernels_df_10.cu", "kernels_df_9.cu",
              "kernels_f32_12.cu", "kernels_f32_11.cu", "kernels_f64_12.cu", "kernels_f64_11.cu",
              "kernels_df_8.cu", "kernels_df_7.cu", "kernels_df_6.cu", "kernels_df_3_5.cu",
              "kernels_f32_10.cu", "kernels_batch_9_10.cu", "kernels_f32_3_6.cu", "kernels_f32_7_8.cu",
              "kernels_f32_9.cu", "kernels_f64_3_8.cu", "kernels_f64_9_10.cu",
              "kernels_batch.cu", "kernels_queue.cu", "kernels_f32.cu", "kernels_f64.cu", "kernels_df.cu",
              "actflow_api.cu",
              "noalloc.cu", "batch.cu",
              "ragged.cu", "server.cu"]
HOST_UNITS = ["spec.cpp", "io.cpp", "driver.cpp", "cli.cpp"]


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the actflow CUDA library cannot be built")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h")) + glob.glob(os.path.join(HOST, "*.h"))


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + p.stdout + p.stderr)
    return p.stdout + p.stderr


def build(verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    # Objects built on another machine type (the tree is shared between an
    # x86-64 build host and aarch64 GPU hosts) are discarded.
    import platform
    stamp = os.path.join(LIB, "BUILD_ARCH")
    arch = platform.machine()
    prev = open(stamp).read().strip() if os.path.exists(stamp) else None
    if prev != arch:
        for f in glob.glob(os.path.join(OBJ, "*.o")) + [os.path.join(LIB, "libactflow.so"), os.path.join(LIB, "actflow")]:
            if os.path.exists(f):
                os.remove(f)
        with open(stamp, "w") as fh:
            fh.write(arch + "\n")
    hdrs = _headers()
    jobs = []
    for u in CUDA_UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(OBJ, u + ".o")
        if _stale(obj, [src] + hdrs):
            jobs.append([nvcc()] + NVCC_FLAGS + ["-c", src, "-o", obj])
    for u in HOST_UNITS:
        src = os.path.join(HOST, u)
        obj = os.path.join(OBJ, u + ".o")
        if _stale(obj, [src] + hdrs):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    so = os.path.join(LIB, "libactflow.so")
    cuda_objs = [os.path.join(OBJ, u + ".o") for u in CUDA_UNITS]
    host_lib_objs = [os.path.join(OBJ, u + ".o") for u in ("spec.cpp", "io.cpp", "driver.cpp")]
    if _stale(so, cuda_objs + host_lib_objs):
        _run([nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", so] + cuda_objs + host_lib_objs)
    exe = os.path.join(LIB, "actflow")
    cli_obj = os.path.join(OBJ, "cli.cpp.o")
    if _stale(exe, [so, cli_obj]):
        _run(["g++", "-o", exe, cli_obj, "-L" + LIB, "-lactflow", "-Wl,-rpath,$ORIGIN"])
    return so


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
