"""Benchmark: grid-point-steps/s of the IF-RK4 vorticity step on one GB300.

Workload (the configuration the headline metric is quoted on): one 2048^2
simulation, FP32, dt = 1e-4 on the [0, 2 pi)^2 box, lambda = 3.5, alpha = -0.8,
beta = 0.01, Gamma0 = -0.045, Gamma2 = 2.5e-5, isotropic 1/2-rule dealiasing,
seeded band-limited initial field (modes 1 <= |k| <= 8, rms 0.01, seed 7).
A bench "step" is one full RK4 step (8 kernels: row pass + column pass per
stage).

    python bench.py [--gpus 1] [--steps K] [--warmup W] [--impl ours|reference]

Our arm times K steps with CUDA events on the solver's stream (state resident
in HBM, L2 flushed by a 256 MB write before every step), then the same metric
end to end through the C ABI with host buffers (set_state from pinned memory,
K steps with the per-step energy read back, get_state), per-kernel CUDA-event
times for the roofline, and the oracle's CPU step as the reported CPU baseline.
The reference arm times the CPU implementation of the step (the oracle, a C
restatement of the reference program's step; the reference itself has no CPU
path) on all host cores, one full 2048^2 step per bench step.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)


# ---- replicas (--gpus N > 1 under torchrun): one independent simulation per
# GPU, no data exchange (the step has none); the ranks meet only at the
# barriers around the timed region and in the max of their times, over gloo.
def replica_device(local_rank, visible):
    """CUDA_VISIBLE_DEVICES for a rank: its own entry of the visible list, or
    its index when the variable is unset (visible is None).  A list that is set
    but has no entry for this rank (including an empty one, which hides every
    GPU) is an error: falling back to the rank's index would select a GPU
    outside the devices this job was given.  The solver library carries its own
    CUDA runtime, so the device is chosen by visibility before anything loads."""
    if visible is None:
        return str(local_rank)
    ids = [d.strip() for d in visible.split(",") if d.strip()]
    if local_rank >= len(ids):
        raise RuntimeError(f"local rank {local_rank} has no device in CUDA_VISIBLE_DEVICES={visible!r} "
                           f"({len(ids)} visible)")
    return ids[local_rank]


def world():
    return int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0"))


def replica_setup():
    """Bind this rank to its GPU and join the host-side process group."""
    n, _ = world()
    if n <= 1:
        return
    lr = int(os.environ.get("LOCAL_RANK", "0"))
    os.environ["CUDA_VISIBLE_DEVICES"] = replica_device(lr, os.environ.get("CUDA_VISIBLE_DEVICES"))
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group("gloo")


def replica_barrier():
    n, _ = world()
    if n > 1:
        import torch.distributed as dist
        dist.barrier()


def replica_max(x):
    """Largest value of x over the ranks (x itself on one GPU)."""
    n, _ = world()
    if n <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())

NX = NY = 2048
PARAMS = dict(lx=2 * math.pi, ly=2 * math.pi, dt=1e-4, lam=3.5, alpha=-0.8, beta=0.01,
              gamma0=-0.045, gamma2=2.5e-5, dealias="half")
SEED = 7
PRECISION = "fp32"
WORKLOAD = "IF-RK4 vorticity step, 2048^2, FP32, dt=1e-4, 1/2-rule dealiasing, band-limited seed 7"
# --config 0: the 256^2 plain-method run (dt 5e-4, the reference's own mask,
# which keeps every mode at 256^2), seed 42; --precision selects FP32 / FP64.
PRESETS = {
    0: dict(n=256, dt=5e-4, dealias="reference", seed=42),
    1: dict(n=2048, dt=1e-4, dealias="half", seed=7),
    # --config 2: 64-member ensemble of 512^2 grids in one batch (one launch per
    # pass for all members), alpha ~ U[-1, -0.3] and lambda ~ U[2, 5] drawn with
    # numpy's default_rng(2), member seeds 1000 + i.
    2: dict(n=512, dt=2.5e-4, dealias="half", seed=1000, members=64),
    # --config 3: ragged batch of 40 runs, grids log-uniform over {128..1024}^2,
    # steps U[1000, 5000], alpha ~ U[-1, -0.3], lambda ~ U[2, 5],
    # dt = 0.1 dx / sqrt(-alpha / beta); master seed 3, run seeds 2000 + i.
    3: dict(n=1024, dt=0.0, dealias="half", seed=2000, runs=40),
    # --config 4: serving trace, Poisson arrivals at 4 requests/s, grids
    # log-uniform over {128..4096}^2, 10% FP64, steps log-uniform 500..20000,
    # parameters as config 2; master seed 4.  --serve-seconds sets the arrival
    # window and --serve-step-scale scales every request's step count.
    4: dict(n=4096, dt=0.0, dealias="half", seed=4, rate=4.0),
}


# arithmetic type of each precision path (df64: double-float, two FP32 per real)
DTYPES = {"fp32": "f32", "fp64": "f64", "df64": "f32x2 (double-float)"}


def apply_preset(cfg, precision, n=None):
    global NX, NY, SEED, PRECISION, WORKLOAD
    p = PRESETS[cfg]
    if cfg in (2, 3):
        precision = "fp32"
    NX = NY = n if n else p["n"]
    SEED = p["seed"]
    PARAMS["dt"] = p["dt"]
    PARAMS["dealias"] = p["dealias"]
    PRECISION = precision
    WORKLOAD = (f"IF-RK4 vorticity step, {NX}^2, {precision.upper()}, dt={p['dt']:g}, "
                f"{'1/2-rule' if p['dealias'] == 'half' else 'reference-mask'} dealiasing, band-limited seed {SEED}")


def workload_config():
    """The workload both arms time (the reference arm prints the same dict)."""
    n, _ = world()
    return {"workload": WORKLOAD, "nx": NX, "ny": NY, "dt": PARAMS["dt"], "dealias": PARAMS["dealias"],
            "precision": PRECISION, "seed": SEED,
            "parallelism": "single GPU" if n == 1 else f"{n} independent replicas (one simulation per GPU, no exchange)",
            "l2": "flushed before every timed step (256 MB write)"}


def ncu_traffic(kernel_key):
    """DRAM read + write bytes per launch of the dominant kernel for this
    workload, from the committed ncu summary of the current build
    (profiles/ncu_traffic_<workload>.txt, lines "<kernel>_dram_bytes_per_launch:
    <bytes>" and "build: <commit>").  None where no capture covers the workload."""
    name = f"ncu_traffic_{NX}x{NY}_{PRECISION}.txt"
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None, None
    vals, build = {}, None
    with open(path) as f:
        for line in f:
            if ":" not in line:
                continue
            k, v = line.split(":", 1)
            k, v = k.strip(), v.strip()
            if k == "build":
                build = v
            elif k.endswith("_dram_bytes_per_launch"):
                try:
                    vals[k[: -len("_dram_bytes_per_launch")]] = float(v.split()[0])
                except ValueError:
                    pass
    return vals.get(kernel_key), f"profiles/{name} (build {build})" if build else f"profiles/{name}"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.p = None
        self.lines = []

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0],
                                       "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.p = None

    def _read(self):
        for line in self.p.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.p is None:
            return None
        time.sleep(0.25)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def oracle_steps(nsteps, threads=0):
    """Time `nsteps` full oracle steps of the workload on host cores."""
    import numpy as np
    import oracle
    from oracle.ic import bandlimited
    w0 = bandlimited(NX, NY, SEED).astype(np.complex64 if PRECISION == "fp32" else np.complex128)
    p = oracle.make_params(NX, NY, PARAMS["lx"], PARAMS["ly"], PARAMS["dt"], PARAMS["lam"], PARAMS["alpha"],
                           PARAMS["beta"], PARAMS["gamma0"], PARAMS["gamma2"], dealias=PARAMS["dealias"])
    t = time.perf_counter()
    oracle.run(p, w0, (0.0, 0.0), nsteps, "f32" if PRECISION == "fp32" else "f64", nthreads=threads)
    return time.perf_counter() - t, oracle.num_threads() if threads == 0 else threads


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    oracle.lib()
    for _ in range(args.warmup):
        oracle_steps(1)
    times = []
    cores = 1
    for _ in range(args.steps):
        dt, cores = oracle_steps(1)
        times.append(dt)
    total = sum(times)
    value = NX * NY * args.steps / total
    out = {
        "impl": "reference", "metric": "grid-point-steps/s", "value": value, "unit": "grid-point-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if PRECISION == "fp32" else "f64", "data": "synthetic",
        "config": workload_config(),
        "cpu_baseline": {"value": value, "unit": "grid-point-steps/s", "cores": cores, "kind": "port",
                         "sample": f"{args.steps} full {NX}x{NY} steps of the oracle (C restatement of "
                                   f"ActFlow_V3-2.cu's step, OpenMP), {PRECISION.upper()}"},
        "e2e": {"value": value, "unit": "grid-point-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def run_ours(args):
    import importlib

    import numpy as np
    import torch

    am = importlib.import_module("2d_active_matter_simulation_gb300")
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    # column-pass launch shape chosen by the autotuner on this GPU (untimed)
    tune = am.autotune(am.make_params(NX, NY, PARAMS["lx"], PARAMS["ly"], PARAMS["dt"], PARAMS["lam"],
                                      PARAMS["alpha"], PARAMS["beta"], gamma0=PARAMS["gamma0"],
                                      gamma2=PARAMS["gamma2"], dealias=PARAMS["dealias"], precision=PRECISION),
                       nsteps=10)
    cdt = np.complex64 if PRECISION == "fp32" else np.complex128
    w0 = am.ic_bandlimited(NX, NY, SEED).astype(cdt)

    def new_sim():
        sm = am.Solver(NX, NY, PARAMS["lx"], PARAMS["ly"], PARAMS["dt"], PARAMS["lam"], PARAMS["alpha"],
                       PARAMS["beta"], gamma0=PARAMS["gamma0"], gamma2=PARAMS["gamma2"], dealias=PARAMS["dealias"],
                       precision=PRECISION)
        sm.set_stream(stream.cuda_stream)
        sm.set_state(w0, (0.0, 0.0))
        return sm

    # The autotuner times back-to-back steps with the fields resident in L2
    # (the production case).  The timed region below flushes the L2 before
    # every step, so the column shapes are re-timed under that condition
    # (untimed, 10 flushed steps each) and the fastest there is used.
    flushed = {}
    for shape in tune[0]:
        am.set_column_shape(PRECISION, NY, shape)
        trial = new_sim()
        trial.step_async(3)
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(10)]
        with torch.cuda.stream(stream):
            for a_, b_ in evs:
                flush.zero_()
                a_.record(stream)
                trial.step_async(1)
                b_.record(stream)
        stream.synchronize()
        flushed[shape] = sum(a_.elapsed_time(b_) for a_, b_ in evs) / len(evs)
        trial.close()
    col_shape = min(flushed, key=flushed.get)
    am.set_column_shape(PRECISION, NY, col_shape)
    sim = new_sim()

    # warm-up
    sim.step_async(max(args.warmup, 0))
    sim.sync()

    # ---- value: device-resident, CUDA events on the solver's stream
    clocks = ClockSampler()
    clocks.start()
    torch.cuda.synchronize()
    replica_barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.zero_()
            ev[i][0].record(stream)
            sim.step_async(1)
            ev[i][1].record(stream)
    stream.synchronize()
    torch.cuda.synchronize()
    ms = [a.elapsed_time(b) for a, b in ev]
    clk = clocks.stop()
    sim.sync()
    replica_barrier()
    nrep, rank = world()
    total_ms = replica_max(sum(ms))
    value = nrep * NX * NY * args.steps / (total_ms / 1e3)

    # ---- per-kernel times for the roofline (same stream, L2 flushed before
    # each replay, as in the timed steps): the step's four row passes alone as
    # one graph, timed like a step; the column passes are the rest of the step
    # (4 row + 4 column = the graph-timed step by construction)
    nprof = max(args.steps, 3)
    evr = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nprof)]
    sim.row_passes_async(1)   # builds the graph (untimed)
    with torch.cuda.stream(stream):
        for i in range(nprof):
            flush.zero_()
            evr[i][0].record(stream)
            sim.row_passes_async(1)
            evr[i][1].record(stream)
    stream.synchronize()
    rows_ms = sum(a.elapsed_time(b) for a, b in evr) / nprof
    row = np.full(4, rows_ms / 4 * nprof)
    col = np.full(4, (total_ms / args.steps - rows_ms) / 4 * nprof)
    H = NY * (NX // 2 + 1)                 # half-plane values per field
    kxc = sim.kx_carried                   # Nx/4 with pruned transforms, Nx/2 without
    Hc = NY * (kxc + 1)                    # values per field the passes move
    s = 8 if PRECISION == "fp32" else 16
    row_avg = row.sum() / (4 * nprof)
    col_avg = col.sum() / (4 * nprof)
    # algorithmic bytes per launch: row pass 5 fields (3 in, 2 out); column
    # pass 7, 8, 8, 7 fields in stages 1..4 (mean 7.5); fields of Hc values
    row_bytes = 5 * s * Hc
    col_bytes = 7.5 * s * Hc
    peak, peak_kind = peaks()
    if col.sum() >= row.sum():
        dom, dom_bytes, dom_ms, key = "column pass (FFT_y, stage update, Biot-Savart, IFFT_y)", col_bytes, col_avg, "col"
    else:
        dom, dom_bytes, dom_ms, key = "row pass (C2R_x, products, R2C_x)", row_bytes, row_avg, "row"
    achieved = dom_bytes / (dom_ms / 1e3) / 1e9
    step_bytes = 50 * s * Hc
    step_achieved = step_bytes / (total_ms / args.steps / 1e3) / 1e9
    full_step_achieved = 50 * s * H / (total_ms / args.steps / 1e3) / 1e9

    # ---- e2e through the C ABI with host buffers (pinned)
    tdt = torch.complex64 if PRECISION == "fp32" else torch.complex128
    w_host = torch.empty((NY, NX // 2 + 1), dtype=tdt, pin_memory=True)
    w_host.numpy()[:] = w0
    w_out = torch.empty((NY, NX // 2 + 1), dtype=tdt, pin_memory=True)
    e_out = torch.empty(args.steps, dtype=torch.float64, pin_memory=True)
    wh, wo, eo = w_host.numpy(), w_out.numpy(), e_out.numpy()
    import ctypes
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    m = np.zeros(2)
    am._check(am.lib.am_set_state(sim.h, wh.ctypes.data, am._dptr(np.zeros(2))), sim.h, "set_state")
    nan_at = ctypes.c_int(-1)
    am._check(am.lib.am_step(sim.h, args.steps, eo.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                             ctypes.byref(nan_at)), sim.h, "step")
    am._check(am.lib.am_get_state(sim.h, wo.ctypes.data, am._dptr(m)), sim.h, "get_state")
    e2e_s = replica_max(time.perf_counter() - t0)
    e2e_value = nrep * NX * NY * args.steps / e2e_s
    state_bytes = H * s
    launches = sim.launches_per_step * args.steps
    sim.close()

    # ---- the FP64-class paths on the same workload (headline only): FP64 and
    # double-float, timed like the steps above (L2 flushed, CUDA events), and
    # how far apart their states are after those steps
    paths = None
    if not args.no_compare and nrep == 1 and PRECISION == "fp32" and NX == 2048 and NY == 2048:
        paths = precision_paths(am, stream, flush, max(args.steps, 10))

    # ---- CPU baseline: the oracle on the host cores, bounded sample
    cpu = None
    if not args.no_cpu and PRECISION == "fp32" and nrep == 1:
        n_cpu = 0
        t_cpu = 0.0
        cores = 1
        while t_cpu < 10.0 and n_cpu < 200:
            dt, cores = oracle_steps(1)
            t_cpu += dt
            n_cpu += 1
        cpu = {"value": NX * NY * n_cpu / t_cpu, "unit": "grid-point-steps/s", "cores": cores, "kind": "port",
               "sample": f"{n_cpu} full {NX}x{NY} steps of the oracle (C restatement of the reference step, "
                         f"OpenMP, FP32), {t_cpu:.1f} s"}

    # ---- the reference's own cuFFT build and the cuFFT floor on this GPU
    # (the headline workload only; rank 0 of a single-GPU run)
    compare = {}
    if not args.no_compare and nrep == 1 and NX == 2048 and NY == 2048 and PRECISION == "fp32":
        from baseline import reference_gpu
        for key_, fn in (("reference_gpu", reference_gpu.time_reference), ("cufft_floor", reference_gpu.time_floor)):
            try:
                compare[key_] = fn(NX, steps=200)
            except Exception as exc:   # a comparator that fails is reported, never fatal
                compare[key_] = {"unavailable": f"{type(exc).__name__}: {exc}"[:300]}
        for key_ in ("reference_gpu", "cufft_floor"):
            if "value" in compare.get(key_, {}):
                compare[key_]["speedup_of_e2e"] = e2e_value / compare[key_]["value"]
                compare[key_]["speedup_of_value"] = value / compare[key_]["value"]

    traffic, traffic_src = ncu_traffic(key) if kxc == NX // 4 else (None, None)
    out = {
        "metric": "grid-point-steps/s", "value": value, "unit": "grid-point-steps/s", "n_gpus": nrep,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": DTYPES[PRECISION], "data": "synthetic",
        "config": workload_config(),
        "timing": "CUDA events on the solver stream, one CUDA graph (8 kernels) per step",
        "tuning": {"column_shape": col_shape, "autotune_column_shape": tune[1], "autotune_ms_per_step": tune[0],
                   "flushed_ms_per_step": flushed, "row_shape": tune[3], "autotune_row_ms_per_step": tune[2]},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "traffic_source": traffic_src, "kernel": dom,
                     "algorithmic_bytes_per_launch": dom_bytes,
                     "avg_launch_ms": dom_ms, "peak_source": peak_kind,
                     "kernel_timing": "row pass: the step's 4 row passes alone as one graph, CUDA events, L2 "
                                      "flushed per replay; column pass: (step - 4 row passes) / 4",
                     "row_pass_ms": row_avg, "column_pass_ms": col_avg,
                     "step_achieved_gbs": step_achieved, "step_frac": step_achieved / peak,
                     "kx_carried": kxc, "pruned": kxc < NX // 2,
                     "full_transform_bytes_per_step": 50 * s * H,
                     "full_transform_equiv_gbs": full_step_achieved},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "grid-point-steps/s", "h2d_bytes_per_step": state_bytes / args.steps,
                "d2h_bytes_per_step": (state_bytes + 8 * args.steps) / args.steps,
                "path": "am_set_state (pinned host) + am_step(K, energy to host) + am_get_state (pinned host)"},
        "gpu_launches": launches,
        "clocks": clk,
    }
    if paths is not None:
        out["precision_paths"] = paths
    out.update(compare)
    if world()[1] == 0:
        print(json.dumps(out), flush=True)


def run_profile_case(args):
    """The workload's step, untimed, for profilers: the seeded field loaded
    with the launch shapes given (no autotuning), then args.steps steps.  The
    kernels run in the order set-up column pass, then (row pass, column pass
    stage s) for s = 1..4 per step."""
    import importlib

    import numpy as np

    am = importlib.import_module("2d_active_matter_simulation_gb300")
    col, row = args.profile_case.split(",")
    am.set_column_shape(PRECISION, NY, col)
    am.set_row_shape(PRECISION, NX, row)
    sim = am.Solver(NX, NY, PARAMS["lx"], PARAMS["ly"], PARAMS["dt"], PARAMS["lam"], PARAMS["alpha"], PARAMS["beta"],
                    gamma0=PARAMS["gamma0"], gamma2=PARAMS["gamma2"], dealias=PARAMS["dealias"], precision=PRECISION)
    w0 = am.ic_bandlimited(NX, NY, SEED)
    sim.set_state(w0.astype(np.complex64) if PRECISION == "fp32" else w0, (0.0, 0.0))
    if args.profile_flush:
        import torch
        stream = torch.cuda.Stream()
        sim.set_stream(stream.cuda_stream)
        flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
        with torch.cuda.stream(stream):
            for _ in range(args.steps):
                flush.zero_()
                sim.step_async(1)
        sim.sync()
        e = np.zeros(0)
    else:
        e = sim.step(args.steps)
    sim.close()
    print(json.dumps({"profile_case": {"workload": WORKLOAD, "column_shape": col, "row_shape": row,
                                       "steps": args.steps, "energy_last": float(e[-1]) if len(e) else None}}),
          flush=True)


def precision_paths(am, stream, flush, nsteps):
    """ms per step of the FP64 and double-float paths on the headline workload
    (seeded field, default launch shapes, L2 flushed before every step) and
    the relative L2 distance of the two states after nsteps + 3 steps."""
    import numpy as np
    import torch

    w0 = am.ic_bandlimited(NX, NY, SEED)
    out, states = {}, {}
    for prec in ("fp64", "df64"):
        sim = am.Solver(NX, NY, PARAMS["lx"], PARAMS["ly"], PARAMS["dt"], PARAMS["lam"], PARAMS["alpha"],
                        PARAMS["beta"], gamma0=PARAMS["gamma0"], gamma2=PARAMS["gamma2"], dealias=PARAMS["dealias"],
                        precision=prec)
        sim.set_stream(stream.cuda_stream)
        sim.set_state(w0, (0.0, 0.0))
        sim.step_async(3)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nsteps)]
        with torch.cuda.stream(stream):
            for a_, b_ in ev:
                flush.zero_()
                a_.record(stream)
                sim.step_async(1)
                b_.record(stream)
        stream.synchronize()
        ms = sum(a_.elapsed_time(b_) for a_, b_ in ev) / nsteps
        states[prec] = sim.get_state()[0]
        sim.close()
        out[prec] = {"ms_per_step": ms, "value": NX * NY / (ms / 1e3), "dtype": DTYPES[prec]}
    out["df64_speedup_over_fp64"] = out["fp64"]["ms_per_step"] / out["df64"]["ms_per_step"]
    out["df64_vs_fp64_rel_l2"] = float(np.linalg.norm(states["df64"] - states["fp64"]) /
                                       np.linalg.norm(states["fp64"]))
    out["steps_compared"] = nsteps + 3
    return out


def run_accuracy(args):
    """Precision form: the FP32 path (bulk FFT and products in FP32, integrating
    factors computed in double and rounded, mean flow and reductions in double
    or compensated FP32) and the double-float path against the FP64 path.

    Short horizon: relative L2 of w_hat after 200 steps from the seeded field.
    Long horizon: the time-mean energy and the time-averaged shell spectrum
    (snapshots every 200 steps) over a window of the saturated flow.  With
    --acc-spinup S the FP64 path first runs S steps from the seeded field and
    every long run starts from that state (FP32 from it rounded); the window is
    then the whole run of --acc-steps steps.  Without it the window is the
    second half of a run from the seeded field.  The flow is chaotic, so the
    two precisions agree only statistically: --acc-twins FP64 runs from the
    same state perturbed by one part in 1e12 (a different seeded perturbation
    per twin) measure the spread of the flow itself, and the FP32 differences
    are read against the largest twin difference (the envelope)."""
    import importlib

    import numpy as np

    am = importlib.import_module("2d_active_matter_simulation_gb300")
    spec = importlib.import_module("2d_active_matter_simulation_gb300.spectrum")
    n_total = args.acc_steps
    w0 = am.ic_bandlimited(NX, NY, SEED)

    def solver(prec):
        return am.Solver(NX, NY, PARAMS["lx"], PARAMS["ly"], PARAMS["dt"], PARAMS["lam"], PARAMS["alpha"],
                         PARAMS["beta"], gamma0=PARAMS["gamma0"], gamma2=PARAMS["gamma2"],
                         dealias=PARAMS["dealias"], precision=prec)

    res = {"if_factors": "double, rounded (auto)"}
    # short horizon from the seeded field
    short = {}
    for prec in ("fp32", "fp64", "df64"):
        sim = solver(prec)
        sim.set_state(w0 if prec != "fp32" else w0.astype(np.complex64))
        sim.step(200)
        short[prec] = sim.get_state()[0].astype(np.complex128)
        sim.close()
    res["short_horizon_steps"] = 200
    res["w_rel_l2_200"] = float(np.linalg.norm(short["fp32"] - short["fp64"]) / np.linalg.norm(short["fp64"]))
    res["w_rel_l2_200_df64"] = float(np.linalg.norm(short["df64"] - short["fp64"]) / np.linalg.norm(short["fp64"]))

    # start of the long runs
    t0 = time.perf_counter()
    if args.acc_spinup > 0:
        sim = solver("fp64")
        sim.set_state(w0)
        sim.step(args.acc_spinup, energy=False)
        s0, m0 = sim.get_state()
        sim.close()
        window_from = 0
    else:
        s0, m0 = w0, np.zeros(2)
        window_from = n_total // 2
    res["spinup_steps"] = args.acc_spinup
    res["spinup_seconds"] = time.perf_counter() - t0

    rng = np.random.default_rng(1234)
    runs = {}
    names = ["fp32", "fp64", "df64"] + [f"twin{i}" for i in range(args.acc_twins)]
    for name in names:
        if name.startswith("twin"):
            # one part in 1e12 per mode, Hermitian on the kx = 0 column
            r = rng.standard_normal(s0.shape)
            r[:, 0] = 0.5 * (r[:, 0] + r[(-np.arange(NY)) % NY, 0])
            start_w = s0 * (1.0 + 1e-12 * r)
        else:
            start_w = s0.astype(np.complex64) if name == "fp32" else s0
        sim = solver(name if name in ("fp32", "df64") else "fp64")
        sim.set_state(start_w, m0)
        t1 = time.perf_counter()
        e, specs, done = [], [], 0
        while done < n_total:
            k = min(200, n_total - done)
            e.append(sim.step(k))
            done += k
            if done > window_from:
                w, m = sim.get_state()
                specs.append(spec.energy_spectrum(w.astype(np.complex128), m, NX, NY, PARAMS["lx"], PARAMS["ly"])[1])
        runs[name] = dict(energy=np.concatenate(e), spec=np.mean(specs, axis=0), seconds=time.perf_counter() - t1)
        sim.close()

    kmax = NX // 4   # shells carried by the 1/2 rule
    ref = runs["fp64"]
    e_ref = float(np.mean(ref["energy"][window_from:]))
    s_ref = ref["spec"][: kmax + 1]

    def diffs(run):
        me = float(np.mean(run["energy"][window_from:]))
        sa = run["spec"][: kmax + 1]
        return {"mean_energy": me, "mean_energy_rel_diff": abs(me / e_ref - 1),
                "spectrum_l1_rel_diff": float(np.sum(np.abs(sa - s_ref)) / np.sum(s_ref)),
                "spectrum_max_rel_diff": spec.spectrum_rel_error(run["spec"], ref["spec"], kmax)}

    res["long_horizon_steps"] = n_total
    res["window_steps"] = [args.acc_spinup + window_from, args.acc_spinup + n_total]
    res["mean_energy_fp64"] = e_ref
    res["fp32"] = diffs(runs["fp32"])
    res["df64"] = diffs(runs["df64"])
    res["twins"] = [diffs(runs[f"twin{i}"]) for i in range(args.acc_twins)]
    if res["twins"]:
        env_e = max(t["mean_energy_rel_diff"] for t in res["twins"])
        env_s = max(t["spectrum_l1_rel_diff"] for t in res["twins"])
        res["twin_envelope"] = {"mean_energy_rel_diff": env_e, "spectrum_l1_rel_diff": env_s}
        res["fp32_within_target"] = {
            "mean_energy": res["fp32"]["mean_energy_rel_diff"] <= max(0.01, env_e),
            "spectrum_l1": res["fp32"]["spectrum_l1_rel_diff"] <= max(0.01, env_s)}
        res["df64_within_envelope"] = {
            "mean_energy": res["df64"]["mean_energy_rel_diff"] <= env_e,
            "spectrum_l1": res["df64"]["spectrum_l1_rel_diff"] <= env_s}
    res["energy_fp64_first_last"] = [float(ref["energy"][0]), float(ref["energy"][-1])]
    res["seconds"] = {k: v["seconds"] for k, v in runs.items()}
    res["gps_fp64"] = NX * NY * n_total / runs["fp64"]["seconds"]
    res["gps_fp32"] = NX * NY * n_total / runs["fp32"]["seconds"]
    res["gps_df64"] = NX * NY * n_total / runs["df64"]["seconds"]
    print(json.dumps({"accuracy": res, "config": {"workload": WORKLOAD}}), flush=True)


def run_batch(args):
    """Config 2: the ensemble advanced by am_batch; value = all members' grid-point-steps/s."""
    import importlib

    import numpy as np
    import torch

    am = importlib.import_module("2d_active_matter_simulation_gb300")
    nb = PRESETS[2]["members"]
    rng = np.random.default_rng(2)
    params = []
    for i in range(nb):
        alpha = float(rng.uniform(-1.0, -0.3))
        lam = float(rng.uniform(2.0, 5.0))
        params.append(am.make_params(NX, NY, PARAMS["lx"], PARAMS["ly"], PARAMS["dt"], lam, alpha, PARAMS["beta"],
                                     gamma0=PARAMS["gamma0"], gamma2=PARAMS["gamma2"], dealias=PARAMS["dealias"]))
    tune = am.autotune(params[0], nsteps=10)   # column-pass launch shape for 512^2 on this GPU
    batch = am.Batch(params)
    w0 = [am.ic_bandlimited(NX, NY, SEED + i).astype(np.complex64) for i in range(nb)]
    for i in range(nb):
        batch.set_state(i, w0[i])
    batch.step(args.warmup, energy=False)
    clocks = ClockSampler()
    clocks.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    batch.step(args.steps, energy=True)   # energies of every member read back each chunk
    dt = time.perf_counter() - t0
    clk = clocks.stop()
    value = nb * NX * NY * args.steps / dt
    batch.close()
    out = {
        "metric": "grid-point-steps/s", "value": value, "unit": "grid-point-steps/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"ensemble of {nb} x {NX}^2, FP32, dt={PARAMS['dt']:g}, 1/2 rule, one batch",
                   "members": nb, "timing": "host wall clock around am_batch_step (graph per step, energies "
                                            "of all members copied back per chunk)",
                   "column_shape": tune[1], "autotune_ms_per_step": tune[0], "row_shape": tune[3],
                   "autotune_row_ms_per_step": tune[2]},
        "gpu_launches": 8 * args.steps, "clocks": clk,
    }
    print(json.dumps(out), flush=True)


def _drawn_params(am, rng, nx, precision="fp32"):
    """alpha ~ U[-1, -0.3], lambda ~ U[2, 5], beta, Gamma0, Gamma2 as config 0, 2 pi box,
    dt = 0.1 dx / u_est with u_est = sqrt(-alpha / beta)."""
    alpha = float(rng.uniform(-1.0, -0.3))
    lam = float(rng.uniform(2.0, 5.0))
    dt = 0.1 * (2 * math.pi / nx) / math.sqrt(-alpha / PARAMS["beta"])
    return am.make_params(nx, nx, PARAMS["lx"], PARAMS["ly"], dt, lam, alpha, PARAMS["beta"],
                          gamma0=PARAMS["gamma0"], gamma2=PARAMS["gamma2"], dealias="half", precision=precision)


def run_ragged(args):
    """Config 3: 40 runs of mixed grids and step counts advanced by one am_ragged
    to completion; value = all runs' grid-point-steps / wall time of am_ragged_run."""
    import importlib

    import numpy as np
    import torch

    am = importlib.import_module("2d_active_matter_simulation_gb300")
    nr = PRESETS[3]["runs"]
    rng = np.random.default_rng(3)
    sizes = [int(2 ** rng.integers(7, 11)) for _ in range(nr)]
    steps = [int(rng.integers(1000, 5001)) for _ in range(nr)]
    params = [_drawn_params(am, rng, n) for n in sizes]
    # column-pass launch shape per grid size, chosen by the autotuner on this GPU
    shapes = {}
    for n in sorted(set(sizes)):
        t = am.autotune(params[sizes.index(n)], nsteps=10)
        shapes[f"{n}^2"] = {"column": t[1], "row": t[3]}
    ics = [am.ic_bandlimited(n, n, 2000 + i).astype(np.complex64) for i, n in enumerate(sizes)]
    # warm-up: the same runs for `warmup` steps each
    warm = am.Ragged(params, [max(args.warmup, 1)] * nr)
    for i in range(nr):
        warm.set_state(i, ics[i])
    warm.run(energy=False)
    warm.close()
    # both ways of launching a step: one launch per pass over the size-sorted
    # work list, and one launch per size class per pass (the classes' tuned
    # shapes); the line's value is the faster, both are reported
    res = {}
    for mode in ("worklist", "per_class"):
        rg = am.Ragged(params, steps)
        rg.set_mode(mode)
        for i in range(nr):
            rg.set_state(i, ics[i])
        clocks = ClockSampler()
        clocks.start()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, gps = rg.run(energy=True)
        dt = time.perf_counter() - t0
        clk = clocks.stop()
        classes = rg.classes
        rg.close()
        res[mode] = dict(value=gps / dt, seconds=dt, gps=gps, clocks=clk)
    best = max(res, key=lambda m: res[m]["value"])
    hist = {f"{n}^2": sizes.count(n) for n in sorted(set(sizes))}
    out = {
        "metric": "grid-point-steps/s", "value": res[best]["value"], "unit": "grid-point-steps/s", "n_gpus": 1,
        "steps": int(sum(steps)), "warmup": args.warmup, "ms_per_step": None,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"ragged batch: {nr} runs, grids {hist}, steps U[1000,5000] (total "
                               f"{sum(steps)} run-steps), per-run dt, 1/2 rule, FP32",
                   "runs": nr, "size_classes": classes, "seconds": res[best]["seconds"],
                   "grid_point_steps": res[best]["gps"], "mode": best,
                   "modes": {m: {"value": v["value"], "seconds": v["seconds"]} for m, v in res.items()},
                   "tuned_shapes": shapes,
                   "timing": "host wall clock around am_ragged_run (one CUDA graph per step; worklist: 8 "
                             "launches per step over all sizes, per_class: 8 per size class as parallel "
                             "branches; energies of every run copied back per segment)"},
        "gpu_launches": _ragged_launches(sizes, steps, per_class=best == "per_class"), "clocks": res[best]["clocks"],
    }
    print(json.dumps(out), flush=True)


def _ragged_launches(sizes, steps, per_class=True):
    """Kernels am_ragged_run launches: per segment (steps up to the next run's
    end, at most 1024), 8 per step for each size class with active runs (per
    class) or 8 per step (work list), plus one step-counter reset."""
    done = [0] * len(steps)
    total = 0
    while True:
        act = [i for i in range(len(steps)) if done[i] < steps[i]]
        if not act:
            return total
        k = min(1024, min(steps[i] - done[i] for i in act))
        total += k * 8 * (len({sizes[i] for i in act}) if per_class else 1) + 1
        for i in act:
            done[i] += k


def _serving_trace(am, window_s, step_scale, rate, seed):
    import numpy as np
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t > window_s:
            return out
        n = int(2 ** rng.integers(7, 13))
        fp64 = bool(rng.uniform() < 0.1)
        steps = int(round(math.exp(rng.uniform(math.log(500), math.log(20000))) * step_scale))
        p = _drawn_params(am, rng, n, "fp64" if fp64 else "fp32")
        out.append((t, p, max(steps, 1), int(rng.integers(0, 2 ** 31))))


def _serve(am, trace, max_active, order):
    import numpy as np
    srv = am.Server(max_active=max_active, chunk_steps=256, order=order)
    t0 = time.perf_counter()
    ids = []
    for t, p, k, sd in trace:
        delay = t - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        ids.append(srv.submit(p, k, seed=sd, want_state=False, want_energy=False))
    res = [srv.wait(i) for i in ids]
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    lat = np.array([r["t_done"] - r["t_submit"] for r in res])
    bad = [r for r in res if r["status"] != am.AM_OK]
    gps = sum(p.nx * p.ny * k for _, p, k, _ in trace)
    return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "gps_per_s": gps / wall, "wall_s": wall, "failed": len(bad),
            "failures": [f"{trace[ids.index(r['id'])][1].nx}^2 "
                         f"{'FP64' if trace[ids.index(r['id'])][1].precision else 'FP32'}: {r['error']}"
                         for r in bad[:3]],
            "peak_active": st["peak_active"], "peak_device_gb": st["peak_device_bytes"] / 1e9}


def run_serving(args):
    """Config 4: a Poisson request trace through am_server (continuous batching)
    and, for comparison, through the same engine with one request at a time."""
    import importlib

    am = importlib.import_module("2d_active_matter_simulation_gb300")
    pre = PRESETS[4]
    # warm-up: a few small requests load every kernel once
    warm = _serving_trace(am, 2.0, 0.002, pre["rate"], 99)
    _serve(am, [(0.0, p, k, s) for _, p, k, s in warm], 16, "arrival")
    trace = _serving_trace(am, args.serve_seconds, args.serve_step_scale, pre["rate"], pre["seed"])
    clocks = ClockSampler()
    clocks.start()
    cb = _serve(am, trace, 16, "arrival")
    clk = clocks.stop()
    one = _serve(am, trace, 1, "arrival")
    nfp64 = sum(1 for _, p, _, _ in trace if p.precision == am.FP64)
    out = {
        "metric": "served p50/p99 job latency", "value": cb["p50_s"], "unit": "s", "n_gpus": 1,
        "steps": len(trace), "warmup": len(warm), "ms_per_step": None, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64", "data": "synthetic",
        "p50_s": cb["p50_s"], "p99_s": cb["p99_s"], "grid_point_steps_per_s": cb["gps_per_s"],
        "continuous_batching": cb, "one_at_a_time": one,
        "config": {"workload": f"serving trace: Poisson {pre['rate']:g}/s over {args.serve_seconds:g} s "
                               f"({len(trace)} requests, {nfp64} FP64), grids log-uniform 128^2..4096^2, steps "
                               f"log-uniform 500..20000 scaled by {args.serve_step_scale:g}, 1/2 rule",
                   "max_active": 16, "chunk_steps": 256, "hbm_budget_gb": 180 * 2 ** 30 / 1e9,
                   "timing": "latency = result ready - submit, on the server's clock; requests submitted "
                             "at their arrival times by a host thread"},
        "gpu_launches": 8 * sum(k for _, _, k, _ in trace), "clocks": clk,
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--no-compare", action="store_true",
                    help="skip timing the reference's cuFFT build and the cuFFT floor")
    ap.add_argument("--accuracy", action="store_true", help="FP32 vs FP64 precision-form check instead")
    ap.add_argument("--acc-steps", type=int, default=20000, help="accuracy: steps of each long run")
    ap.add_argument("--acc-spinup", type=int, default=0, help="accuracy: FP64 steps before the long runs")
    ap.add_argument("--acc-twins", type=int, default=4, help="accuracy: perturbed FP64 runs (chaotic spread)")
    ap.add_argument("--config", type=int, default=1, choices=sorted(PRESETS))
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64", "df64"])
    ap.add_argument("--n", type=int, default=0,
                    help="configs 0/1: grid size N (N x N) instead of the preset's, e.g. 4096 (fields exceed L2)")
    ap.add_argument("--serve-seconds", type=float, default=20.0, help="config 4: arrival window")
    ap.add_argument("--serve-step-scale", type=float, default=0.05, help="config 4: step-count scale")
    ap.add_argument("--profile-case", metavar="COL,ROW", default="",
                    help="configs 0/1: no timing; load the seeded field with the given column and row shapes "
                         "(e.g. wide8,lockstep) and run --steps steps: a short, deterministic command for ncu")
    ap.add_argument("--profile-flush", action="store_true",
                    help="with --profile-case: flush the L2 (256 MB write) before every step, as the timed region does")
    args = ap.parse_args()
    if args.impl == "ours":
        replica_setup()   # before torch or the solver touch a GPU
    if args.n and args.config not in (0, 1):
        ap.error("--n applies to configs 0 and 1")
    apply_preset(args.config, args.precision, args.n or None)
    if args.accuracy:
        run_accuracy(args)
        return
    if args.profile_case:
        if args.config not in (0, 1):
            ap.error("--profile-case applies to configs 0 and 1")
        run_profile_case(args)
        return
    if args.config in (2, 3, 4) and world()[1] != 0:
        return   # the ensemble, ragged and serving workloads run on one GPU (rank 0)
    if args.config == 2 and args.impl == "ours":
        run_batch(args)
        return
    if args.config == 3 and args.impl == "ours":
        run_ragged(args)
        return
    if args.config == 4 and args.impl == "ours":
        run_serving(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
