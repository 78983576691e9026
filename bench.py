#!/usr/bin/env python
"""Benchmark of the QMCToolsCL hot path on GB300.

Default workload (the headline configuration): rank-1 lattice in Gray order
plus a uniform random shift mod 1, r = 16 randomisations, n = 2^20 points,
d = 64 dimensions, float64 output (8 GiB per step), generating vector of
odd integers in [1, 2^20) and shifts U[0,1), both seeded
(np.random.SFC64(2)).  One step = one pass of the path over that batch:

  value  -- the fused batched kernel (qmc_lat_gen_shift: generation + shift in
            one launch, writes only the shifted points), inputs resident in HBM,
            timed with CUDA events on the launching stream;
  plain  -- the reference's two calls (lat_gen_gray then lat_shift_mod_1) as
            two launches with the intermediate array in HBM;
  e2e    -- the public API with host numpy buffers: host->device copy of the
            inputs, the kernel, device->host copy of the 8 GiB result into
            pinned host memory, every step.

The output (8 GiB) is far larger than L2 (129 MB), so no flush is needed
between steps.  cpu_baseline times the oracle (a C restatement of the
reference C backend) over all host cores on a sample of the same workload.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference's CPU implementation (the oracle port;
the reference's own compiled backend is not available on the GPU host) on
the same metric and workload.  Under torchrun (N>1) every rank runs its own
replica of the workload (weak scaling, no data exchange); rank 0 prints.
"""
import argparse
import concurrent.futures
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "points/s + % HBM roofline, batched vs plain on 1 GB300; FFT Gsamples/s @≤1e-6 err"
R, LOG2N, D = 16, 20, 64
PROFILE_LOG2N = 16  # --small: the same kernel on 512 MiB of output, for ncu captures
SEED = 2
FALLBACK_HBM_GBS = 6800.0
# DRAM bytes / algorithmic bytes of the two captured tensor-core FFT passes (n = 2^20, 24
# vectors, 48 B per sample): (403.5 + 155.5 + 202.1 + 341.8) MB / 1208.0 MB
TC_FFT_TRAFFIC_RATIO = 0.9131


def workload_inputs(seed=SEED):
    import qmctoolscl_gb300 as q
    rng = np.random.Generator(np.random.SFC64(seed))
    g = (rng.integers(0, 1 << 19, (R, D)) * 2 + 1).astype(np.uint64)
    shifts = q.lat_get_shifts(rng, R, D)
    return g, shifts


# ---------------------------------------------------------------- CPU side

def cpu_pipeline(g, shifts, n, threads, n_start=0, bufs=None):
    """The reference pipeline (Gray-order lattice, then shift mod 1) run by
    the oracle for rows n_start .. n_start+n-1, one randomisation per task
    over `threads` host threads; bufs = (x, xr) of shape (R, n, D) to reuse."""
    import oracle
    U = np.uint64
    x, xr = bufs if bufs is not None else (np.empty((R, n, D)), np.empty((R, n, D)))

    def one(l):
        oracle.call("lat_gen_gray", U(1), U(n), U(D), U(n_start), np.ascontiguousarray(g[l:l + 1]), x[l:l + 1])
        oracle.call("lat_shift_mod_1", U(1), U(n), U(D), U(1), x[l:l + 1], np.ascontiguousarray(shifts[l:l + 1]),
                    xr[l:l + 1])

    t0 = time.perf_counter()
    with concurrent.futures.ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(one, range(R)))
    return time.perf_counter() - t0, xr


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


CPU_SAMPLE_LOG2N = 18
REF_LOG2N = LOG2N  # rows per step of the reference arm: the whole workload


def cpu_baseline(g, shifts):
    """The whole workload (all 2^20 rows) on the host, in row ranges of
    2^18 through reused buffers (about 16 CPU-seconds on 16 cores)."""
    import oracle
    oracle.oracle_lib()
    threads = host_threads()
    n = 1 << CPU_SAMPLE_LOG2N
    parts = (1 << LOG2N) // n
    bufs = (np.empty((R, n, D)), np.empty((R, n, D)))
    cpu_pipeline(g, shifts, n, threads, 0, bufs)  # untimed: touches the buffers' pages, warms the pool
    t = sum(cpu_pipeline(g, shifts, n, threads, k * n, bufs)[0] for k in range(parts))
    return {"value": R * n * parts / t, "unit": "points/s", "cores": threads, "kind": "port",
            "sample": "the whole workload, r=16, n=2^%d, d=64, as %d row ranges of 2^%d (n_start = k*2^%d) "
                      "through reused buffers; lat_gen_gray then lat_shift_mod_1 by the oracle (C restatement "
                      "of the reference C backend, gcc -O2 -ffp-contract=off), one randomisation per thread"
                      % (LOG2N, parts, CPU_SAMPLE_LOG2N, CPU_SAMPLE_LOG2N),
            "seconds": t, "cpu_seconds": t * threads}


AS_SHIPPED_LOG2N = 16


def cpu_as_shipped(g, shifts):
    """The reference as its users run it today: one call per function, the
    whole r on one host thread (its C loops are serial), timed with
    perf_counter around each call as qmctoolscl/util.py:104-114 times it.
    Run on the first 2^16 rows (1/16 of the workload) and reported per point:
    the loops are linear in n."""
    import oracle
    U = np.uint64
    n = 1 << AS_SHIPPED_LOG2N
    x, xr = np.empty((R, n, D)), np.empty((R, n, D))
    oracle.call("lat_gen_gray", U(R), U(1 << 10), U(D), U(0), g, x)  # untimed: loads the library
    t0 = time.perf_counter()
    oracle.call("lat_gen_gray", U(R), U(n), U(D), U(0), g, x)
    t1 = time.perf_counter()
    oracle.call("lat_shift_mod_1", U(R), U(n), U(D), U(R), x, shifts, xr)
    t2 = time.perf_counter()
    return {"value": R * n / (t2 - t0), "unit": "points/s", "cores": 1, "kind": "port",
            "sample": "r=16, n=2^%d, d=64 (1/16 of the rows; per-point rate, the loops are linear in n): "
                      "lat_gen_gray then lat_shift_mod_1, one oracle call each over all r on one thread, "
                      "timed per call like qmctoolscl/util.py:104-114" % AS_SHIPPED_LOG2N,
            "seconds_per_call": {"lat_gen_gray": t1 - t0, "lat_shift_mod_1": t2 - t1},
            "extrapolated_full_step_s": (t2 - t0) * (1 << (LOG2N - AS_SHIPPED_LOG2N))}


# ---------------------------------------------------------------- clocks

class ClockSampler:
    FIELDS = ["index", "clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.active",
              "clocks_event_reasons.hw_slowdown", "clocks_event_reasons.hw_thermal_slowdown",
              "clocks_event_reasons.sw_thermal_slowdown", "clocks_event_reasons.sw_power_cap"]

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + ",".join(self.FIELDS),
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        rows = []
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) != len(self.FIELDS):
                continue
            try:
                rows.append({"sm": float(parts[1]), "max": float(parts[2]), "pw": float(parts[3]),
                             "hw": parts[5], "hwt": parts[6], "swt": parts[7], "pcap": parts[8]})
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        pmax = max(r_["pw"] for r_ in rows)
        load = [r_ for r_ in rows if r_["pw"] >= 0.5 * pmax] or rows
        reasons = set()
        for r_ in load:
            for key, name in (("hw", "hw_slowdown"), ("hwt", "hw_thermal_slowdown"),
                              ("swt", "sw_thermal_slowdown"), ("pcap", "sw_power_cap")):
                if r_[key].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median([r_["sm"] for r_ in load])), "sm_max_mhz": max(r_["max"] for r_ in rows),
                "reasons": sorted(reasons), "samples_under_load": len(load), "power_w_max": pmax}


# ---------------------------------------------------------------- helpers

def measured_peak():
    path = os.path.join(HERE, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback 6.8 TB/s"


def profiled_value(name, key):
    """The number after `key:` in the committed ncu summary profiles/<name>, or None."""
    path = os.path.join(HERE, "profiles", name)
    try:
        with open(path) as f:
            for ln in f:
                if ln.startswith(key + ":"):
                    return float(ln.split(":", 1)[1].split()[0])
    except (OSError, ValueError):
        pass
    return None


SMS = 152
FP64_LANES_PER_SM_CLK = 2  # GB300: 1.25 TFLOP/s FP64 = 2 FMA lanes per SM per clock at 2.07 GHz


def fp64_roofline(warp_inst, ms, sm_mhz):
    """Fraction of the FP64 pipe's issue rate: warp-level FP64 instructions
    (32 lanes each) against SMs x 2 lanes per clock at the sampled SM clock."""
    if warp_inst is None or not sm_mhz:
        return None
    lane_ops = 32.0 * warp_inst
    peak = SMS * FP64_LANES_PER_SM_CLK * sm_mhz * 1e6
    ach = lane_ops / (ms / 1e3)
    return {"bound": "fp64", "achieved": ach / 1e12, "peak": peak / 1e12, "unit": "T FP64 lane-ops/s",
            "frac": ach / peak, "fp64_warp_inst_per_launch": warp_inst, "sm_mhz": sm_mhz}


def profiled_traffic(name):
    """dram read+write bytes per launch of `name` from the committed ncu summary."""
    path = os.path.join(HERE, "profiles", name)
    try:
        with open(path) as f:
            for ln in f:
                if ln.startswith("traffic_bytes_per_launch:"):
                    return float(ln.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


def dist_setup(backend=None):
    """One process per GPU (torchrun environment); NCCL on GPUs, gloo for the
    CPU tests of the replica logic."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = backend or ("nccl" if torch.cuda.is_available() else "gloo")
        if backend == "nccl":
            torch.cuda.set_device(local)
            dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        else:
            dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- arms

def headline_config():
    """The headline workload, the same for both arms of the benchmark."""
    points = R * (1 << LOG2N)
    return {"workload": "rank-1 lattice Gray order + shift mod 1, r=16, n=2^20, d=64", "r": R, "n": 1 << LOG2N,
            "d": D, "points_per_step": points, "coords_per_step": points * D,
            "l2": "8 GiB output per step >> 129 MB L2, no flush needed"}


def run_reference(args):
    """The reference's CPU implementation of the path (the oracle port: its C backend restated,
    lat_gen_gray then lat_shift_mod_1) over all host threads, every step the whole workload as
    row ranges of 2^18 through reused buffers."""
    world, rank, _local = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), 0
    if rank != 0:
        return
    import oracle
    oracle.oracle_lib()
    g, shifts = workload_inputs()
    threads = host_threads()
    rows = 1 << REF_LOG2N
    n = min(1 << CPU_SAMPLE_LOG2N, rows)
    parts = rows // n
    bufs = (np.empty((R, n, D)), np.empty((R, n, D)))

    def step():
        return sum(cpu_pipeline(g, shifts, n, threads, k * n, bufs)[0] for k in range(parts))

    for _ in range(args.warmup):
        step()
    times = [step() for _ in range(args.steps)]
    ms = 1e3 * float(np.mean(times))
    value = R * n * parts / (ms / 1e3)
    line = {"metric": METRIC, "value": value, "unit": "points/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded np.random.SFC64(2))",
            "impl": "reference",
            "config": dict(headline_config(), parallelism="%d host threads" % threads,
                           kernel="the oracle port of the reference C backend, rows in ranges of 2^%d"
                                  % CPU_SAMPLE_LOG2N),
            "cpu_baseline": {"value": value, "unit": "points/s", "cores": threads, "kind": "port",
                             "sample": "the whole workload every step (r=16, n=2^20, d=64) as %d row ranges of "
                                       "2^%d through reused buffers, one randomisation per thread"
                                       % (parts, CPU_SAMPLE_LOG2N)},
            "e2e": {"value": value, "unit": "points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    from qmctoolscl_gb300 import _ffi, batch
    lib = _ffi.lib()
    n = 1 << (PROFILE_LOG2N if args.small else LOG2N)
    g, shifts = workload_inputs(SEED + 1000 * rank)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    h = stream.cuda_stream
    g_d = torch.from_numpy(g.view(np.int64)).to(dev)
    s_d = torch.from_numpy(shifts).to(dev)
    xr_d = torch.empty((R, n, D), dtype=torch.float64, device=dev)

    def fused():
        _ffi.check(lib.qmc_lat_gen_shift(R, n, D, 0, 1, g_d.data_ptr(), s_d.data_ptr(), xr_d.data_ptr(), h),
                   "lat_gen_shift")

    # parity spot check of this very launch configuration against the oracle
    fused()
    torch.cuda.synchronize()
    _, xr_sample = cpu_pipeline(g, shifts, 1 << 10, host_threads())
    assert np.array_equal(xr_d[:, :1 << 10].cpu().numpy().view(np.uint64), xr_sample.view(np.uint64)), \
        "fused kernel output differs from the oracle"

    clocks = ClockSampler(local)
    clocks.start()
    for _ in range(args.warmup):
        fused()
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        fused()
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    ms_fused = e0.elapsed_time(e1) / args.steps
    ms_fused_max = max_over_ranks(ms_fused, world)
    if args.small:  # profiling mode: the fused kernel only
        clocks.stop()
        if rank == 0:
            print(json.dumps({"small": True, "n": n, "ms_per_step": ms_fused_max,
                              "gbs": 8.0 * R * n * D / (ms_fused_max / 1e3) / 1e9}), flush=True)
        return None

    # plain: the reference's two calls as two launches
    x_d = torch.empty((R, n, D), dtype=torch.float64, device=dev)

    def plain():
        _ffi.check(lib.qmc_lat_gen_gray(R, n, D, 0, g_d.data_ptr(), x_d.data_ptr(), h), "lat_gen_gray")
        _ffi.check(lib.qmc_lat_shift_mod_1(R, n, D, R, x_d.data_ptr(), s_d.data_ptr(), xr_d.data_ptr(), h),
                   "lat_shift_mod_1")

    for _ in range(args.warmup):
        plain()
    torch.cuda.synchronize()
    barrier(world)
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    for _ in range(args.steps):
        plain()
    p1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    ms_plain = max_over_ranks(p0.elapsed_time(p1) / args.steps, world)
    clk = clocks.stop()
    del x_d

    # e2e: public API with host numpy buffers, transfers inside the timed
    # region every step: the inputs are copied host->device, the 8 GiB result
    # reaches the pinned host array either written by the kernel over the
    # CPU-GPU link (direct) or staged in HBM and copied back (staged)
    xr_host = batch.pinned_empty((R, n, D))
    e2e_steps = max(1, min(args.steps, 5))
    e2e = {}
    for mode, direct in (("direct", True), ("staged", False)):
        xr_host[:, :1 << 10] = 0.0
        batch.lattice_gen_shift(R, n, D, 0, g, shifts, xr_host, order="gray", direct_out=direct)  # warm-up
        torch.cuda.synchronize()
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            A = batch.lattice_gen_shift(R, n, D, 0, g, shifts, xr_host, order="gray", direct_out=direct)
        torch.cuda.synchronize()
        t_e2e = max_over_ranks((time.perf_counter() - t0) / e2e_steps, world)
        assert np.array_equal(xr_host[:, :1 << 10].view(np.uint64), xr_sample.view(np.uint64))
        e2e[mode] = {"value": world * R * n / t_e2e, "unit": "points/s", "h2d_bytes_per_step": A.h2d_bytes,
                     "d2h_bytes_per_step": A.d2h_bytes, "steps": e2e_steps, "ms_per_step": 1e3 * t_e2e,
                     "direct_host_write": A.direct}
    best = max(e2e, key=lambda k: e2e[k]["value"])
    e2e_line = dict(e2e[best])
    e2e_line["path"] = ("qmctoolscl_gb300.batch.lattice_gen_shift with numpy inputs and a pinned numpy output, "
                        "%s" % ("written by the kernel over NVLink-C2C" if best == "direct"
                                else "staged in HBM and copied back"))
    e2e_line["other"] = {k: v for k, v in e2e.items() if k != best}
    # the CPU-GPU link's own rate for the same bytes: one device-to-host copy of the result
    # into the same pinned array (the e2e path cannot beat it)
    xr_t = torch.from_numpy(xr_host.reshape(-1))
    xr_t.copy_(xr_d.reshape(-1), non_blocking=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    xr_t.copy_(xr_d.reshape(-1), non_blocking=True)
    torch.cuda.synchronize()
    t_link = time.perf_counter() - t0
    link_gbs = 8.0 * R * n * D / t_link / 1e9
    e2e_line["link"] = {"d2h_copy_ms": 1e3 * t_link, "d2h_gbs": link_gbs,
                        "e2e_d2h_gbs": e2e_line["d2h_bytes_per_step"] / (e2e_line["ms_per_step"] / 1e3) / 1e9,
                        "note": "plain device-to-host copy of the same result into the same pinned array"}
    del xr_t, xr_host
    # what a reference user's code does unchanged: lat_gen_gray then lat_shift_mod_1 through
    # the drop-in API with numpy arrays (pageable), every array copied in and out by each call
    e2e_line["other"]["drop_in"] = drop_in_e2e(g, shifts, n, xr_sample, world)

    if rank != 0:
        return None
    points = R * n
    value = world * points / (ms_fused_max / 1e3)
    peak, peak_src = measured_peak()
    alg_bytes = 8.0 * R * n * D  # each coordinate written once as a float64
    achieved = alg_bytes / (ms_fused / 1e3) / 1e9
    traffic = profiled_traffic("lat_gen_shift_kernel_r16_n2p20_d64.md")
    line = {
        "metric": METRIC, "value": value, "unit": "points/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_fused_max, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded np.random.SFC64(2); odd g in [1,2^20), "
                                                     "shifts U[0,1))",
        "config": dict(headline_config(), parallelism="replicas" if world > 1 else "1 GPU",
                       kernel="the fused batched kernel (lat_gen_kernel<ORDER_GRAY,SHIFT>)"),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_source": peak_src,
                     "kernel": "lat_gen_kernel<ORDER_GRAY,SHIFT> (qmc_lat_gen_shift)",
                     "alg_bytes_per_launch": alg_bytes},
        "plain": {"ms_per_step": ms_plain, "points_per_s": world * points / (ms_plain / 1e3), "launches_per_step": 2,
                  "alg_bytes_per_step": 24.0 * R * n * D,
                  "achieved_gbs": 24.0 * R * n * D / (ms_plain / 1e3) / 1e9,
                  "fused_speedup": ms_plain / ms_fused_max},
        "e2e": e2e_line,
        "gpu_launches": args.steps,
        "clocks": clk,
        "cpu_baseline": cpu_baseline(g, shifts),
        "cpu_as_shipped": cpu_as_shipped(g, shifts),
    }
    return line


def drop_in_e2e(g, shifts, n, xr_sample, world):
    """lat_gen_gray then lat_shift_mod_1 through qmctoolscl_gb300's drop-in
    functions with numpy arrays, as the reference's documented use calls them;
    each call copies its inputs to the GPU and its outputs back (8 GiB out of
    lat_gen_gray, 8 GiB in and 8 GiB out of lat_shift_mod_1)."""
    import torch
    import qmctoolscl_gb300 as q
    U = np.uint64
    x, xr = np.empty((R, n, D)), np.empty((R, n, D))
    x[:] = 0.0  # touch the pages outside the timed region, as a caller's reused arrays are
    xr[:] = 0.0
    q.lat_gen_gray(U(R), U(n), U(D), U(0), g, x)  # warm-up
    steps = 2
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(steps):
        q.lat_gen_gray(U(R), U(n), U(D), U(0), g, x)
        q.lat_shift_mod_1(U(R), U(n), U(D), U(R), x, shifts, xr)
    t = max_over_ranks((time.perf_counter() - t0) / steps, world)
    assert np.array_equal(xr[:, :1 << 10].view(U), xr_sample.view(U)), "drop-in calls differ from the oracle"
    nb = 8 * R * n * D
    return {"value": world * R * n / t, "unit": "points/s", "ms_per_step": 1e3 * t, "steps": steps,
            "h2d_bytes_per_step": g.nbytes + shifts.nbytes + nb, "d2h_bytes_per_step": 2 * nb,
            "path": "qmctoolscl_gb300.lat_gen_gray then qmctoolscl_gb300.lat_shift_mod_1, numpy arrays in "
                    "pageable memory, copies inside each call"}


# ---------------------------------------------------------------- other configurations

def gpu_ms(fn, steps, warmup, stream):
    """Average milliseconds per call of fn, CUDA events on `stream`."""
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def graph_ms(fn_h, steps, warmup):
    """Average milliseconds per call of fn_h(stream_handle) when `steps` calls
    are captured in one CUDA graph and replayed: the device time of a
    workload too small to cover its host launch overhead (CUDA events on the
    replay stream)."""
    import torch
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(warmup):
            fn_h(side.cuda_stream)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=side):
        for _ in range(steps):
            fn_h(side.cuda_stream)
    g.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(side):
        e0.record(side)
        g.replay()
        e1.record(side)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def dev_tensor(a):
    import torch
    a = np.ascontiguousarray(a)
    return torch.from_numpy(a.view(np.int64) if a.dtype == np.uint64 else a).cuda()


def triangular_net_matrices(rng, d, m, tbits):
    """d generating matrices of m columns with tbits rows, MSB first: dimension 0
    the identity, the others random upper-unit-triangular (seeded)."""
    C = np.zeros((1, d, m), np.uint64)
    for j in range(d):
        M = np.eye(tbits, m, dtype=np.uint64)
        if j > 0:
            M = M + np.triu(rng.integers(0, 2, (tbits, m)), 1).astype(np.uint64)
        for k in range(m):
            v = 0
            for t in range(tbits):
                if M[t, k]:
                    v |= 1 << (63 - t if tbits == 64 else 62 - t)
            C[0, j, k] = v
    return C


def roofline(alg_bytes, ms):
    peak, src = measured_peak()
    ach = alg_bytes / (ms / 1e3) / 1e9
    return {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak, "traffic": None,
            "peak_source": src, "alg_bytes_per_launch": alg_bytes}


def run_net_plain(args):
    """Base-2 digital net, natural order + digital shift + float: r=1, d=16,
    m=16 (n=65536), tmax=63."""
    import torch
    import qmctoolscl_gb300 as q
    from qmctoolscl_gb300 import _ffi
    lib = _ffi.lib()
    rng = np.random.Generator(np.random.SFC64(1))
    r, d, m = 1, 16, 16
    n = 1 << m
    C = triangular_net_matrices(rng, d, m, 63)
    shifts = q.dnb2_get_digital_shifts(rng, r, d, 63)
    lsh, tm = np.zeros(r, np.uint64), np.full(r, 63, np.uint64)
    Cd, sd, ld, td = dev_tensor(C), dev_tensor(shifts), dev_tensor(lsh), dev_tensor(tm)
    xb = torch.empty(r * n * d, dtype=torch.int64, device="cuda")
    xrb = torch.empty_like(xb)
    x = torch.empty(r * n * d, dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream()
    h = st.cuda_stream

    def plain_on(hs):
        _ffi.check(lib.qmc_dnb2_gen_natural(r, n, d, 0, m, Cd.data_ptr(), xb.data_ptr(), hs), "gen")
        _ffi.check(lib.qmc_dnb2_digital_shift(r, n, d, r, ld.data_ptr(), xb.data_ptr(), sd.data_ptr(),
                                              xrb.data_ptr(), hs), "shift")
        _ffi.check(lib.qmc_dnb2_integer_to_float(r, n, d, td.data_ptr(), xrb.data_ptr(), x.data_ptr(), hs), "float")

    def fused_on(hs):
        _ffi.check(lib.qmc_dnb2_gen_fused(r, n, d, 0, m, Cd.data_ptr(), r, 0, ld.data_ptr(), r, sd.data_ptr(),
                                          td.data_ptr(), xrb.data_ptr(), x.data_ptr(), hs), "fused")

    # one call per step from Python (the host's launch overhead is inside: 16.8 MB is about 2.5 us of
    # HBM time), and the same calls replayed from one captured CUDA graph (the device's time)
    ms_plain_eager = gpu_ms(lambda: plain_on(h), args.steps, args.warmup, st)
    ms_fused_eager = gpu_ms(lambda: fused_on(h), args.steps, args.warmup, st)
    graph_steps = max(args.steps, 20)
    ms_plain = graph_ms(plain_on, graph_steps, args.warmup)
    ms_fused = graph_ms(fused_on, graph_steps, args.warmup)
    # parity of the timed outputs against the oracle chain
    import oracle
    U = np.uint64
    o_xb = np.empty((r, n, d), U)
    oracle.call("dnb2_gen_natural", U(r), U(n), U(d), U(0), U(m), C, o_xb)
    o_xrb = np.empty_like(o_xb)
    oracle.call("dnb2_digital_shift", U(r), U(n), U(d), U(r), lsh, o_xb, shifts, o_xrb)
    o_x = np.empty((r, n, d))
    oracle.call("dnb2_integer_to_float", U(r), U(n), U(d), tm, o_xrb, o_x)
    assert np.array_equal(xrb.cpu().numpy().view(U), o_xrb.reshape(-1))
    assert np.array_equal(x.cpu().numpy().view(U), o_x.reshape(-1).view(U))
    # e2e: the drop-in API with numpy arrays, the three reference calls
    hxb, hxrb, hx = np.empty((r, n, d), U), np.empty((r, n, d), U), np.empty((r, n, d))
    e2e_steps = max(3, min(args.steps, 10))
    q.dnb2_gen_natural(U(r), U(n), U(d), U(0), U(m), C, hxb)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        q.dnb2_gen_natural(U(r), U(n), U(d), U(0), U(m), C, hxb)
        q.dnb2_digital_shift(U(r), U(n), U(d), U(r), lsh, hxb, shifts, hxrb)
        q.dnb2_integer_to_float(U(r), U(n), U(d), tm, hxrb, hx)
    t_e2e = (time.perf_counter() - t0) / e2e_steps
    assert np.array_equal(hx.view(U), o_x.view(U))
    # CPU: the oracle chain, one thread (r=1)
    t0 = time.perf_counter()
    oracle.call("dnb2_gen_natural", U(r), U(n), U(d), U(0), U(m), C, o_xb)
    oracle.call("dnb2_digital_shift", U(r), U(n), U(d), U(r), lsh, o_xb, shifts, o_xrb)
    oracle.call("dnb2_integer_to_float", U(r), U(n), U(d), tm, o_xrb, o_x)
    t_cpu = time.perf_counter() - t0
    pts = r * n
    return {"metric": METRIC, "value": pts / (ms_fused / 1e3), "unit": "points/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_fused, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64+f64", "data": "synthetic (np.random.SFC64(1))",
            "config": {"workload": "base-2 digital net, natural order + digital shift + float, r=1, d=16, m=16 "
                                   "(n=65536), tmax=63 (fused kernel, both outputs; steps replayed from one "
                                   "captured CUDA graph)", "r": r, "n": n, "d": d},
            "roofline": dict(roofline(16.0 * r * n * d, ms_fused), kernel="dnb2_gen_kernel (fused shift + float)",
                             note="16.8 MB per launch, below the HBM ramp: launch-latency bound even from a graph; "
                                  "the output fits in the 129 MB L2, so one launch's DRAM bytes do not measure it "
                                  "(traffic null)"),
            "eager": {"ms_per_step": ms_fused_eager, "points_per_s": pts / (ms_fused_eager / 1e3),
                      "plain_ms_per_step": ms_plain_eager,
                      "note": "one ctypes call per step from Python: the host's launch overhead is inside"},
            "plain": {"ms_per_step": ms_plain, "points_per_s": pts / (ms_plain / 1e3), "launches_per_step": 3,
                      "fused_speedup": ms_plain / ms_fused, "note": "the three reference calls, graph replay"},
            "e2e": {"value": pts / t_e2e, "unit": "points/s", "ms_per_step": 1e3 * t_e2e,
                    "h2d_bytes_per_step": C.nbytes + shifts.nbytes + 16 + 2 * r * n * d * 8,
                    "d2h_bytes_per_step": 3 * r * n * d * 8,
                    "path": "drop-in API, numpy arrays, dnb2_gen_natural -> dnb2_digital_shift -> "
                            "dnb2_integer_to_float"},
            "gpu_launches": graph_steps, "graph_steps": graph_steps,
            "cpu_baseline": {"value": pts / t_cpu, "unit": "points/s", "cores": 1, "kind": "port",
                             "sample": "the full workload, oracle chain, one thread (r=1)"}}


def cfg3_uniform_inputs(rng):
    import qmctoolscl_gb300 as q
    r, d_pre, alpha, m, tmax = 64, 64, 2, 20, 64
    C = triangular_net_matrices(rng, d_pre, m, 64)
    S = q.dnb2_get_linear_scramble_matrix(rng, r, d_pre, tmax, tmax, False)
    shifts = q.dnb2_get_digital_shifts(rng, r, d_pre // alpha, 64)
    return r, d_pre, alpha, m, C, S, shifts


def run_net_lms(args):
    """Base-2 net LMS + interlacing (alpha=2) + natural-order generation +
    digital shift: r=64, d_pre=64 -> d=32, m=20 (n=2^20), tmax=64; and an
    uneven batch of 256 requests (log2 n in [12,20], d in {8..64}) in one
    persistent launch / graph replay, against per-request plain calls."""
    import torch
    import qmctoolscl_gb300 as q
    from qmctoolscl_gb300 import _ffi, batch
    lib = _ffi.lib()
    rng = np.random.Generator(np.random.SFC64(3))
    r, d_pre, alpha, m, C, S, shifts = cfg3_uniform_inputs(rng)
    d, n = d_pre // alpha, 1 << m
    if args.small:  # profiling mode: 8 randomisations (2 GiB of output), no uneven batch
        r = 8
        S, shifts = np.ascontiguousarray(S[:r]), np.ascontiguousarray(shifts[:r])
    st = torch.cuda.Stream()
    h = st.cuda_stream
    Cd, Sd, sd = dev_tensor(C), dev_tensor(S), dev_tensor(shifts)
    lsh = dev_tensor(np.zeros(r, np.uint64))
    xrb = torch.empty(r * n * d, dtype=torch.int64, device="cuda")
    plan = batch.NetPlan([dict(r=r, n=n, d=d, alpha=alpha, d_pre=d_pre, mmax=m, tmax=64, tmax_new=64,
                               tmax_alpha=64, r_C=1, order="natural", C=Cd, S=Sd, lshifts=lsh, shifts=sd, xb=xrb)])
    with torch.cuda.stream(st):
        ms_plan = gpu_ms(lambda: plan.run(st), args.steps, args.warmup, st)
        ms_graph = gpu_ms(lambda: plan.graph_launch(st), args.steps, args.warmup, st)
        C_lms = torch.empty(r * d_pre * m, dtype=torch.int64, device="cuda")
        C_a = torch.empty(r * d * m, dtype=torch.int64, device="cuda")
        xb = torch.empty_like(xrb)
        xrb2 = torch.empty_like(xrb)

        def plain():
            _ffi.check(lib.qmc_dnb2_linear_matrix_scramble(r, d_pre, m, 1, 64, Sd.data_ptr(), Cd.data_ptr(),
                                                           C_lms.data_ptr(), h), "lms")
            _ffi.check(lib.qmc_dnb2_interlace(r, d, m, d_pre, 64, 64, alpha, C_lms.data_ptr(), C_a.data_ptr(), h),
                       "interlace")
            _ffi.check(lib.qmc_dnb2_gen_natural(r, n, d, 0, m, C_a.data_ptr(), xb.data_ptr(), h), "gen")
            _ffi.check(lib.qmc_dnb2_digital_shift(r, n, d, r, lsh.data_ptr(), xb.data_ptr(), sd.data_ptr(),
                                                  xrb2.data_ptr(), h), "shift")

        ms_plain = gpu_ms(plain, max(3, args.steps // 4), args.warmup, st)
    torch.cuda.synchronize()
    same = bool(torch.equal(xrb, xrb2))
    del xb, xrb2
    # spot check against the oracle chain on the first randomisation, 2^12 points
    import oracle
    U = np.uint64
    nn = 1 << 12
    Cl = np.empty((1, d_pre, m), U)
    oracle.call("dnb2_linear_matrix_scramble", U(1), U(d_pre), U(m), U(1), U(64), np.ascontiguousarray(S[:1]), C, Cl)
    Ca = np.empty((1, d, m), U)
    oracle.call("dnb2_interlace", U(1), U(d), U(m), U(d_pre), U(64), U(64), U(alpha), Cl, Ca)
    ob = np.empty((1, nn, d), U)
    oracle.call("dnb2_gen_natural", U(1), U(nn), U(d), U(0), U(m), Ca, ob)
    orb = np.empty_like(ob)
    oracle.call("dnb2_digital_shift", U(1), U(nn), U(d), U(1), np.zeros(1, U), ob, np.ascontiguousarray(shifts[:1]),
                orb)
    assert same and np.array_equal(xrb[:nn * d].cpu().numpy().view(U), orb.reshape(-1))
    del xrb, plan
    torch.cuda.empty_cache()
    if args.small:
        return {"small": True, "r": r, "graph_ms": ms_graph, "plain_ms": ms_plain,
                "gbs": 8.0 * r * n * d / (ms_graph / 1e3) / 1e9}

    # uneven batch of 256 single-randomisation requests
    urng = np.random.Generator(np.random.SFC64(33))
    C128 = triangular_net_matrices(urng, 128, m, 64)  # base matrices for d_pre = 2d up to 128
    reqs, plain_args = [], []
    total_pts = total_coords = 0
    for k in range(256):
        L = int(urng.integers(12, 21))
        dk = int(urng.choice(np.arange(8, 65, 8)))
        nk = 1 << L
        Sk = q.dnb2_get_linear_scramble_matrix(urng, 1, 2 * dk, 64, 64, False)
        shk = q.dnb2_get_digital_shifts(urng, 1, dk, 64)
        Ck = dev_tensor(np.ascontiguousarray(C128[:, :2 * dk, :]))
        out = torch.empty(nk * dk, dtype=torch.int64, device="cuda")
        req = dict(r=1, n=nk, d=dk, alpha=2, d_pre=2 * dk, mmax=m, tmax=64, tmax_new=64, tmax_alpha=64, r_C=1,
                   order="natural", C=Ck, S=dev_tensor(Sk), lshifts=dev_tensor(np.zeros(1, U)), shifts=dev_tensor(shk),
                   xb=out)
        reqs.append(req)
        plain_args.append(dict(req, C_lms=torch.empty(2 * dk * m, dtype=torch.int64, device="cuda"),
                               C_a=torch.empty(dk * m, dtype=torch.int64, device="cuda"),
                               tmp=torch.empty(nk * dk, dtype=torch.int64, device="cuda"),
                               out2=torch.empty(nk * dk, dtype=torch.int64, device="cuda")))
        total_pts += nk
        total_coords += nk * dk
    uplan = batch.NetPlan(reqs)
    with torch.cuda.stream(st):
        tuned = uplan.tune(stream=st, reps=2)
        ms_u_plan = gpu_ms(lambda: uplan.run(st), args.steps, args.warmup, st)
        ms_u_graph = gpu_ms(lambda: uplan.graph_launch(st), args.steps, args.warmup, st)

        def uneven_plain():
            for a in plain_args:
                dk, nk = a["d"], a["n"]
                lib.qmc_dnb2_linear_matrix_scramble(1, 2 * dk, m, 1, 64, a["S"].data_ptr(), a["C"].data_ptr(),
                                                    a["C_lms"].data_ptr(), h)
                lib.qmc_dnb2_interlace(1, dk, m, 2 * dk, 64, 64, 2, a["C_lms"].data_ptr(), a["C_a"].data_ptr(), h)
                lib.qmc_dnb2_gen_natural(1, nk, dk, 0, m, a["C_a"].data_ptr(), a["tmp"].data_ptr(), h)
                lib.qmc_dnb2_digital_shift(1, nk, dk, 1, a["lshifts"].data_ptr(), a["tmp"].data_ptr(),
                                           a["shifts"].data_ptr(), a["out2"].data_ptr(), h)

        ms_u_plain = gpu_ms(uneven_plain, max(3, args.steps // 4), 2, st)
    torch.cuda.synchronize()
    u_same = all(bool(torch.equal(a["xb"], a["out2"])) for a in plain_args)
    assert u_same, "uneven plan differs from the per-request calls"
    pts = r * n
    return {"metric": METRIC, "value": pts / (ms_graph / 1e3), "unit": "points/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_graph, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic (np.random.SFC64(3))",
            "config": {"workload": "base-2 net LMS + interlacing (alpha=2) + natural order + digital shift, r=64, "
                                   "d_pre=64 -> d=32, m=20 (n=2^20), tmax=64 (batched plan, graph replay)",
                       "r": r, "n": n, "d": d},
            "roofline": dict(roofline(8.0 * r * n * d, ms_graph), kernel="net_batch_kernel (graph replay)",
                             traffic=(lambda t: None if t is None else t * r / 8.0)(
                                 profiled_traffic("net_batch_kernel_lms_interlace_shift_r8_n2p20_d32.md")),
                             traffic_note="ncu DRAM bytes of the r=8 capture, scaled by r/8 (the coordinates)"),
            "batched_uniform": {"plan_ms": ms_plan, "graph_ms": ms_graph, "plain_ms": ms_plain,
                                "plain_launches": 4, "speedup_vs_plain": ms_plain / ms_graph},
            "uneven_batch": {"requests": 256, "points": total_pts, "coords": total_coords,
                             "plan_ms": ms_u_plan, "graph_ms": ms_u_graph, "plain_ms": ms_u_plain,
                             "plain_launches": 4 * 256, "plan_launches": 2,
                             "points_per_s": total_pts / (ms_u_graph / 1e3),
                             "achieved_gbs": 8.0 * total_coords / (ms_u_graph / 1e3) / 1e9,
                             "speedup_vs_plain": ms_u_plain / ms_u_graph, "tuning": list(tuned)},
            "gpu_launches": 2 * args.steps}


def run_fft(args):
    """Bit-reversed-order FFT (and FWHT on the real parts) of 4096 vectors of
    uneven lengths 2^10..2^20 (log2 length uniform, seeded), entries iid
    N(0,1): the FP64 radix-2 kernels (one call per length) against the
    tensor-core kernels (BF16 splits, FP32 accumulation), with the relative L2
    error of the tensor-core result against the FP64 one per length."""
    import torch
    from qmctoolscl_gb300 import _ffi
    lib = _ffi.lib()
    rng = np.random.Generator(np.random.SFC64(5))
    L = rng.integers(10, 21, 4096 if not args.small else 256)
    counts = {int(l): int((L == l).sum()) for l in sorted(set(L.tolist()))}
    groups = []
    for l, cnt in counts.items():
        n = 1 << l
        xr = rng.standard_normal((cnt, n))
        xi = rng.standard_normal((cnt, n))
        groups.append(dict(L=l, n=n, cnt=cnt, xr0=torch.from_numpy(xr).cuda(), xi0=torch.from_numpy(xi).cuda()))
    samples = sum(g["n"] * g["cnt"] for g in groups)
    st = torch.cuda.current_stream()
    h = st.cuda_stream
    for g in groups:
        g["xr"], g["xi"] = g["xr0"].clone(), g["xi0"].clone()
        g["twr"] = torch.empty(g["n"], dtype=torch.float64, device="cuda")
        g["twi"] = torch.empty_like(g["twr"])

    def fp64():
        for g in groups:
            _ffi.check(lib.qmc_fft_bro_1d_radix2(g["cnt"], 1, g["n"] // 2, g["twr"].data_ptr(), g["twi"].data_ptr(),
                                                 g["xr"].data_ptr(), g["xi"].data_ptr(), h), "fft")

    def tc():
        for g in groups:
            _ffi.check(lib.qmc_tc_fft_bro_1d(g["cnt"], 1, g["n"] // 2, g["xr"].data_ptr(), g["xi"].data_ptr(), h),
                       "tc_fft")

    def wht64():
        for g in groups:
            _ffi.check(lib.qmc_fwht_1d_radix2(g["cnt"], 1, g["n"] // 2, g["xr"].data_ptr(), h), "fwht")

    def wht_tc():
        for g in groups:
            _ffi.check(lib.qmc_tc_fwht_1d(g["cnt"], 1, g["n"] // 2, g["xr"].data_ptr(), h), "tc_fwht")

    steps, warm = max(3, min(args.steps, 10)), 3
    ms = {}
    for name, fn in (("fft_fp64", fp64), ("fft_tc", tc), ("fwht_fp64", wht64), ("fwht_tc", wht_tc)):
        ms[name] = gpu_ms(fn, steps, warm, st)  # in place: repeated transforms of whatever is there
    # accuracy: one transform of the original data by each path
    err = {}
    for g in groups:
        xr64, xi64 = g["xr0"].clone(), g["xi0"].clone()
        _ffi.check(lib.qmc_fft_bro_1d_radix2(g["cnt"], 1, g["n"] // 2, g["twr"].data_ptr(), g["twi"].data_ptr(),
                                             xr64.data_ptr(), xi64.data_ptr(), h), "fft")
        xrt, xit = g["xr0"].clone(), g["xi0"].clone()
        _ffi.check(lib.qmc_tc_fft_bro_1d(g["cnt"], 1, g["n"] // 2, xrt.data_ptr(), xit.data_ptr(), h), "tc_fft")
        wr64, wrt = g["xr0"].clone(), g["xr0"].clone()
        _ffi.check(lib.qmc_fwht_1d_radix2(g["cnt"], 1, g["n"] // 2, wr64.data_ptr(), h), "fwht")
        _ffi.check(lib.qmc_tc_fwht_1d(g["cnt"], 1, g["n"] // 2, wrt.data_ptr(), h), "tc_fwht")
        torch.cuda.synchronize()
        num = torch.sqrt(((xrt - xr64) ** 2 + (xit - xi64) ** 2).sum(dim=1))
        den = torch.sqrt((xr64 ** 2 + xi64 ** 2).sum(dim=1))
        wnum = torch.linalg.norm(wrt - wr64, dim=1)
        wden = torch.linalg.norm(wr64, dim=1)
        err[g["L"]] = {"fft_max": float((num / den).max()), "fwht_max": float((wnum / wden).max()), "vectors": g["cnt"]}
    # fused FFT -> pointwise product -> IFFT (the reference's fast kernel matrix-vector product)
    # against the two transforms alone (a lower bound for the three steps done separately)
    for g in groups:
        lam = rng.standard_normal((2, g["n"]))
        g["lr"], g["li"] = torch.from_numpy(lam[0]).cuda(), torch.from_numpy(lam[1]).cuda()

    def conv_fused():
        for g in groups:
            _ffi.check(lib.qmc_tc_fft_mul_ifft(g["cnt"], 1, g["n"] // 2, g["lr"].data_ptr(), g["li"].data_ptr(), 0, 0,
                                               1.0, g["xr"].data_ptr(), g["xi"].data_ptr(), h), "tc_fft_mul_ifft")

    def conv_transforms_only():
        for g in groups:
            _ffi.check(lib.qmc_tc_fft_bro_1d(g["cnt"], 1, g["n"] // 2, g["xr"].data_ptr(), g["xi"].data_ptr(), h),
                       "tc_fft")
            _ffi.check(lib.qmc_tc_ifft_bro_1d(g["cnt"], 1, g["n"] // 2, g["xr"].data_ptr(), g["xi"].data_ptr(), h),
                       "tc_ifft")

    ms["conv_fused"] = gpu_ms(conv_fused, steps, warm, st)
    ms["conv_transforms"] = gpu_ms(conv_transforms_only, steps, warm, st)
    conv_err = {}
    for g in groups:  # one vector per length against numpy
        m_ = g["L"]
        brv = np.zeros(g["n"], dtype=np.int64)
        idx_ = np.arange(g["n"])
        for b in range(m_):
            brv |= ((idx_ >> b) & 1) << (m_ - 1 - b)
        z = g["xr0"][0].cpu().numpy() + 1j * g["xi0"][0].cpu().numpy()
        lam_c = g["lr"].cpu().numpy() + 1j * g["li"].cpu().numpy()
        want = np.fft.ifft(np.fft.fft(z[brv], norm="ortho") * lam_c, norm="ortho")[brv]
        xr1, xi1 = g["xr0"][:1].clone(), g["xi0"][:1].clone()
        _ffi.check(lib.qmc_tc_fft_mul_ifft(1, 1, g["n"] // 2, g["lr"].data_ptr(), g["li"].data_ptr(), 0, 0, 1.0,
                                           xr1.data_ptr(), xi1.data_ptr(), h), "tc_fft_mul_ifft")
        got = xr1[0].cpu().numpy() + 1j * xi1[0].cpu().numpy()
        conv_err[g["L"]] = float(np.linalg.norm(got - want) / np.linalg.norm(want))
    # FP64 result against numpy on one vector of the largest length
    g = groups[-1]
    m = g["L"]
    br = np.zeros(g["n"], dtype=np.int64)
    idx = np.arange(g["n"])
    for b in range(m):
        br |= ((idx >> b) & 1) << (m - 1 - b)
    z = g["xr0"][0].cpu().numpy() + 1j * g["xi0"][0].cpu().numpy()
    want = np.fft.fft(z[br], norm="ortho")
    xr64, xi64 = g["xr0"][:1].clone(), g["xi0"][:1].clone()
    _ffi.check(lib.qmc_fft_bro_1d_radix2(1, 1, g["n"] // 2, g["twr"].data_ptr(), g["twi"].data_ptr(),
                                         xr64.data_ptr(), xi64.data_ptr(), h), "fft")
    got = xr64[0].cpu().numpy() + 1j * xi64[0].cpu().numpy()
    fp64_vs_numpy = float(np.linalg.norm(got - want) / np.linalg.norm(want))
    worst = max(e["fft_max"] for e in err.values())
    passes = lambda l: 1 if l <= 12 else 2  # noqa: E731
    # bytes per complex sample: one pass reads and writes FP64 (re, im), 32 B; two passes
    # read FP64 and write the FP32 intermediate (24 B), then read it and write FP64 (24 B)
    per_sample = lambda l: 32.0 if l <= 12 else 48.0  # noqa: E731
    alg_tc = sum(per_sample(g["L"]) * g["n"] * g["cnt"] for g in groups)
    return {"metric": METRIC, "value": samples / (ms["fft_tc"] / 1e3) / 1e9, "unit": "Gsamples/s", "n_gpus": 1,
            "steps": steps, "warmup": warm, "ms_per_step": ms["fft_tc"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16x3 products, fp32 accumulate, fp64 I/O",
            "data": "synthetic (np.random.SFC64(5)), N(0,1) complex",
            "config": {"workload": "bit-reversed FFT of %d vectors, log2 n uniform in [10,20]" % len(L),
                       "samples": samples, "lengths": counts},
            "roofline": dict(roofline(alg_tc, ms["fft_tc"]), kernel="tc_pass_kernel<FFT> (all passes of a step)",
                             traffic=alg_tc * TC_FFT_TRAFFIC_RATIO,
                             note="32 B per complex sample for one pass (FP64 read+write), 48 B for two (FP64 in, "
                                  "FP32 intermediate, FP64 out); traffic = algorithmic bytes x the DRAM/algorithmic "
                                  "ratio of the ncu capture in profiles/tc_pass_kernel_fft_n2p20.md"),
            "fp64": {"fft_ms": ms["fft_fp64"], "fwht_ms": ms["fwht_fp64"],
                     "fft_gsamples_per_s": samples / (ms["fft_fp64"] / 1e3) / 1e9,
                     "fp64_vs_numpy_rel_l2": fp64_vs_numpy},
            "tc": {"fft_ms": ms["fft_tc"], "fwht_ms": ms["fwht_tc"], "fft_speedup_vs_fp64": ms["fft_fp64"] / ms["fft_tc"],
                   "fwht_speedup_vs_fp64": ms["fwht_fp64"] / ms["fwht_tc"], "max_rel_l2_error": worst,
                   "error_by_log2n": err},
            "fft_mul_ifft": {"fused_ms": ms["conv_fused"], "fft_plus_ifft_ms": ms["conv_transforms"],
                             "speedup_vs_transforms_alone": ms["conv_transforms"] / ms["conv_fused"],
                             "max_rel_l2_error_vs_numpy": max(conv_err.values()), "error_by_log2n": conv_err,
                             "note": "qmc_tc_fft_mul_ifft: y <- IFFT(FFT(y) * lam), lam of n values per length, "
                                     "against qmc_tc_fft_bro_1d + qmc_tc_ifft_bro_1d with no pointwise step"},
            "gpu_launches": steps * sum(passes(g["L"]) for g in groups)}


def first_primes(k):
    out, c = [], 2
    while len(out) < k:
        if all(c % p for p in out if p * p <= c):
            out.append(c)
        c += 1
    return out


def halton_inputs(r, log2n, d, seed=4):
    """Per-dimension inputs of the randomised Halton workload: bases = the
    first d primes, tmax_j = ceil(64/log2 b), mmax_j = ceil(log2n/log2 b)
    (at least the base-b digits of n-1), identity generating matrices, and
    the reference's generators for S, perms and shifts called per dimension
    (d=1, r_b=1, tmax_new=tmax_j) in dimension order."""
    import math
    import qmctoolscl_gb300 as q
    rng = np.random.Generator(np.random.SFC64(seed))
    dims = []
    for b in first_primes(d):
        tmax = math.ceil(64 / math.log2(b))
        mmax, v = 0, (1 << log2n) - 1
        while v:
            v //= b
            mmax += 1
        mmax = max(mmax, math.ceil(log2n / math.log2(b)))
        bb = np.array([[b]], np.uint64)
        C = np.ascontiguousarray(q.gdn_get_halton_generating_matrix(1, 1, max(mmax, tmax))[:, :, :mmax, :tmax])
        dims.append(dict(b=b, tmax=tmax, mmax=mmax, C=C,
                         S=q.gdn_get_linear_scramble_matrix(rng, r, 1, tmax, tmax, 1, bb),
                         perms=q.gdn_get_digital_permutations(rng, r, 1, tmax, 1, bb),
                         shifts=q.gdn_get_digital_shifts(rng, r, 1, tmax, 1, bb)))
    return dims


def halton_inputs_gpu(r, log2n, d, seed=4):
    """halton_inputs with every random array drawn on the GPU (the same
    helpers with a device-resident generator: the same numpy streams, bit for
    bit); the generating matrices (identity, no randomness) are built on the
    host as the reference builds them."""
    import math
    import qmctoolscl_gb300 as q
    rng = np.random.Generator(np.random.SFC64(seed))
    dg = q.DeviceGenerator(rng)
    dims = []
    for b in first_primes(d):
        tmax = math.ceil(64 / math.log2(b))
        mmax, v = 0, (1 << log2n) - 1
        while v:
            v //= b
            mmax += 1
        mmax = max(mmax, math.ceil(log2n / math.log2(b)))
        bb = np.array([[b]], np.uint64)
        C = np.ascontiguousarray(q.gdn_get_halton_generating_matrix(1, 1, max(mmax, tmax))[:, :, :mmax, :tmax])
        dims.append(dict(b=b, tmax=tmax, mmax=mmax, C=C,
                         S=q.gdn_get_linear_scramble_matrix(dg, r, 1, tmax, tmax, 1, bb),
                         perms=q.gdn_get_digital_permutations(dg, r, 1, tmax, 1, bb),
                         shifts=q.gdn_get_digital_shifts(dg, r, 1, tmax, 1, bb)))
    dg.sync()
    return dims


def halton_oracle(dims, l, i0, cnt):
    """The reference chain on the oracle, one dimension per call, for
    randomisation l and points [i0, i0+cnt): an (cnt, d) float64 array."""
    import oracle
    U = np.uint64
    out = np.empty((cnt, len(dims)))
    for j, dm in enumerate(dims):
        b, tmax, mmax = dm["b"], dm["tmax"], dm["mmax"]
        bb = np.array([[b]], U)
        S = np.ascontiguousarray(dm["S"][l:l + 1])
        C_lms = np.empty((1, 1, mmax, tmax), U)
        oracle.call("gdn_linear_matrix_scramble", U(1), U(1), U(mmax), U(1), U(1), U(tmax), U(tmax), bb, S, dm["C"],
                    C_lms)
        xdig = np.empty((1, cnt, 1, tmax), U)
        oracle.call("gdn_gen_natural", U(1), U(cnt), U(1), U(1), U(mmax), U(tmax), U(i0), bb, C_lms, xdig)
        xp = np.empty_like(xdig)
        oracle.call("gdn_digital_permutation", U(1), U(cnt), U(1), U(1), U(1), U(tmax), U(tmax), U(b),
                    np.ascontiguousarray(dm["perms"][l:l + 1]), xdig, xp)
        xs = np.empty_like(xdig)
        oracle.call("gdn_digital_shift", U(1), U(cnt), U(1), U(1), U(1), U(tmax), U(tmax), bb,
                    np.ascontiguousarray(dm["shifts"][l:l + 1]), xp, xs)
        x = np.empty((1, cnt, 1))
        oracle.call("gdn_integer_to_float", U(1), U(cnt), U(1), U(1), U(tmax), bb, xs, x)
        out[:, j] = x[0, :, 0]
    return out


def run_halton(args):
    """Randomised Halton / generalized digital net: bases = first 100 primes,
    d=100, n=2^18, r=32, tmax_j = ceil(64/log2 b); LMS -> generation ->
    digit permutation -> digital shift -> float, bit-exact.  value: the fused
    plan (prepare + generate per step); plain: the reference's five calls per
    dimension through the C ABI with the digit tensors in HBM."""
    import torch
    from qmctoolscl_gb300 import _ffi, batch, halton
    lib = _ffi.lib()
    r, log2n, d = (8 if args.small else 32), 18, 100
    n = 1 << log2n
    pts_e2e = r * n
    dims = halton_inputs(r, log2n, d)
    st = torch.cuda.current_stream()
    h = st.cuda_stream
    ddims = [dict(b=dm["b"], tmax=dm["tmax"], mmax=dm["mmax"], C=dev_tensor(dm["C"]), S=dev_tensor(dm["S"]),
                  perms=dev_tensor(dm["perms"]), shifts=dev_tensor(dm["shifts"])) for dm in dims]
    x = torch.empty((r, n, d), dtype=torch.float64, device="cuda")
    plan = halton.HaltonPlan(r, n, 0, ddims, x)

    def fused():
        plan.prepare(st)
        plan.run(st)

    _ffi.check(lib.qmc_device_error_reset(h), "reset")
    plan.prepare(st)
    if args.small:  # profiling mode: the default split of the adds, generation only
        ms_gen = gpu_ms(lambda: plan.run(st), args.steps, args.warmup, st)
        return {"small": True, "r": r, "gen_ms": ms_gen, "gbs": 8.0 * r * n * d / (ms_gen / 1e3) / 1e9}
    # the share of digit adds on the FP64 unit (the rest in integer arithmetic): pick the fastest
    sweep = {}
    for share in (0.0, 0.25, 0.5, 0.75, 1.0):
        plan.set_fp64_share(share)
        sweep[share] = gpu_ms(lambda: plan.run(st), 3, 1, st)
    best_share = min(sweep, key=sweep.get)
    plan.set_fp64_share(best_share)
    clocks = ClockSampler(0)
    clocks.start()
    ms_gen = gpu_ms(lambda: plan.run(st), max(args.steps, 10), args.warmup, st)
    ms_fused = gpu_ms(fused, args.steps, args.warmup, st)
    clk = clocks.stop()
    _ffi.check(lib.qmc_device_error_check(h), "halton plan")
    # parity: two slices against the oracle chain
    for l, i0 in ((0, 0), (r - 1, n - 1500)):
        want = halton_oracle(dims, l, i0, 1500)
        got = x[l, i0:i0 + 1500].cpu().numpy()
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), "fused Halton differs from the oracle"

    # plain: per dimension, LMS -> gen -> perm -> shift -> float, then the column into x
    tmax_hi = max(dm["tmax"] for dm in dims)
    mm_hi = max(dm["mmax"] for dm in dims)
    xdig = torch.empty(r * n * tmax_hi, dtype=torch.int64, device="cuda")
    xp, xs = torch.empty_like(xdig), torch.empty_like(xdig)
    C_lms = torch.empty(r * mm_hi * tmax_hi, dtype=torch.int64, device="cuda")
    col = torch.empty((r, n), dtype=torch.float64, device="cuda")
    x2 = torch.empty_like(x)
    bases = [dev_tensor(np.array([[dm["b"]]], np.uint64)) for dm in dims]

    def plain():
        for j, (dm, dd) in enumerate(zip(dims, ddims)):
            b, tmax, mmax, bp = dm["b"], dm["tmax"], dm["mmax"], bases[j].data_ptr()
            _ffi.check(lib.qmc_gdn_linear_matrix_scramble(r, 1, mmax, 1, 1, tmax, tmax, bp, dd["S"].data_ptr(),
                                                          dd["C"].data_ptr(), C_lms.data_ptr(), h), "lms")
            _ffi.check(lib.qmc_gdn_gen_natural(r, n, 1, 1, mmax, tmax, 0, bp, C_lms.data_ptr(), xdig.data_ptr(), h),
                       "gen")
            _ffi.check(lib.qmc_gdn_digital_permutation(r, n, 1, r, 1, tmax, tmax, b, dd["perms"].data_ptr(),
                                                       xdig.data_ptr(), xp.data_ptr(), h), "perm")
            _ffi.check(lib.qmc_gdn_digital_shift(r, n, 1, r, 1, tmax, tmax, bp, dd["shifts"].data_ptr(),
                                                 xp.data_ptr(), xs.data_ptr(), h), "shift")
            _ffi.check(lib.qmc_gdn_integer_to_float(r, n, 1, 1, tmax, bp, xs.data_ptr(), col.data_ptr(), h), "float")
            x2[:, :, j].copy_(col)

    ms_plain = gpu_ms(plain, 2, 1, st)
    torch.cuda.synchronize()
    assert torch.equal(x.view(torch.int64), x2.view(torch.int64)), "fused Halton differs from the plain chain"
    digit_bytes = sum(r * n * dm["tmax"] * 8 for dm in dims)
    del xdig, xp, xs, x2, col
    torch.cuda.empty_cache()

    # e2e: numpy inputs copied in, the points written into pinned host memory, every step
    xh = batch.pinned_empty((r, n, d))
    halton.generalized_net_fused(r, n, 0, dims, xh)
    e2e_steps = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        A = halton.generalized_net_fused(r, n, 0, dims, xh, check=False)
    t_e2e = (time.perf_counter() - t0) / e2e_steps
    assert np.array_equal(xh.view(np.uint64), x.cpu().numpy().view(np.uint64))
    # e2e with the randomisation inputs drawn every step: by numpy on the host (the reference's
    # helpers, then copied in), or on the GPU from a device-resident generator (no input copies)
    dims_gpu = halton_inputs_gpu(r, log2n, d)
    for dh, dg_ in zip(dims, dims_gpu):  # the GPU draws are numpy's, bit for bit
        for key in ("S", "perms", "shifts"):
            assert np.array_equal(dg_[key].cpu().numpy().view(np.uint64), dh[key]), "device inputs differ"
    e2e_inputs = {}
    for mode, make in (("host_numpy_inputs", lambda: halton_inputs(r, log2n, d)),
                       ("gpu_inputs", lambda: halton_inputs_gpu(r, log2n, d))):
        make()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            A_in = halton.generalized_net_fused(r, n, 0, make(), xh, check=False)
        t_in = (time.perf_counter() - t0) / e2e_steps
        assert np.array_equal(xh.view(np.uint64), x.cpu().numpy().view(np.uint64))
        t_gen = time.perf_counter()
        make()
        torch.cuda.synchronize()
        t_gen = time.perf_counter() - t_gen
        e2e_inputs[mode] = {"value": pts_e2e / t_in, "unit": "points/s", "ms_per_step": 1e3 * t_in,
                            "input_generation_ms": 1e3 * t_gen, "h2d_bytes_per_step": A_in.h2d_bytes,
                            "d2h_bytes_per_step": A_in.d2h_bytes}

    # uneven batch: 64 requests of random r (1-4), n (2^10-2^16), n_start, d (4-100, first d primes);
    # one plan (graph replay: preparation + one generation launch) against one plan per request
    urng = np.random.Generator(np.random.SFC64(44))
    ureqs, uplans = [], []
    upoints = ucoords = 0
    for k in range(64):
        ur, un = int(urng.integers(1, 5)), 1 << int(urng.integers(10, 17))
        udim, ustart = int(urng.integers(4, 101)), int(urng.integers(0, 1 << 20))
        udims = halton_inputs(ur, 21, udim, seed=1000 + k)  # mmax for indices below 2^21
        dd = [dict(b=dm["b"], tmax=dm["tmax"], mmax=dm["mmax"], C=dev_tensor(dm["C"]), S=dev_tensor(dm["S"]),
                   perms=dev_tensor(dm["perms"]), shifts=dev_tensor(dm["shifts"])) for dm in udims]
        ux = torch.empty(ur * un * udim, dtype=torch.float64, device="cuda")
        ureqs.append(dict(r=ur, n=un, n_start=ustart, dims=dd, x=ux))
        upoints += ur * un
        ucoords += ur * un * udim
    ust = torch.cuda.Stream()
    ubatch = halton.HaltonBatch(ureqs)
    ms_u_graph = gpu_ms(lambda: ubatch.graph_launch(ust), args.steps, args.warmup, ust)
    with torch.cuda.stream(ust):
        singles = [halton.HaltonPlan(q_["r"], q_["n"], q_["n_start"], q_["dims"], q_["x"]) for q_ in ureqs]

        def per_request():
            for pl in singles:
                pl.prepare(ust)
                pl.run(ust)

        ms_u_single = gpu_ms(per_request, max(3, args.steps // 2), 2, ust)
    torch.cuda.synchronize()
    # parity: the last request's first 256 points of randomisation 0 against the oracle
    lq = ureqs[-1]
    lw = halton_oracle(halton_inputs(lq["r"], 21, len(lq["dims"]), seed=1000 + 63), 0, lq["n_start"], 256)
    lg = lq["x"].view(lq["r"], lq["n"], -1)[0, :256].cpu().numpy()
    assert np.array_equal(lg.view(np.uint64), lw.view(np.uint64)), "Halton batch differs from the oracle"
    for pl in singles:
        pl.close()
    ubatch.close()
    del ureqs, singles

    # CPU: the oracle chain on a sample of randomisation 0 (all of it on 16 cores, about 15
    # CPU-seconds), all host threads
    threads = host_threads()
    pieces = [(0, k * 4096, 4096) for k in range(min(4 * threads, n // 4096))]
    halton_oracle(dims, 0, 0, 64)
    t0 = time.perf_counter()
    with concurrent.futures.ThreadPoolExecutor(threads) as ex:
        list(ex.map(lambda a: halton_oracle(dims, *a), pieces))
    t_cpu = time.perf_counter() - t0
    cpu_pts = sum(p[2] for p in pieces)
    pts = r * n
    alg = 8.0 * r * n * d
    fp64_r8 = profiled_value("halton_gen_kernel_r32_n2p18_d100.md", "fp64_warp_inst_per_launch_r8")
    return {"metric": METRIC, "value": pts / (ms_fused / 1e3), "unit": "points/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_fused, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32 digits, f64 adds (split FP64 unit / integer by the tuned share)",
            "data": "synthetic (np.random.SFC64(4)): reference generators per dimension",
            "config": {"workload": "randomised Halton, bases = first 100 primes, d=100, n=2^18, r=32, "
                                   "tmax_j=ceil(64/log2 b), LMS + permutation + digital shift + float "
                                   "(fused plan: prepare + generate)", "r": r, "n": n, "d": d,
                       "l2": "6.7 GB output per step >> 129 MB L2, no flush needed"},
            "roofline": dict(roofline(alg, ms_gen), kernel="halton_gen_kernel",
                             traffic=profiled_traffic("halton_gen_kernel_r32_n2p18_d100.md"),
                             note="generation kernel alone; bound by the FP64 unit's digit adds (one per digit, "
                                  "the FP64 pipe about 70 % busy in the ncu capture) and integer issue, not HBM"),
            "fp64_roofline": dict(fp64_roofline(
                None if fp64_r8 is None else fp64_r8 * r / 8.0, ms_gen, clk.get("sm_mhz")) or {},
                note="generation kernel against the FP64 pipe's issue rate (2 lanes per SM per clock at the median "
                     "SM clock sampled while timing); executed FP64 instructions from the ncu capture of the r=8 case "
                     "in profiles/halton_gen_kernel_r32_n2p18_d100.md, scaled by r/8"),
            "generate_only_ms": ms_gen,
            "uneven_batch": {"requests": 64, "points": upoints, "coords": ucoords, "graph_ms": ms_u_graph,
                             "per_request_plans_ms": ms_u_single, "speedup": ms_u_single / ms_u_graph,
                             "launches": {"graph": 5, "per_request": 5 * 64},
                             "achieved_gbs": 8.0 * ucoords / (ms_u_graph / 1e3) / 1e9},
            "fp64_share": {"chosen": best_share, "generate_ms_by_share": {str(k): v for k, v in sweep.items()}},
            "plain": {"ms_per_step": ms_plain, "points_per_s": pts / (ms_plain / 1e3), "launches_per_step": 5 * d,
                      "digit_tensor_bytes": digit_bytes, "fused_speedup": ms_plain / ms_fused},
            "e2e": {"value": pts / t_e2e, "unit": "points/s", "ms_per_step": 1e3 * t_e2e,
                    "h2d_bytes_per_step": A.h2d_bytes, "d2h_bytes_per_step": A.d2h_bytes,
                    "direct_host_write": A.direct,
                    "path": "qmctoolscl_gb300.halton.generalized_net_fused, numpy inputs, pinned numpy output",
                    "other": {k: dict(v, path="randomisation inputs drawn every step (%s), then "
                                              "generalized_net_fused into the pinned output"
                                              % ("numpy on the host, copied in" if k.startswith("host")
                                                 else "on the GPU from a DeviceGenerator, no input copies"))
                              for k, v in e2e_inputs.items()}},
            "gpu_launches": 3 * args.steps, "clocks": clk,
            "cpu_baseline": {"value": cpu_pts / t_cpu, "unit": "points/s", "cores": threads, "kind": "port",
                             "sample": "randomisation 0, %d points in %d pieces of 4096, all 100 dimensions; the "
                                       "oracle chain per dimension, one piece per thread" % (cpu_pts, len(pieces)),
                             "seconds": t_cpu, "cpu_seconds": t_cpu * threads}}


def run_gdn_plain(args):
    """The plain drop-in generalized-net functions, one call each through the
    C ABI, at the per-dimension shape of the randomised Halton workload
    (r=32, n=2^18, d=1, tmax = ceil(64/log2 b), mmax = ceil(18/log2 b)) for
    bases 2, 3 and 541: gdn_linear_matrix_scramble -> gdn_gen_natural ->
    gdn_digital_permutation -> gdn_digital_shift -> gdn_integer_to_float,
    each timed alone with its HBM bytes (digits are u64 words)."""
    import math
    import torch
    import qmctoolscl_gb300 as q
    from qmctoolscl_gb300 import _ffi
    lib = _ffi.lib()
    r, n = (4 if args.small else 32), 1 << 18  # small: the gdn chain only, r = 4 (0.5 GB digit arrays)
    st = torch.cuda.current_stream()
    h = st.cuda_stream
    U = np.uint64
    peak, _src = measured_peak()
    res, total_ms = {}, 0.0
    for b in (2, 3, 541):
        tmax, mmax = math.ceil(64 / math.log2(b)), math.ceil(18 / math.log2(b))
        rng = np.random.Generator(np.random.SFC64(b))
        bb = np.array([[b]], U)
        C = np.ascontiguousarray(q.gdn_get_halton_generating_matrix(1, 1, max(mmax, tmax))[:, :, :mmax, :tmax])
        S = q.gdn_get_linear_scramble_matrix(rng, r, 1, tmax, tmax, 1, bb)
        P = q.gdn_get_digital_permutations(rng, r, 1, tmax, 1, bb)
        H = q.gdn_get_digital_shifts(rng, r, 1, tmax, 1, bb)
        Cd, Sd, Pd, Hd, bd = dev_tensor(C), dev_tensor(S), dev_tensor(P), dev_tensor(H), dev_tensor(bb)
        Cl = torch.empty(r * mmax * tmax, dtype=torch.int64, device="cuda")
        xd = torch.empty(r * n * tmax, dtype=torch.int64, device="cuda")
        xp, xs = torch.empty_like(xd), torch.empty_like(xd)
        x = torch.empty(r * n, dtype=torch.float64, device="cuda")
        calls = {
            "gdn_linear_matrix_scramble": lambda: lib.qmc_gdn_linear_matrix_scramble(
                r, 1, mmax, 1, 1, tmax, tmax, bd.data_ptr(), Sd.data_ptr(), Cd.data_ptr(), Cl.data_ptr(), h),
            "gdn_gen_natural": lambda: lib.qmc_gdn_gen_natural(r, n, 1, 1, mmax, tmax, 0, bd.data_ptr(), Cl.data_ptr(),
                                                               xd.data_ptr(), h),
            "gdn_digital_permutation": lambda: lib.qmc_gdn_digital_permutation(
                r, n, 1, r, 1, tmax, tmax, b, Pd.data_ptr(), xd.data_ptr(), xp.data_ptr(), h),
            "gdn_digital_shift": lambda: lib.qmc_gdn_digital_shift(r, n, 1, r, 1, tmax, tmax, bd.data_ptr(),
                                                                   Hd.data_ptr(), xp.data_ptr(), xs.data_ptr(), h),
            "gdn_integer_to_float": lambda: lib.qmc_gdn_integer_to_float(r, n, 1, 1, tmax, bd.data_ptr(),
                                                                         xs.data_ptr(), x.data_ptr(), h),
        }
        words = 8.0 * r * n * tmax
        alg = {"gdn_linear_matrix_scramble": 8.0 * r * mmax * tmax, "gdn_gen_natural": words,
               "gdn_digital_permutation": 2 * words, "gdn_digital_shift": 2 * words,
               "gdn_integer_to_float": words + 8.0 * r * n}
        per = {}
        for name, fn in calls.items():
            _ffi.check(fn(), name)
        for name, fn in calls.items():
            ms = gpu_ms(fn, args.steps, args.warmup, st)
            per[name] = {"ms": ms, "alg_bytes": alg[name], "gbs": alg[name] / (ms / 1e3) / 1e9,
                         "frac": alg[name] / (ms / 1e3) / 1e9 / peak}
            total_ms += ms
        # bit-exact: the last randomisation's first 1024 points against the oracle chain
        want = halton_oracle([dict(b=b, tmax=tmax, mmax=mmax, C=C, S=S, perms=P, shifts=H)], r - 1, 0, 1024)
        got = x.view(r, n)[r - 1, :1024].cpu().numpy()
        assert np.array_equal(got.view(U), want[:, 0].view(U)), "plain gdn chain differs from the oracle"
        res["b=%d (tmax=%d, mmax=%d)" % (b, tmax, mmax)] = per
    gdn_ms = total_ms
    if args.small:
        return {"small": True, "r": r, "kernels": res}
    # the other plain families at their benchmark shapes: base-2 nets (r=64, n=2^20, d=32, from the
    # LMS + interlacing inputs) and rank-1 lattices (r=16, n=2^20, d=64)
    rng3 = np.random.Generator(np.random.SFC64(3))
    r3, d_pre, alpha, m, C3, S3, sh3 = cfg3_uniform_inputs(rng3)
    d3, n3 = d_pre // alpha, 1 << m
    C3d, S3d, sh3d = dev_tensor(C3), dev_tensor(S3), dev_tensor(sh3)
    lsh, tms = dev_tensor(np.zeros(r3, U)), dev_tensor(np.full(r3, 64, U))
    C_lms = torch.empty(r3 * d_pre * m, dtype=torch.int64, device="cuda")
    C_a = torch.empty(r3 * d3 * m, dtype=torch.int64, device="cuda")
    xb = torch.empty(r3 * n3 * d3, dtype=torch.int64, device="cuda")
    xrb, xf = torch.empty_like(xb), torch.empty(r3 * n3 * d3, dtype=torch.float64, device="cuda")
    w3 = 8.0 * r3 * n3 * d3
    g2, s2 = workload_inputs()
    g2d, s2d = dev_tensor(g2), torch.from_numpy(s2).cuda()
    xl = torch.empty(R * (1 << LOG2N) * D, dtype=torch.float64, device="cuda")
    xlr = torch.empty_like(xl)
    w2, n2 = 8.0 * R * (1 << LOG2N) * D, 1 << LOG2N
    other = [
        ("dnb2_linear_matrix_scramble", lambda: lib.qmc_dnb2_linear_matrix_scramble(
            r3, d_pre, m, 1, 64, S3d.data_ptr(), C3d.data_ptr(), C_lms.data_ptr(), h), 8.0 * r3 * d_pre * m),
        ("dnb2_interlace", lambda: lib.qmc_dnb2_interlace(r3, d3, m, d_pre, 64, 64, alpha, C_lms.data_ptr(),
                                                          C_a.data_ptr(), h), 8.0 * r3 * d3 * m),
        ("dnb2_gen_natural", lambda: lib.qmc_dnb2_gen_natural(r3, n3, d3, 0, m, C_a.data_ptr(), xb.data_ptr(), h), w3),
        ("dnb2_gen_gray", lambda: lib.qmc_dnb2_gen_gray(r3, n3, d3, 0, m, C_a.data_ptr(), xb.data_ptr(), h), w3),
        ("dnb2_digital_shift", lambda: lib.qmc_dnb2_digital_shift(r3, n3, d3, r3, lsh.data_ptr(), xb.data_ptr(),
                                                                  sh3d.data_ptr(), xrb.data_ptr(), h), 2 * w3),
        ("dnb2_integer_to_float", lambda: lib.qmc_dnb2_integer_to_float(r3, n3, d3, tms.data_ptr(), xrb.data_ptr(),
                                                                        xf.data_ptr(), h), 2 * w3),
        ("lat_gen_gray", lambda: lib.qmc_lat_gen_gray(R, n2, D, 0, g2d.data_ptr(), xl.data_ptr(), h), w2),
        ("lat_gen_natural", lambda: lib.qmc_lat_gen_natural(R, n2, D, 0, g2d.data_ptr(), xl.data_ptr(), h), w2),
        ("lat_gen_linear", lambda: lib.qmc_lat_gen_linear(R, n2, D, g2d.data_ptr(), xl.data_ptr(), h), w2),
        ("lat_shift_mod_1", lambda: lib.qmc_lat_shift_mod_1(R, n2, D, R, xl.data_ptr(), s2d.data_ptr(),
                                                            xlr.data_ptr(), h), 2 * w2),
    ]
    fam = {}
    for name, fn, by in other:
        _ffi.check(fn(), name)
        ms = gpu_ms(fn, args.steps, args.warmup, st)
        fam[name] = {"ms": ms, "alg_bytes": by, "gbs": by / (ms / 1e3) / 1e9, "frac": by / (ms / 1e3) / 1e9 / peak}
    # parity of the last outputs: base-2 net and lattice slices against the oracle
    import oracle
    nn = 1 << 10
    ob = np.empty((1, nn, d3), U)
    Cl = np.empty((1, d_pre, m), U)
    oracle.call("dnb2_linear_matrix_scramble", U(1), U(d_pre), U(m), U(1), U(64), np.ascontiguousarray(S3[:1]), C3, Cl)
    Ca = np.empty((1, d3, m), U)
    oracle.call("dnb2_interlace", U(1), U(d3), U(m), U(d_pre), U(64), U(64), U(alpha), Cl, Ca)
    oracle.call("dnb2_gen_gray", U(1), U(nn), U(d3), U(0), U(m), Ca, ob)
    assert np.array_equal(xb[:nn * d3].cpu().numpy().view(U), ob.reshape(-1)), "dnb2 plain differs from the oracle"
    _ffi.check(lib.qmc_lat_gen_gray(R, n2, D, 0, g2d.data_ptr(), xl.data_ptr(), h), "lat_gen_gray")
    _ffi.check(lib.qmc_lat_shift_mod_1(R, n2, D, R, xl.data_ptr(), s2d.data_ptr(), xlr.data_ptr(), h), "shift")
    torch.cuda.synchronize()
    _t, xr_s = cpu_pipeline(g2, s2, nn, host_threads())
    assert np.array_equal(xlr.view(R, n2, D)[:, :nn].cpu().numpy().view(U), xr_s.view(U)), \
        "lattice plain differs from the oracle"
    res["base-2 nets r=64, n=2^20, d=32 and lattices r=16, n=2^20, d=64"] = fam
    pts = 3 * r * n
    return {"metric": METRIC, "value": pts / (gdn_ms / 1e3), "unit": "points/s (gdn chain, one dimension per base)",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": gdn_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64 digits, f64",
            "data": "synthetic (seeded np.random.SFC64): reference generators",
            "config": {"workload": "every plain drop-in kernel one call at a time: gdn chain per dimension "
                                   "(r=32, n=2^18, d=1, bases 2, 3, 541), base-2 nets (r=64, n=2^20, d=32), "
                                   "lattices (r=16, n=2^20, d=64)",
                       "l2": "arrays 0.5-17 GB >> 129 MB L2"},
            "roofline": dict(roofline(sum(v["alg_bytes"] for k_, p_ in res.items() if k_.startswith("b=")
                                          for v in p_.values()), gdn_ms),
                             kernel="the five plain gdn kernels, all bases (value); every kernel's own fraction "
                                    "under kernels"),
            "kernels": res, "gpu_launches": (15 + len(other)) * args.steps}


def run_qrng(args):
    """The generalized Halton sequence of halton_qrng (qmctoolscl/c_funcs/halton_qrng.c:3-162):
    n = 2^20 points of d = 100 dimensions (the first 100 primes), generalized multipliers,
    through the C ABI; checked against the oracle on a slice; the oracle over all host threads
    (one dimension per task) as the CPU baseline."""
    import torch
    import oracle
    from qmctoolscl_gb300 import _ffi
    lib = _ffi.lib()
    n, d = 1 << (16 if args.small else 20), 100
    rng = np.random.Generator(np.random.SFC64(6))
    randu_np = rng.random(d * 32)
    dvec_np = np.arange(d, dtype=np.int32)
    randu, dvec = torch.from_numpy(randu_np).cuda(), torch.from_numpy(dvec_np).cuda()
    res = torch.empty(d * n, dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream()
    h = st.cuda_stream

    def step():
        _ffi.check(lib.qmc_halton_qrng(n, d, 0, 1, res.data_ptr(), randu.data_ptr(), dvec.data_ptr(), h), "qrng")

    ms = gpu_ms(step, args.steps, args.warmup, st)
    _ffi.check(lib.qmc_device_error_check(h), "qrng")
    # parity on a slice: every dimension, points n0 .. n0+4095 of the same run
    nn, n0 = 4096, n // 2
    want = np.empty(d * nn)
    oracle.halton_qrng(nn, d, n0, 1, want, randu_np, dvec_np)
    got = res.view(d, n)[:, n0:n0 + nn].cpu().numpy().reshape(-1)
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), "halton_qrng differs from the oracle"
    # CPU: the oracle on all host threads, one dimension per task, a sample of the points
    threads = host_threads()
    ns = 1 << (15 if args.small else 19)  # about 10 CPU-seconds on 16 cores

    def one_dim(j):
        r_ = np.empty(ns)
        oracle.halton_qrng(ns, 1, 0, 1, r_, np.ascontiguousarray(randu_np[j * 32:(j + 1) * 32]), dvec_np[j:j + 1])

    t0 = time.perf_counter()
    with concurrent.futures.ThreadPoolExecutor(threads) as ex:
        list(ex.map(one_dim, range(d)))
    t_cpu = time.perf_counter() - t0
    pts = n
    return {"metric": METRIC, "value": pts / (ms / 1e3), "unit": "points/s (d=100)", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64 adds and divides (the reference's Horner steps)",
            "data": "synthetic (np.random.SFC64(6)) digit-shift uniforms",
            "config": {"workload": "halton_qrng, generalized, n=2^%d, d=100 (first 100 primes)" % (n.bit_length() - 1),
                       "n": n, "d": d, "l2": "%.0f MB output per step" % (8 * n * d / 1e6)},
            "roofline": dict(roofline(8.0 * n * d, ms), kernel="halton_qrng_kernel",
                             note="bound by instruction issue on two units, not by HBM: each digit step is the "
                                  "reference's rounded add and divide, a quarter of the warps on the FP64 pipe and "
                                  "the rest in integer arithmetic (ncu: FP64 pipe 64 %, ALU 63 %, issue 76 %; "
                                  "profiles/halton_qrng_kernel_n2p20_d100.md)"),
            "gpu_launches": args.steps,
            "cpu_baseline": {"value": ns / t_cpu, "unit": "points/s (d=100)", "cores": threads, "kind": "port",
                             "sample": "2^%d points of all 100 dimensions, one dimension per thread, by the oracle "
                                       "(C restatement of halton_qrng.c)" % (ns.bit_length() - 1), "seconds": t_cpu,
                             "cpu_seconds": t_cpu * threads}}


def run_nus(args):
    """Nested uniform (Owen) scrambling of base-2 net points, bit for bit the reference's
    dnb2_nested_uniform_scramble (qmctoolscl/rand_funcs.py:162-253) with numpy SFC64
    generators: r=64 replications x d=32 dimensions (2048 generators, fresh trees every step),
    n=2^20 natural-order net points (m=20, 64-bit keys: tmax = tmax_new = 64), through the C ABI
    with inputs and generator states resident on the GPU; e2e through the Python drop-in with
    numpy arrays and numpy Generators.  Checked against the oracle on the first 4096 points of
    five generators; the oracle over all host threads as the CPU baseline."""
    import torch
    import oracle
    import qmctoolscl_gb300 as q
    from qmctoolscl_gb300 import _ffi, nus
    lib = _ffi.lib()
    r, m, d = (16, 16, 32) if args.small else (64, 20, 32)
    n, G = 1 << m, r * d
    rng = np.random.Generator(np.random.SFC64(7))
    C = np.zeros((1, d, m), dtype=np.uint64)
    for j in range(d):
        M = np.triu(rng.integers(0, 2, (m, m)), 1) + np.eye(m, dtype=np.int64)
        for k in range(m):
            C[0, j, k] = sum(int(M[t, k]) << (63 - t) for t in range(m))
    dC = torch.from_numpy(C.reshape(-1).view(np.int64)).cuda()
    xb = torch.empty(n * d, dtype=torch.int64, device="cuda")
    q.dnb2_gen_natural(1, n, d, 0, m, dC, xb)
    xrb = torch.empty(G * n, dtype=torch.int64, device="cuda")  # r x n x d
    seeds = np.random.SeedSequence(7).spawn(G)
    states0 = np.stack([nus.sfc64_state_words(np.random.Generator(np.random.SFC64(sd))) for sd in seeds])
    st0 = torch.from_numpy(states0.reshape(-1).view(np.int64)).cuda()
    stw = torch.empty_like(st0)
    free, _tot = torch.cuda.mem_get_info()
    per = nus.workspace_bytes(n, 0, 1)
    count = max(1, min(G, min(free // 2, 160 << 30) // per))  # every generator in one chunk where it fits
    wbytes = nus.workspace_bytes(n, 0, count)
    work = torch.empty(wbytes, dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream()
    h = st.cuda_stream

    def step():
        stw.copy_(st0)
        _ffi.check(lib.qmc_dnb2_nested_uniform_scramble(r, n, d, 1, 64, 64, stw.data_ptr(), 0, None, None,
                                                        xb.data_ptr(), xrb.data_ptr(), None, None, work.data_ptr(),
                                                        wbytes, h), "nus")

    ms = gpu_ms(step, args.steps, args.warmup, st)
    _ffi.check(lib.qmc_device_error_check(h), "nus")
    # parity: the first 4096 points of five generators (a point's result depends only on
    # the points before it), against the oracle from the same initial states
    xb_np = xb.cpu().numpy().view(np.uint64).reshape(1, n, d)
    out = xrb.view(r, n, d)
    nn = 4096
    for (l, j) in ((0, 0), (0, 1), (1, 7), (r - 1, d - 1), (r // 2, d // 2)):
        w = states0[l * d + j].copy()
        want = np.zeros((1, nn, 1), dtype=np.uint64)
        f = oracle.NusForest(1)
        f.scramble(1, nn, 1, 1, 64, 64, w, np.ascontiguousarray(xb_np[:, :nn, j:j + 1]), want)
        f.close()
        got = out[l, :nn, j].cpu().numpy().view(np.uint64)
        assert np.array_equal(got, want.reshape(-1)), "nested uniform scramble differs from the oracle"
    N = n + 1
    passes = 8
    top = min(passes, ((N - 1).bit_length() + 4 + 7) // 8)
    chunks = -(-G // count)
    launches = chunks * (1 + 3 * top + 1 + 2 + 1 + 3)
    del work
    torch.cuda.empty_cache()
    # e2e: the drop-in with numpy arrays (xb 1 x n x d in, xrb r x n x d out) and fresh
    # numpy Generators / root nodes per call
    xrb_np = np.empty((r, n, d), dtype=np.uint64)
    e2e_steps = max(1, min(args.steps, 3))
    times = []
    for it in range(e2e_steps + 1):
        gens = np.array([np.random.Generator(np.random.SFC64(sd)) for sd in seeds], dtype=object).reshape(r, d)
        roots = np.array([q.NUSNode_dnb2() for _ in range(G)]).reshape(r, d)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        q.dnb2_nested_uniform_scramble(r, n, d, 1, 64, 64, gens, roots, xb_np, xrb_np)
        times.append(time.perf_counter() - t0)
        del gens, roots
    t_e2e = float(np.mean(times[1:]))
    assert np.array_equal(xrb_np[:2, :nn].reshape(-1), out[:2, :nn].cpu().numpy().view(np.uint64).reshape(-1))
    del xrb_np
    # CPU: the oracle over all host threads, whole generators (all n points) of replications 0-1
    threads = host_threads()
    gs = min(G, 4 * d) if not args.small else min(G, 16 * d)  # about 10 CPU-seconds

    def one_gen(k):
        l, j = divmod(k, d)
        w = states0[k].copy()
        o = np.zeros((1, n, 1), dtype=np.uint64)
        f = oracle.NusForest(1)
        f.scramble(1, n, 1, 1, 64, 64, w, np.ascontiguousarray(xb_np[:, :, j:j + 1]), o)
        f.close()

    t0 = time.perf_counter()
    with concurrent.futures.ThreadPoolExecutor(threads) as ex:
        list(ex.map(one_gen, range(gs)))
    t_cpu = time.perf_counter() - t0
    pts = G * n
    return {"metric": METRIC, "value": pts / (ms / 1e3), "unit": "points/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64 (keys, GF(2) bits) and the SFC64 stream",
            "data": "synthetic: natural-order net points of random upper-unit-triangular matrices "
                    "(np.random.SFC64(7)); generators SFC64(SeedSequence(7).spawn(r*d))",
            "config": {"workload": "dnb2_nested_uniform_scramble, r=%d, n=2^%d, d=%d, tmax=tmax_new=64, "
                                   "fresh trees" % (r, m, d), "r": r, "n": n, "d": d,
                       "generators_per_chunk": int(count), "chunks": int(chunks),
                       "l2": "%.1f GB output per step" % (8.0 * pts / 1e9)},
            "roofline": dict(roofline(8.0 * (n * d + pts), ms), kernel="the whole pipeline",
                             note="not an HBM-bound path: per generator one serial pass of the SFC64 stream "
                                  "(numpy's draw order) plus a radix sort, a radix tree and a tree walk per point; "
                                  "achieved counts only the point I/O (xb in, xrb out)"),
            "e2e": {"value": pts / t_e2e, "unit": "points/s", "seconds_per_call": t_e2e,
                    "h2d_bytes_per_step": int(8 * n * d + 48 * G), "d2h_bytes_per_step": int(8 * pts + 56 * G),
                    "path": "qmctoolscl_gb300.dnb2_nested_uniform_scramble with numpy arrays and Generators"},
            "gpu_launches": args.steps * launches,
            "cpu_baseline": {"value": gs * n / t_cpu, "unit": "points/s", "cores": threads, "kind": "port",
                             "sample": "%d whole generators (2^%d points each), one per thread, by the oracle "
                                       "(C restatement of the reference's tree walk)" % (gs, m),
                             "seconds": t_cpu}}


def run_gdn_nus(args):
    """Nested uniform (Owen) scrambling of generalized nets, bit for bit the reference's
    gdn_nested_uniform_scramble (qmctoolscl/rand_funcs.py:262-356) with numpy SFC64 generators:
    Halton points in the first 8 primes (natural order, identity matrices), r=16, n=2^16,
    tmax=16, tmax_new=20, fresh trees, through the drop-in with device arrays; e2e with numpy
    arrays.  Checked against the oracle on the first 512 points of three generators; the
    oracle over all host threads as the CPU baseline."""
    import torch
    import oracle
    import qmctoolscl_gb300 as q
    from qmctoolscl_gb300 import nus
    r, m = (4, 12) if args.small else (16, 16)
    n, d, tmax, tmax_new = 1 << m, 8, 16, 20
    G = r * d
    bases_np = np.array([[2, 3, 5, 7, 11, 13, 17, 19]], dtype=np.uint64)
    C = torch.from_numpy(np.tile(np.eye(tmax, dtype=np.uint64)[None, None], (1, d, 1, 1)).reshape(-1).view(np.int64)).cuda()
    dbases = torch.from_numpy(bases_np.reshape(-1).view(np.int64)).cuda()
    xdig = torch.empty(n * d * tmax, dtype=torch.int64, device="cuda")
    q.gdn_gen_natural(1, n, d, 1, tmax, tmax, 0, dbases, C, xdig)
    xr = torch.empty(G * n * tmax_new, dtype=torch.int64, device="cuda")
    seeds = np.random.SeedSequence(8).spawn(G)
    st = torch.cuda.current_stream()

    def call(xin, xout):
        gens = np.array([np.random.Generator(np.random.SFC64(sd)) for sd in seeds], dtype=object).reshape(r, d)
        roots = np.array([q.NUSNode_gdn() for _ in range(G)]).reshape(r, d)
        q.gdn_nested_uniform_scramble(r, n, d, 1, 1, tmax, tmax_new, gens, roots, bases_np, xin, xout)

    ms = gpu_ms(lambda: call(xdig, xr), args.steps, args.warmup, st)
    xd_np = xdig.cpu().numpy().view(np.uint64).reshape(1, n, d, tmax)
    out = xr.view(r, n, d, tmax_new)
    nn = 512
    for (l, j) in ((0, 0), (1, 3), (r - 1, d - 1)):
        w = nus.sfc64_state_words(np.random.Generator(np.random.SFC64(seeds[l * d + j])))
        want = np.zeros((1, nn, 1, tmax_new), dtype=np.uint64)
        f = oracle.GdnNusForest(1)
        assert f.scramble(1, nn, 1, 1, 1, tmax, tmax_new, w, bases_np[:, j:j + 1].copy(),
                          np.ascontiguousarray(xd_np[:, :nn, j:j + 1]), want) == 0
        f.close()
        got = out[l, :nn, j].cpu().numpy().view(np.uint64)
        assert np.array_equal(got, want.reshape(nn, tmax_new)), "base-b nested uniform scramble differs from the oracle"
    # e2e: numpy arrays in and out
    xr_np = np.empty((r, n, d, tmax_new), dtype=np.uint64)
    call(xd_np, xr_np)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    call(xd_np, xr_np)
    t_e2e = time.perf_counter() - t0
    # CPU: the oracle, whole generators of replication 0 (all 8 bases), one per thread
    threads = host_threads()

    def one_gen(k):
        j = k % d
        w = nus.sfc64_state_words(np.random.Generator(np.random.SFC64(seeds[k])))
        o = np.zeros((1, n, 1, tmax_new), dtype=np.uint64)
        f = oracle.GdnNusForest(1)
        f.scramble(1, n, 1, 1, 1, tmax, tmax_new, w, bases_np[:, j:j + 1].copy(),
                   np.ascontiguousarray(xd_np[:, :, j:j + 1]), o)
        f.close()

    # the whole workload, every generator, largest bases first so the threads finish together
    gs = G
    order = sorted(range(G), key=lambda k: -int(bases_np[0, k % d]))
    t0 = time.perf_counter()
    with concurrent.futures.ThreadPoolExecutor(threads) as ex:
        list(ex.map(one_gen, order))
    t_cpu = time.perf_counter() - t0
    pts = G * n
    return {"metric": METRIC, "value": pts / (ms / 1e3), "unit": "points/s (d=8, 20 digits each)", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64 digits, 128-bit keys, the SFC64 stream",
            "data": "synthetic: natural-order Halton digits in bases 2..19; generators "
                    "SFC64(SeedSequence(8).spawn(r*d))",
            "config": {"workload": "gdn_nested_uniform_scramble, r=%d, n=2^%d, d=8 (first 8 primes), tmax=16, "
                                   "tmax_new=20, fresh trees" % (r, m), "r": r, "n": n, "d": d},
            "roofline": dict(roofline(8.0 * (n * d * tmax + pts * tmax_new), ms), kernel="the whole pipeline",
                             note="bound by the serial SFC64 stream of the base-19 generators (numpy's masked "
                                  "draws for b-1 swap indices per level, for every level below each point's "
                                  "branch): one producer lane per generator at about 40 cycles per 64-bit step, "
                                  "decoding warps beside it; the swaps themselves run one thread per "
                                  "permutation; achieved counts only the digit I/O"),
            "e2e": {"value": pts / t_e2e, "unit": "points/s", "seconds_per_call": t_e2e,
                    "h2d_bytes_per_step": int(8 * n * d * tmax + 48 * G),
                    "d2h_bytes_per_step": int(8 * pts * tmax_new + 48 * G),
                    "path": "qmctoolscl_gb300.gdn_nested_uniform_scramble with numpy arrays and Generators"},
            "gpu_launches": args.steps * (10 + 3 * min(8, (n.bit_length() + 4 + 7) // 8)),  # one chunk
            "cpu_baseline": {"value": gs * n / t_cpu, "unit": "points/s", "cores": threads, "kind": "port",
                             "sample": "the whole workload: all %d generators (2^%d points each, bases 2..19) over the "
                                       "host threads, largest bases first, by the oracle (C restatement of the "
                                       "reference's tree walk)" % (gs, m),
                             "seconds": t_cpu}}


# the default run's "configs" object: every other configuration of the benchmark, each its own
# workload function (the same as --workload <name>), with at most this many timed steps
CONFIGS = [("cfg1_net_plain", "net_plain", 10), ("cfg3_net_lms", "net_lms", 10), ("cfg4_halton", "halton", 10),
           ("cfg5_fft", "fft", 10), ("plain_drop_in", "plain", 10), ("halton_qrng", "qrng", 10),
           ("nus_base2", "nus", 3), ("nus_base_b", "gdn_nus", 3)]
_REPEATED = ("metric", "n_gpus", "higher_is_better", "scaling", "vs_baseline")


def run_configs(args):
    """Each configuration in CONFIGS on this GPU, one after another, freeing its
    device and pinned memory before the next; an entry holds its workload's
    line (without the keys the headline line already states) and its wall
    time, or the error that stopped it."""
    import copy
    import gc
    import torch
    out = {}
    for key, name, max_steps in CONFIGS:
        a = copy.copy(args)
        a.steps = max(1, min(args.steps, max_steps))
        t0 = time.perf_counter()
        try:
            entry = {k: v for k, v in WORKLOADS[name](a).items() if k not in _REPEATED}
        except Exception as e:  # a failing configuration is reported in its entry, the others still run
            entry = {"error": "%s: %s" % (type(e).__name__, e)}
        entry["workload_flag"] = "--workload " + name
        entry["wall_s"] = time.perf_counter() - t0
        out[key] = entry
        gc.collect()
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
    return out


WORKLOADS = {"net_plain": run_net_plain, "net_lms": run_net_lms, "fft": run_fft, "halton": run_halton,
             "plain": run_gdn_plain, "gdn_plain": run_gdn_plain, "qrng": run_qrng, "nus": run_nus,
             "gdn_nus": run_gdn_nus}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="lattice", choices=["lattice"] + sorted(WORKLOADS),
                    help="lattice (default): the headline configuration; the others print their own line")
    ap.add_argument("--no-configs", action="store_true",
                    help="default workload only: leave out the other configurations' entries")
    ap.add_argument("--small", action="store_true",
                    help="profiling mode: the fused kernel only, on n=2^%d (512 MiB output)" % PROFILE_LOG2N)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload != "lattice":
        import torch
        torch.cuda.set_device(0)
        print(json.dumps(WORKLOADS[args.workload](args)), flush=True)
    else:
        line = run_ours(args)
        if line is not None:  # rank 0
            if line.get("n_gpus") == 1 and not args.small and not args.no_configs:
                line["configs"] = run_configs(args)
            print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
