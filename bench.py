"""Benchmark of the GB300 Lloyd k-means engine.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--form auto|plain|mixed-bf16|mixed-fp16]
                    [--workload c3|c2|c1|c4|c5]

A step is one Lloyd iteration (fused assignment + accumulation, reduction,
relocation gate, division, shift test) over the whole synthetic data set.
Default workload (c3): n = 10,000,000 samples x d = 64 float32 features,
k = 1024 clusters, Gaussian blobs (1024 centres uniform in [-5, 5]^64,
per-blob sigma uniform in [0.5, 2.0], seed 2), seeded random-row init.

value    iterations/s with X already resident in HBM, timed with CUDA events
         on the fit's stream over exactly K steps (max over ranks).
e2e      the same metric through the drop-in Python surface
         (kmeans_lloyd_driver) with host buffers: pinned host -> device copies
         of X, weights and initial centroids, K iterations, and the device ->
         host read of labels, centroids and inertia, all inside the timed region.
roofline for the dominant kernel (assignment + accumulation), from its CUDA
         event times inside the timed region.
cpu_baseline  the CPU oracle (C++/OpenMP restatement of the reference path) on
         a bounded sample of the same workload, scaled to iterations/s.
parity   outside the timed regions: one step of the headline form from the
         initial centroids and the final pass, against the oracle on all
         samples (label agreement, centroid and inertia relative errors).
serve    p50/p99 request latency and throughput of the serving loop (continuous
         batching, HBM admission) on the first requests of the c5 stream, for
         the plain and mixed-fp16 forms (--serve-sample requests; 0 skips it).

--workload c4   256 independent fits (n log-uniform in [2e3, 2e6], d in
                {8, 16, 32, 64, 128}, k log-uniform in [4, 512], 50 iterations)
                through the batched engine: instance-iterations/s, beside a
                loop of single plain fits of the same instances.
--workload c5   the full serving stream: 10,000 requests, Poisson arrivals at
                500/s, 80 % fits (n in [1e4, 5e6], d in {16, 32, 64}, k in
                [8, 1024], tol 1e-4, max_iter 300), 20 % predictions (n in
                [1e3, 1e6]) against earlier fits, 150 GB admission budget;
                p50/p99 latency and throughput for the plain and mixed forms.

--impl reference times the reference's algorithm on the host cores.  The
reference itself (SYCL/DPC++ + dpctl) cannot be built here, so its CPU
restatement (oracle/kmref.cpp) stands in for it.

Multi-GPU (torchrun): the Lloyd loop is not sharded in this build; each rank
runs an independent replica and value counts the iterations of all replicas
("scaling": "weak").
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

METRIC = "Lloyd iter/s + %roofline (10M×64, k=1024), mixed vs FP32; serve p50/p99"

WORKLOADS = {
    # name: n, d, n_centers, k, box, std (scalar or (lo, hi) per blob), seed, far_first
    "c3": dict(n=10_000_000, d=64, centers=1024, k=1024, box=(-5.0, 5.0), std=(0.5, 2.0), seed=2,
               far_first=False, desc="10M x 64 float32 Gaussian blobs, k=1024, random-row init"),
    "c2": dict(n=5_000_000, d=14, centers=127, k=127, box=(-10.0, 10.0), std=1.5, seed=1,
               far_first=True, desc="5M x 14 float32 Gaussian blobs, k=127, centroid 0 = 1e3*ones"),
    "c1": dict(n=50_000, d=14, centers=16, k=16, box=(-10.0, 10.0), std=1.0, seed=0,
               far_first=False, desc="50k x 14 float32 Gaussian blobs, k=16"),
    "c2f64": dict(n=5_000_000, d=14, centers=127, k=127, box=(-10.0, 10.0), std=1.5, seed=1,
                  far_first=True, dtype="f64",
                  desc="5M x 14 float64 Gaussian blobs, k=127, centroid 0 = 1e3*ones"),
}

# Nominal dense FP64 rate of one GB300 (no measured FP64 peak is available).
FP64_NOMINAL_TFLOPS = 1.25

FORMS = {"plain": 0, "mixed-bf16": 1, "mixed-fp16": 2}

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of
# the dominant kernel per sample, from one ncu capture at n=1,000,000 of the
# workload's shape (profiles/mixed_assign_c3_n1M.txt and
# profiles/tile_kernel_plain_c3_n1M.txt); the kernels stream every sample
# once, so a launch's traffic scales with n.
TRAFFIC_PER_SAMPLE = {("c3", "mixed-fp16"): 404.9, ("c3", "plain"): 267.6}


# ---------------------------------------------------------------------------
# synthetic data (shared with the tests)
# ---------------------------------------------------------------------------
def make_blobs(n, d, n_centers, center_box, std, seed, dtype=np.float32):
    """Isotropic Gaussian blobs with equal blob sizes, rows shuffled.

    Returns (X_t (d, n) C-contiguous, centers (n_centers, d), blob_of_row (n,)).
    `std` is a scalar, a (lo, hi) tuple (per-blob sigma uniform in [lo, hi]) or
    an array of per-blob standard deviations.
    """
    rng = np.random.default_rng(seed)
    centers = rng.uniform(center_box[0], center_box[1], size=(n_centers, d))
    if isinstance(std, tuple):
        stds = rng.uniform(std[0], std[1], size=n_centers)
    else:
        stds = np.broadcast_to(np.asarray(std, dtype=np.float64), (n_centers,))
    blob = rng.permutation(n) % n_centers
    X_t = np.empty((d, n), dtype=dtype)
    chunk = 1 << 20
    for i0 in range(0, n, chunk):
        b = blob[i0:i0 + chunk]
        noise = rng.standard_normal((b.size, d), dtype=np.float32)
        X_t[:, i0:i0 + chunk] = (centers[b] + noise * stds[b, None]).T.astype(dtype)
    return X_t, centers, blob


def random_row_init(X_t, k, seed, far_first=False):
    """Initial centroids (d, k): X rows at seeded indices without replacement.

    far_first replaces centroid 0 by 1e3 * ones (forces an empty cluster)."""
    rng = np.random.default_rng(seed + 7919)
    idx = rng.choice(X_t.shape[1], size=k, replace=False)
    C = np.ascontiguousarray(X_t[:, idx])
    if far_first:
        C[:, 0] = 1e3
    return C


def workload(name, n=None):
    """The named workload, optionally with fewer samples (profiling captures)."""
    w = dict(WORKLOADS[name])
    if n:
        w["n"] = int(n)
        w["desc"] = w["desc"] + " (n reduced to %d)" % w["n"]
    return w


def workload_data(name, n=None):
    w = workload(name, n)
    dt = np.float64 if w.get("dtype") == "f64" else np.float32
    X_t, _, _ = make_blobs(w["n"], w["d"], w["centers"], w["box"], w["std"], w["seed"], dtype=dt)
    C0 = random_row_init(X_t, w["k"], w["seed"], far_first=w["far_first"])
    return X_t, C0


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, gpu_id=None, interval_ms=50):
        self.cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                    f"-lms={interval_ms}"]
        if gpu_id:
            self.cmd.append(f"--id={gpu_id}")
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(self.cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], [], set()
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(self.NAMES, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


# ---------------------------------------------------------------------------
# CPU oracle timing (cpu_baseline and the reference arm)
# ---------------------------------------------------------------------------
def cpu_step_time(X_t, C0, n_s):
    from oracle import kmref

    Xs = np.ascontiguousarray(X_t[:, :n_s])
    w = np.ones(n_s, X_t.dtype)
    t0 = time.perf_counter()
    kmref.fused_lloyd_single_step(Xs, w, C0)
    return time.perf_counter() - t0


def calibrate_cpu_sample(X_t, C0, target_s):
    n = X_t.shape[1]
    n_s = min(n, 20_000)
    t = cpu_step_time(X_t, C0, n_s)
    n_s = int(min(n, max(1000, n_s * target_s / max(t, 1e-6))))
    return n_s


def cpu_baseline(X_t, C0, target_s=10.0):
    from oracle import kmref

    n = X_t.shape[1]
    n_s = calibrate_cpu_sample(X_t, C0, target_s)
    t = cpu_step_time(X_t, C0, n_s)
    return {"value": (n_s / n) / t, "unit": "iter/s", "cores": kmref.num_threads(), "kind": "port",
            "sample": f"one Lloyd step (assignment + accumulation) over the first {n_s} of {n} "
                      f"samples, scaled by n/{n_s}; oracle/kmref.cpp, OpenMP"}


# ---------------------------------------------------------------------------
# distributed helpers (replicas)
# ---------------------------------------------------------------------------
def dist_setup(n_gpus):
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl", device_id=torch.device(f"cuda:{local}"))
    return world, rank, local


def gpu_local_cpus(local):
    """Host CPUs next to GPU `local` (its PCI device's local_cpulist), or None."""
    import torch

    try:
        p = torch.cuda.get_device_properties(local)
        bus = "%04x:%02x:%02x.0" % (p.pci_domain_id, p.pci_bus_id, p.pci_device_id)
        with open("/sys/bus/pci/devices/%s/local_cpulist" % bus) as f:
            text = f.read().strip()
        cpus = set()
        for part in text.split(","):
            if "-" in part:
                a, b = part.split("-")
                cpus.update(range(int(a), int(b) + 1))
            elif part:
                cpus.add(int(part))
        cpus &= os.sched_getaffinity(0)
        return cpus or None
    except Exception:
        return None


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def all_max(world, v):
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist

    # NCCL reduces device tensors; gloo (CPU process groups) host tensors
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
def run_reference(args, world, rank):
    """CPU reference arm: the reference algorithm on the host cores."""
    from oracle import kmref

    if rank != 0:
        return
    w = workload(args.workload, args.n)
    X_t, C0 = workload_data(args.workload, args.n)
    n = X_t.shape[1]
    n_s = calibrate_cpu_sample(X_t, C0, target_s=1.5)
    for _ in range(args.warmup):
        cpu_step_time(X_t, C0, n_s)
    times = [cpu_step_time(X_t, C0, n_s) for _ in range(args.steps)]
    t_step = sum(times) / len(times)
    value = (n_s / n) / t_step
    sample = (f"each step: one Lloyd step (assignment + accumulation) over the first {n_s} of {n} "
              f"samples, scaled by n/{n_s}; the reference (SYCL/DPC++) cannot be built here, so its "
              f"C++ restatement oracle/kmref.cpp runs with OpenMP on all host threads")
    line = {
        "metric": METRIC, "value": value, "unit": "iter/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / value,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if X_t.dtype == np.float64 else "f32",
        "data": "synthetic", "impl": "reference",
        "config": {"workload": args.workload, "desc": w["desc"], "n": w["n"], "d": w["d"], "k": w["k"]},
        "cpu_baseline": {"value": value, "unit": "iter/s", "cores": kmref.num_threads(),
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _time_form(L, capi, Xg, wg, C0, n, d, k, form, steps, warmup, world, local, sample_clocks):
    """Creates a fit session for `form` and times exactly `steps` iterations."""
    import torch

    stream = torch.cuda.Stream()
    cur = torch.from_numpy(C0.copy()).cuda()
    res_c = torch.empty_like(cur)
    lab = torch.empty(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    fit = ctypes.c_void_p()
    c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    c0.record(stream)
    create = L.kmc_fit_create_f64_i32 if Xg.dtype == torch.float64 else L.kmc_fit_create_f32_i32
    capi.check(create(Xg.data_ptr(), wg.data_ptr(), cur.data_ptr(), lab.data_ptr(),
                      res_c.data_ptr(), n, d, k, 0.0, warmup + steps + 1,
                      FORMS[form], stream.cuda_stream, ctypes.byref(fit)))
    c1.record(stream)
    c1.synchronize()
    prep_ms = c0.elapsed_time(c1)
    try:
        capi.check(L.kmc_fit_set_profiling(fit, 1))
        capi.check(L.kmc_fit_step(fit, warmup))
        stream.synchronize()
        ms0, n0, l0 = ctypes.c_double(), ctypes.c_int64(), ctypes.c_int64()
        capi.check(L.kmc_fit_phase_time(fit, 0, ctypes.byref(ms0), ctypes.byref(n0)))
        capi.check(L.kmc_fit_launch_count(fit, ctypes.byref(l0)))
        r0 = ctypes.c_int64()
        capi.check(L.kmc_fit_rechecked(fit, None, ctypes.byref(r0), None))
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        uuid = None
        try:
            uuid = "GPU-" + str(torch.cuda.get_device_properties(local).uuid)
        except Exception:
            pass
        barrier(world)
        torch.cuda.synchronize()
        with ClockSampler(uuid if sample_clocks else None) as clk:
            if sample_clocks:
                time.sleep(0.15)
            ev0.record(stream)
            capi.check(L.kmc_fit_step(fit, steps))
            ev1.record(stream)
            ev1.synchronize()
            torch.cuda.synchronize()
            barrier(world)
            if sample_clocks:
                time.sleep(0.05)
        elapsed_ms = all_max(world, ev0.elapsed_time(ev1))
        ms1, n1, l1 = ctypes.c_double(), ctypes.c_int64(), ctypes.c_int64()
        capi.check(L.kmc_fit_phase_time(fit, 0, ctypes.byref(ms1), ctypes.byref(n1)))
        capi.check(L.kmc_fit_launch_count(fit, ctypes.byref(l1)))
        r1, err = ctypes.c_int64(), ctypes.c_int()
        capi.check(L.kmc_fit_rechecked(fit, None, ctypes.byref(r1), ctypes.byref(err)))
        it, done, shift = ctypes.c_int64(), ctypes.c_int(), ctypes.c_double()
        capi.check(L.kmc_fit_status(fit, ctypes.byref(it), ctypes.byref(done), ctypes.byref(shift)))
    finally:
        capi.check(L.kmc_fit_destroy(fit))
    assert it.value == warmup + steps, (it.value, "the loop stopped early")
    assert err.value == 0, "tensor-core kernel reported a device-side timeout"
    kern_ms = (ms1.value - ms0.value) / max(1, n1.value - n0.value)
    return {"value": world * steps / (elapsed_ms / 1000.0), "ms_per_step": elapsed_ms / steps,
            "kernel_ms": kern_ms, "launches": int(l1.value - l0.value),
            "rechecked_per_step": (r1.value - r0.value) / steps, "prep_ms": prep_ms,
            "clocks": clk.summary() if sample_clocks else None}


def _roofline(workload, form, n, d, k, kern_ms, clocks, sm_count, f64=False):
    peaks, peak_src = measured_peaks()
    flops = 2.0 * n * k * d
    achieved = flops / (kern_ms * 1e-3) / 1e12
    if f64:
        peak = FP64_NOMINAL_TFLOPS
        r = {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
             "peak_source": "nominal dense FP64 rate of a GB300 (no measured FP64 peak); the "
                            "plain float64 form runs on the FP64 pipe",
             "kernel": "tile_kernel (exact fused assignment + accumulation, float64)"}
    elif form == "plain":
        clk_mhz = (clocks or {}).get("sm_max_mhz") or 2070.0
        peak = sm_count * 128 * 2 * clk_mhz * 1e6 / 1e12
        r = {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
             "peak_source": f"nominal FP32 FFMA rate ({sm_count} SMs x 128 lanes x 2 flop x "
                            f"{clk_mhz:.0f} MHz); the plain form runs on the FP32 pipe",
             "kernel": "tile_kernel (exact fused assignment + accumulation)"}
    else:
        # the timed region is tens of milliseconds: the burst figure applies
        peak = peaks.get("bf16_tflops", 1900.0)
        r = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
             "peak_source": f"bf16_tflops (burst) of MEASURED_PEAKS.json ({peak_src}); the "
                            "fp16 dense tensor rate equals the bf16 one",
             "kernel": "mixed_assign_kernel + recheck_kernel (tcgen05 assignment + accumulation)"}
    per_sample = TRAFFIC_PER_SAMPLE.get((workload, form))
    r.update({"frac": achieved / peak, "traffic": per_sample * n if per_sample else None,
              "traffic_source": ("ncu capture at n=1M of this shape, scaled by n" if per_sample
                                 else "not captured for this workload"),
              "kernel_ms": kern_ms,
              "flops_per_launch": flops,
              # plain: X (fp32) once + labels; mixed: the fp16/bf16 image for the
              # contraction, the fp32 rows for the exact sums, labels
              "algorithmic_bytes_per_launch": n * d * ((8 if f64 else 4) if form == "plain" else 6) + 4 * n})
    return r


def parity_report(L, capi, X_t, C0, Xg, wg, form):
    """One Lloyd step of `form` from C0 and the final pass against the new centroids,
    compared with the oracle on the same input (outside every timed region).

    Reports the share of labels equal to the oracle's (all samples, both passes),
    the largest centroid error relative to the largest centroid coordinate, and the
    inertia's relative error against the oracle's long-double sum."""
    import torch

    from oracle import kmref

    d, n = X_t.shape
    k = C0.shape[1]
    w_h = np.ones(n, np.float32)
    cur = torch.from_numpy(C0.copy()).cuda()
    res = torch.empty_like(cur)
    lab = torch.empty(n, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    fit = ctypes.c_void_p()
    capi.check(L.kmc_fit_create_f32_i32(Xg.data_ptr(), wg.data_ptr(), cur.data_ptr(), lab.data_ptr(),
                                        res.data_ptr(), n, d, k, 0.0, 1, FORMS[form],
                                        stream.cuda_stream, ctypes.byref(fit)))
    try:
        capi.check(L.kmc_fit_step(fit, 1))
        torch.cuda.synchronize()
        lab1, C1 = lab.cpu().numpy(), cur.cpu().numpy()
        it, inr = ctypes.c_int64(), ctypes.c_double()
        capi.check(L.kmc_fit_finalize(fit, ctypes.byref(it), ctypes.byref(inr)))
        lab2 = lab.cpu().numpy()
    finally:
        capi.check(L.kmc_fit_destroy(fit))
    t0 = time.perf_counter()
    lab1_o, C1_o, _, relocated = kmref.lloyd_iteration(X_t, w_h, C0)
    lab2_o = kmref.assignment(X_t, C1)
    inr_o = kmref.sum_ld(kmref.compute_inertia(X_t, w_h, C1, lab2_o))
    return {
        "form": form,
        "what": "one Lloyd step from the initial centroids, then the final pass, vs the oracle "
                "(reference arithmetic, long-double sums) on the same input; all samples",
        "step_label_agreement": float(np.mean(lab1 == lab1_o)),
        "final_label_agreement": float(np.mean(lab2 == lab2_o)),
        "centroid_max_rel_err": float(np.abs(C1 - C1_o).max() / np.abs(C1_o).max()),
        "inertia_rel_err": abs(inr.value - inr_o) / abs(inr_o),
        "relocated": bool(relocated),
        "oracle_seconds": time.perf_counter() - t0,
    }


# ---------------------------------------------------------------------------
# batched fits (c4) and the serving stream (c5)
# ---------------------------------------------------------------------------
def _loguniform_int(rng, lo, hi):
    return int(np.exp(rng.uniform(np.log(lo), np.log(hi))))


def c4_instances(count=256, seed=4):
    """(n, d, k, seed) of the c4 batch: n log-U[2e3, 2e6], d in {8..128}, k log-U[4, 512]."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = _loguniform_int(rng, 2_000, 2_000_000)
        d = int(rng.choice([8, 16, 32, 64, 128]))
        k = min(_loguniform_int(rng, 4, 512), n)
        out.append((n, d, k, 1000 + i))
    return out


def c5_requests(capi, count=10_000, rate=500.0, seed=5):
    """The c5 request stream as kmc_serve_request_t records (seeded)."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, count))
    arr = (capi.ServeRequest * count)()
    fits = []
    for r in range(count):
        if fits and rng.random() < 0.2:
            m = fits[int(rng.integers(len(fits)))]
            d, k = arr[m].n_features, arr[m].n_clusters
            n = _loguniform_int(rng, 1_000, 1_000_000)
            arr[r] = capi.ServeRequest(float(arrivals[r]), 1, d, n, k, k, 7_000 + r, 0.0, 0, m, 1.0, 1.0)
        else:
            n = _loguniform_int(rng, 10_000, 5_000_000)
            d = int(rng.choice([16, 32, 64]))
            k = min(_loguniform_int(rng, 8, 1024), n)
            arr[r] = capi.ServeRequest(float(arrivals[r]), 0, d, n, k, k, 7_000 + r, 1e-4, 300, -1,
                                       1.0, 1.0)
            fits.append(r)
    return arr


def serve_stream(L, capi, reqs, count, form, budget=150 * 10 ** 9, max_active=512):
    """Replays the first `count` requests; returns the latency summary."""
    import torch

    sub = (capi.ServeRequest * count)(*reqs[:count])
    res = (capi.ServeResult * count)()
    mk = ctypes.c_double()
    capi.check(L.kmc_serve_run(sub, count, FORMS[form], budget, max_active,
                               torch.cuda.current_stream().cuda_stream, res, ctypes.byref(mk)))
    lat = np.array([res[r].finish_s - sub[r].arrival_s for r in range(count)])
    ok = np.array([res[r].status == 0 for r in range(count)])
    fits = np.array([sub[r].kind == 0 for r in range(count)])
    return {"requests": count, "completed": int(ok.sum()),
            "p50_s": float(np.percentile(lat[ok], 50)), "p99_s": float(np.percentile(lat[ok], 99)),
            "fit_p50_s": float(np.percentile(lat[ok & fits], 50)) if (ok & fits).any() else None,
            "predict_p50_s": float(np.percentile(lat[ok & ~fits], 50)) if (ok & ~fits).any() else None,
            "throughput_rps": count / mk.value, "makespan_s": mk.value,
            "mean_iterations": float(np.mean([res[r].n_iter for r in range(count) if sub[r].kind == 0]))}


def run_c5(args, world, rank, local):
    import torch

    from kmeans_dpcpp_gb300 import capi

    torch.cuda.set_device(local)
    L = capi.lib()
    count = args.n or 10_000
    reqs = c5_requests(capi, count)
    forms = {}
    for form in ("mixed-fp16", "plain"):
        forms[form] = serve_stream(L, capi, reqs, count, form)
    head = forms["mixed-fp16"]
    line = {"metric": "serve p50/p99 latency (c5 request stream)", "value": head["p99_s"], "unit": "s",
            "n_gpus": world, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp16", "data": "synthetic (seeded Gaussian blobs generated on the device at admission)",
            "config": {"workload": "c5", "requests": count, "arrival_rate_per_s": 500.0,
                       "hbm_budget_bytes": 150 * 10 ** 9, "parallelism": f"replicas{world}"},
            "forms": forms}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_c4(args, world, rank, local):
    import torch

    from kmeans_dpcpp_gb300 import capi

    torch.cuda.set_device(local)
    L = capi.lib()
    inst = c4_instances()
    if args.n:
        inst = inst[:args.n]
    stream = torch.cuda.current_stream()
    s = stream.cuda_stream
    data = []
    for (n, d, k, sd) in inst:
        X = torch.empty((d, n), dtype=torch.float32, device="cuda")
        capi.check(L.kmc_generate_blobs_f32(X.data_ptr(), n, d, k, -10.0, 10.0, 1.0, 1.0, sd, s))
        rows = (ctypes.c_int32 * k)()
        capi.check(L.kmc_seeded_rows(n, k, sd, rows))
        C0 = X[:, torch.tensor(list(rows), dtype=torch.int64, device="cuda")].contiguous()
        data.append((X, C0))
    w_all = {n: torch.ones(n, dtype=torch.float32, device="cuda") for (n, _, _, _) in inst}
    iters = 50
    # the autotuner measures each (d, k bucket) once, outside the timed region
    for (n, d, k, _) in inst:
        v = ctypes.c_int()
        capi.check(L.kmc_tile_variant(d, k, s, ctypes.byref(v)))

    def batched():
        h = ctypes.c_void_p()
        capi.check(L.kmc_batch_create(len(inst), s, ctypes.byref(h)))
        keep = []
        try:
            for (n, d, k, _), (X, C0) in zip(inst, data):
                C = C0.clone()
                lab = torch.empty(n, dtype=torch.int32, device="cuda")
                keep.append((C, lab))
                q = ctypes.c_int64()
                capi.check(L.kmc_batch_add_fit_f32(h, X.data_ptr(), w_all[n].data_ptr(), C.data_ptr(),
                                                   lab.data_ptr(), n, d, k, 0.0, iters, ctypes.byref(q)))
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            capi.check(L.kmc_batch_run(h))
            torch.cuda.synchronize()
            return time.perf_counter() - t0
        finally:
            capi.check(L.kmc_batch_destroy(h))

    def single_loop():
        t = 0.0
        for (n, d, k, _), (X, C0) in zip(inst, data):
            C = C0.clone()
            res = torch.empty_like(C)
            lab = torch.empty(n, dtype=torch.int32, device="cuda")
            fit = ctypes.c_void_p()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            capi.check(L.kmc_fit_create_f32_i32(X.data_ptr(), w_all[n].data_ptr(), C.data_ptr(),
                                                lab.data_ptr(), res.data_ptr(), n, d, k, 0.0, iters, 0, s,
                                                ctypes.byref(fit)))
            try:
                capi.check(L.kmc_fit_run(fit))
                it, inr = ctypes.c_int64(), ctypes.c_double()
                capi.check(L.kmc_fit_finalize(fit, ctypes.byref(it), ctypes.byref(inr)))
            finally:
                capi.check(L.kmc_fit_destroy(fit))
            torch.cuda.synchronize()
            t += time.perf_counter() - t0
        return t

    def served_mixed():
        # the mixed form's batched path: the request server runs the fits as
        # concurrent graph-replayed tensor-core sessions
        srv = ctypes.c_void_p()
        capi.check(L.kmc_server_open(FORMS["mixed-fp16"], 150 * 10 ** 9, len(inst), s, ctypes.byref(srv)))
        keep, tickets = [], []
        try:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for (n, d, k, _), (X, C0) in zip(inst, data):
                lab = torch.empty(n, dtype=torch.int32, device="cuda")
                Cout = torch.empty_like(C0)
                keep.append((lab, Cout))
                q = ctypes.c_int64()
                capi.check(L.kmc_server_submit_fit_f32(srv, X.data_ptr(), w_all[n].data_ptr(), C0.data_ptr(),
                                                       lab.data_ptr(), Cout.data_ptr(), n, d, k, 0.0, iters,
                                                       ctypes.byref(q)))
                tickets.append(q.value)
            done_iters = 0
            for q in tickets:
                st, it, inr = ctypes.c_int(), ctypes.c_int64(), ctypes.c_double()
                capi.check(L.kmc_server_wait(srv, q, ctypes.byref(st), ctypes.byref(it), ctypes.byref(inr)))
                capi.check(st.value)
                done_iters += it.value
            torch.cuda.synchronize()
            return time.perf_counter() - t0, done_iters
        finally:
            capi.check(L.kmc_server_close(srv))

    def single_mixed_loop():
        t, done_iters = 0.0, 0
        for (n, d, k, _), (X, C0) in zip(inst, data):
            C = C0.clone()
            res = torch.empty_like(C)
            lab = torch.empty(n, dtype=torch.int32, device="cuda")
            fit = ctypes.c_void_p()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            capi.check(L.kmc_fit_create_f32_i32(X.data_ptr(), w_all[n].data_ptr(), C.data_ptr(),
                                                lab.data_ptr(), res.data_ptr(), n, d, k, 0.0, iters,
                                                FORMS["mixed-fp16"], s, ctypes.byref(fit)))
            try:
                capi.check(L.kmc_fit_run(fit))
                it, inr = ctypes.c_int64(), ctypes.c_double()
                capi.check(L.kmc_fit_finalize(fit, ctypes.byref(it), ctypes.byref(inr)))
                done_iters += it.value
            finally:
                capi.check(L.kmc_fit_destroy(fit))
            torch.cuda.synchronize()
            t += time.perf_counter() - t0
        return t, done_iters

    batched()  # warm-up: allocator pools, graphs, kernel attributes
    t_batch = batched()
    t_single = single_loop()
    served_mixed()  # warm-up
    t_mixed, it_mixed = served_mixed()
    t_mixed_single, it_mixed_single = single_mixed_loop()
    total = len(inst) * iters
    flops = sum(2.0 * n * k * d for (n, d, k, _) in inst) * iters
    line = {"metric": "batched fits: instance-iterations/s (c4)", "value": total / t_batch,
            "unit": "instance-iter/s", "n_gpus": world, "steps": iters, "warmup": 1,
            "ms_per_step": 1e3 * t_batch / iters, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Gaussian blobs on the device)",
            "config": {"workload": "c4", "instances": len(inst), "iterations": iters,
                       "total_samples": sum(i[0] for i in inst), "parallelism": f"replicas{world}"},
            "distance_tflops": flops / t_batch / 1e12,
            "single_fit_loop": {"value": total / t_single, "seconds": t_single},
            "speedup_vs_single_fit_loop": t_single / t_batch,
            "batched_seconds": t_batch,
            "mixed_fp16": {"value": it_mixed / t_mixed, "unit": "instance-iter/s", "seconds": t_mixed,
                           "instance_iterations": it_mixed,
                           "path": "request server: concurrent graph-replayed tensor-core sessions",
                           "single_fit_loop": {"value": it_mixed_single / t_mixed_single,
                                               "seconds": t_mixed_single},
                           "speedup_vs_single_fit_loop": (it_mixed / t_mixed) / (it_mixed_single / t_mixed_single)}}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_gb300(args, world, rank, local):
    import torch

    import kmeans_dpcpp_gb300 as kdp
    from kmeans_dpcpp_gb300 import capi

    torch.cuda.set_device(local)
    L = capi.lib()
    w = workload(args.workload, args.n)
    n, d, k = w["n"], w["d"], w["k"]
    X_t, C0 = workload_data(args.workload, args.n)
    f64 = X_t.dtype == np.float64
    # the mixed tensor-core forms take float32 data
    form = ("plain" if f64 else "mixed-fp16") if args.form == "auto" else args.form
    sm_count = torch.cuda.get_device_properties(local).multi_processor_count

    Xg = torch.from_numpy(X_t).cuda()
    wg = torch.ones(n, dtype=Xg.dtype, device="cuda")
    head = _time_form(L, capi, Xg, wg, C0, n, d, k, form, args.steps, args.warmup, world, local, True)
    forms = {form: head}
    if not args.no_compare and not f64:
        for other in ("plain", "mixed-bf16", "mixed-fp16"):
            if other not in forms:
                st = min(args.steps, 10) if other == "plain" else args.steps
                forms[other] = _time_form(L, capi, Xg, wg, C0, n, d, k, other, st, args.warmup, world,
                                          local, False)
    roofline = _roofline(args.workload, form, n, d, k, head["kernel_ms"], head["clocks"], sm_count,
                         f64=f64)

    # ---- end to end through the drop-in surface, host buffers ----
    e2e = None
    if not args.no_e2e:
        # The pinned host buffers are allocated and filled from the CPUs next
        # to the GPU, so their pages sit on the GPU's side of the host (a
        # caller placing its buffers would do the same); the affinity is
        # restored afterwards.
        saved = os.sched_getaffinity(0)
        near = gpu_local_cpus(local)
        if near:
            os.sched_setaffinity(0, near)
        try:
            X_h = torch.from_numpy(X_t).pin_memory()
            w_h = torch.ones(n, dtype=Xg.dtype).pin_memory()
            C_h = torch.from_numpy(C0.copy()).pin_memory()
            lab_h = torch.empty(n, dtype=torch.int32).pin_memory()
            Cres_h = torch.empty_like(C_h).pin_memory()
        finally:
            os.sched_setaffinity(0, saved)
        Xd = torch.empty_like(Xg)
        wd = torch.empty_like(wg)
        Cd = torch.from_numpy(C0.copy()).cuda()
        Crd = torch.empty_like(Cd)
        labd = torch.empty(n, dtype=torch.int32, device="cuda")
        barrier(world)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Xd.copy_(X_h, non_blocking=True)
        wd.copy_(w_h, non_blocking=True)
        Cd.copy_(C_h, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        t1 = time.perf_counter()
        n_iter, inertia = kdp.kmeans_lloyd_driver(Xd, wd, Cd, labd, Crd, 0.0, False, args.steps, 8, 128,
                                                  0.7, None, form=form)
        t2 = time.perf_counter()
        lab_h.copy_(labd)
        Cres_h.copy_(Crd)
        torch.cuda.synchronize()
        t3 = time.perf_counter()
        t_e2e = all_max(world, t3 - t0)
        assert n_iter == args.steps
        h2d = X_t.nbytes + X_t.itemsize * n + C0.nbytes
        d2h = 4 * n + C0.nbytes + X_t.itemsize
        e2e = {"value": world * n_iter / t_e2e, "unit": "iter/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h,
               "host_buffers_on_cpus": (("%d CPUs local to the GPU" % len(near)) if near
                                        else "not placed (no local CPU list)"),
               "split_ms": {"h2d": 1e3 * (t1 - t0), "driver_call": 1e3 * (t2 - t1),
                            "d2h": 1e3 * (t3 - t2)},
               "note": "one kmeans_lloyd_driver call (form=%s) of K iterations (tol=0): pinned-host "
                       "copies of X, weights, init centroids in and labels, centroids, inertia out, "
                       "plus the one-time operand conversion; bytes are per call" % form}
        del Xd, X_h

    line = {
        "metric": METRIC, "value": head["value"], "unit": "iter/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": ("f64" if f64 else "f32") if form == "plain" else form.split("-")[1],
        "data": "synthetic",
        "config": {"workload": args.workload, "desc": w["desc"], "n": n, "d": d, "k": k,
                   "form": form, "parallelism": f"replicas{world}",
                   "l2": "inputs larger than L2 (X is %.2f GB)" % (X_t.nbytes / 1e9)},
        "roofline": roofline,
        "clocks": head["clocks"],
        "gpu_launches": head["launches"],
        "e2e": e2e,
        "forms": {f: {kk: v for kk, v in r.items() if kk != "clocks"} for f, r in forms.items()},
    }
    if "plain" in forms and form != "plain":
        line["speedup_vs_plain_fp32"] = head["value"] / forms["plain"]["value"]
    if args.serve_sample > 0:
        reqs = c5_requests(capi, args.serve_sample)
        line["serve"] = {"sample": "first %d requests of the c5 stream (Poisson 500/s, 150 GB "
                                   "admission budget)" % args.serve_sample,
                         "forms": {f: serve_stream(L, capi, reqs, args.serve_sample, f)
                                   for f in ("mixed-fp16", "plain")}}
    if rank == 0 and not args.no_parity and form != "plain":
        line["parity"] = parity_report(L, capi, X_t, C0, Xg, wg, form)
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(X_t, C0, target_s=args.cpu_seconds)
    if rank == 0:
        print(json.dumps(line), flush=True)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--form", choices=["auto"] + sorted(FORMS), default="auto")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + ["c4", "c5"], default="c3")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the parity block (one step + final pass against the oracle)")
    ap.add_argument("--no-compare", action="store_true",
                    help="time only the headline form (no plain / other mixed comparison)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--n", type=int, default=None,
                    help="fewer samples than the workload names (small profiling captures); "
                         "for c4 / c5 the number of instances / requests")
    ap.add_argument("--serve-sample", type=int, default=300,
                    help="requests of the c5 stream replayed for the serve key (0: skip)")
    args = ap.parse_args(argv)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        world = int(os.environ.get("WORLD_SIZE", "1"))
        rank = int(os.environ.get("RANK", "0"))
        run_reference(args, world, rank)
        return
    world, rank, local = dist_setup(args.gpus)
    if args.workload == "c4":
        run_c4(args, world, rank, local)
    elif args.workload == "c5":
        run_c5(args, world, rank, local)
    else:
        run_gb300(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
