"""Benchmark of the radar path tracer on GB300 (one JSON line on rank 0).

Workload (one step): the tessellated PEC sphere above a ground plane — icosphere level 6
(81,920 triangles, r = 0.5 m) on a 20 m x 20 m ground quad, sensor at 10 m range and
0.5 m height, up to 3 bounces, 2^22 Halton samples, one chirp 77-81 GHz with 512 ADC
samples — traced by one persistent launch of the plain FP32 path with the reference's
33-bin frame splat. The metric is paths/s.

  value  device-timed (CUDA events on the launching stream) throughput with poses,
         budgets and the scene BVH resident in HBM; L2 is flushed between steps by
         writing a 512 MiB buffer (outside the timed events).
  e2e    the same metric through the public C ABI call with HOST buffers
         (hsr_simulate_batch: pinned poses/budgets in, the normalised frame row out,
         synchronised), wall-clock per step.
  roofline  dominant kernel k_trace: algorithmic bytes = exact BVH node (64 B) and
         triangle (48 B) fetches of a counting launch over the same samples, divided by
         the kernel's CUDA-event time; peak = measured HBM copy bandwidth.
  cpu_baseline  the oracle's FP32 restatement with its own BVH, on all host cores, on a
         bounded sample of the same workload.

--impl reference times the CPU restatement of the reference path (the reference itself
needs Embree/OptiX/Eigen, absent here) on the host cores with the same metric.
Multi-GPU: replicas (each rank traces its own disjoint Halton range of the same pose;
no collective on the data path), reported as weak scaling.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "paths/s"
WORKLOAD = "icosphere-L6 (81,920 tris) + 20x20 m ground, sensor 10 m / 0.5 m, 3 bounces, 2^22 samples, N=512"


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


def init_dist(world):
    if world <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo")
    return dist


def max_over_ranks(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            import tempfile
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def cpu_baseline(w, tracer, samples, threads=0):
    """The oracle's FP32 restatement (test infrastructure) timed on the host cores."""
    from oracle import pyoracle
    ora = pyoracle.Scene(w.mesh)
    t0 = time.perf_counter()
    ora.simulate(w.rf, w.frame, w.tx[0], w.rx[0], tracer, samples, precision=32, threads=threads)
    dt = time.perf_counter() - t0
    cores = threads or os.cpu_count()
    return samples / dt, cores, dt


def run_reference(args, rank, world, dist):
    """--impl reference: the CPU restatement of the reference path on the host cores."""
    if rank != 0:
        return
    from hussar_gb300 import PathTracer, scenes
    from oracle import pyoracle
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
    w = scenes.sphere_ground_workload(samples=1 << 22)
    t = PathTracer()
    t.doGuiding = False
    t.maxDepth = w.max_depth
    ora = pyoracle.Scene(w.mesh)
    sample = args.ref_samples
    for _ in range(args.warmup):
        ora.simulate(w.rf, w.frame, w.tx[0], w.rx[0], t, sample // 8, precision=32)
    times = []
    for k in range(args.steps):
        t0 = time.perf_counter()
        ora.simulate(w.rf, w.frame, w.tx[0], w.rx[0], t, sample, offset=k * sample, precision=32)
        times.append(time.perf_counter() - t0)
    ms = 1000.0 * sum(times) / len(times)
    value = sample / (ms / 1000.0)
    cores = os.cpu_count()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "samples_per_step": sample, "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": value, "unit": "paths/s", "cores": cores, "kind": "port",
                         "sample": "%d Halton samples of the same pose per step (of 2^22)" % sample},
        "e2e": {"value": value, "unit": "paths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gb300(args, rank, world, local_rank, dist):
    import ctypes

    import torch

    from hussar_gb300 import PathTracer, _lib, gb300, scenes

    torch.cuda.set_device(local_rank)
    L = _lib.lib()
    w = scenes.sphere_ground_workload(samples=1 << 22)
    S = int(w.budget[0])
    t = PathTracer()
    t.doGuiding = False
    t.maxDepth = w.max_depth
    be = gb300.Backend(w.mesh, None)
    N = w.frame.samplesPerChirp
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.current_stream(dev)
    txa = w.tx[0].to_c()
    ant_bytes = bytes(txa)
    d_tx = torch.frombuffer(bytearray(ant_bytes), dtype=torch.uint8).to(dev)
    d_rx = d_tx.clone()
    d_budget = torch.tensor([S], dtype=torch.int64, device=dev)
    # each rank traces its own Halton range [rank*S, (rank+1)*S): replicas, weak scaling
    d_offset = torch.tensor([rank * S], dtype=torch.int64, device=dev)
    d_rows = torch.zeros(2 * N, dtype=torch.float32, device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    rf_c = w.rf.to_c()
    fl_c = t.flags_c()

    def step():
        _lib.check(L.hsr_simulate_batch_device(
            be.handle, ctypes.byref(rf_c), N, ctypes.byref(fl_c), 1, ctypes.c_void_p(d_tx.data_ptr()),
            ctypes.c_void_p(d_rx.data_ptr()), ctypes.c_void_p(d_budget.data_ptr()),
            ctypes.c_void_p(d_offset.data_ptr()), _lib.HSR_PHASE_REFERENCE_FP32, _lib.HSR_SPLAT_DIRICHLET16,
            ctypes.c_void_p(d_rows.data_ptr()), ctypes.c_void_p(stream.cuda_stream)))

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()

    clocks = ClockSampler(local_rank)
    barrier(dist)
    torch.cuda.synchronize()
    clocks.start()
    launches0 = L.hsr_launch_count()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    kernel_ms = []
    for k in range(args.steps):
        flush.fill_(k & 0xff)  # > L2 (129 MB), outside the timed events
        ev[k][0].record(stream)
        step()
        ev[k][1].record(stream)
        if args.kernel_times:
            kms = ctypes.c_float()
            _lib.check(L.hsr_last_kernel_ms(be.handle, ctypes.byref(kms)))
            kernel_ms.append(kms.value)
    torch.cuda.synchronize()
    launches = L.hsr_launch_count() - launches0
    barrier(dist)
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    ms = max_over_ranks(dist, sum(step_ms) / len(step_ms))
    value = world * S / (ms / 1000.0)

    if args.kernel_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world,
                              "steps": args.steps, "ms_per_step": ms, "kernel_only": True,
                              "gpu_launches": int(launches), "clocks": clk}), flush=True)
        return

    # trace-kernel time alone (events around the kernel inside the library), for the roofline
    kms = ctypes.c_float()
    flush.fill_(1)
    step()
    _lib.check(L.hsr_last_kernel_ms(be.handle, ctypes.byref(kms)))
    trace_ms = kms.value

    # e2e through the public host-buffer API: pinned poses in, normalised row out, synchronous
    P = 1
    h_tx = (_lib.AntennaC * P)(txa)
    h_rx = (_lib.AntennaC * P)(txa)
    h_budget = torch.tensor([S], dtype=torch.int64).pin_memory()
    h_offset = torch.tensor([rank * S], dtype=torch.int64).pin_memory()
    h_rows = torch.zeros(2 * N, dtype=torch.float32).pin_memory()
    e2e_times = []
    for k in range(args.steps):
        flush.fill_(k & 0xff)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _lib.check(L.hsr_simulate_batch(
            be.handle, ctypes.byref(rf_c), N, ctypes.byref(fl_c), P, ctypes.cast(h_tx, ctypes.c_void_p),
            ctypes.cast(h_rx, ctypes.c_void_p), ctypes.c_void_p(h_budget.data_ptr()),
            ctypes.c_void_p(h_offset.data_ptr()), _lib.HSR_PHASE_REFERENCE_FP32, _lib.HSR_SPLAT_DIRICHLET16,
            ctypes.c_void_p(h_rows.data_ptr()), ctypes.c_void_p(stream.cuda_stream)))
        e2e_times.append(time.perf_counter() - t0)
    e2e_ms = max_over_ranks(dist, 1000.0 * sum(e2e_times) / len(e2e_times))
    h2d = 2 * ctypes.sizeof(_lib.AntennaC) * P + 16 * P
    d2h = 8 * N * P

    if rank != 0:
        return
    counts = be.traversal_counts(w.rf, N, t, w.tx, w.rx, [S], [0])
    peak, peak_kind = measured_peaks()
    achieved = counts["bytes"] / (trace_ms / 1000.0) / 1e9
    cores = os.cpu_count()
    cpu_val, cpu_cores, cpu_s = cpu_baseline(w, t, args.cpu_samples)
    line = {
        "metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "paths_per_step_per_gpu": S, "poses": 1, "max_bounces": 3,
                   "range_bins": N, "phase": "reference-fp32", "splat": "dirichlet16",
                   "l2": "flushed between steps (512 MiB write)", "parallelism": "replicas x%d" % world},
        "e2e": {"value": world * S / (e2e_ms / 1000.0), "unit": "paths/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None, "kernel": "k_trace",
                     "kernel_ms": trace_ms, "algorithmic_bytes": counts["bytes"], "rays": counts["rays"],
                     "nodes": counts["nodes"], "tris": counts["tris"], "peak_source": peak_kind},
        "cpu_baseline": {"value": cpu_val, "unit": "paths/s", "cores": cpu_cores, "kind": "port",
                         "sample": "%d Halton samples of the same pose (%.1f s wall)" % (args.cpu_samples, cpu_s)},
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-samples", type=int, default=1 << 20)
    ap.add_argument("--ref-samples", type=int, default=1 << 20)
    ap.add_argument("--kernel-times", action="store_true")
    ap.add_argument("--kernel-only", action="store_true",
                    help="timed steps only (no e2e, counting, CPU baseline): the profiling command")
    args = ap.parse_args()
    rank, world, local_rank = dist_env()
    dist = init_dist(world)
    if args.impl == "reference":
        run_reference(args, rank, world, dist)
    else:
        run_gb300(args, rank, world, local_rank, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
