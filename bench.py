"""Benchmark of the radar path tracer on GB300 (one JSON line on rank 0).

Workload (default, --workload boxes): the batched configuration -- one seeded scene of
~1 M triangles (83,334 random axis-aligned boxes, edges 0.2-5 m, on a 100 m x 100 m
ground quad) viewed from 4096 sensor poses at 1 m height with random yaw, per-pose
budgets log-uniform in 2^16..2^22 Halton samples, up to 4 bounces, 256 range bins. One
step is one batch of 256 of the 4096 poses (step k traces batch k mod 16, so 16 steps
cover every pose once) run as one persistent launch inside a captured CUDA graph, in the
product's batched form: split-FP64 phase and the fine range histogram synthesised into
the 256 IF bins by the split-BF16 tcgen05 GEMM. The metric is paths/s.

  value  device-timed (CUDA events on the launching stream) throughput with the 4096
         poses, budgets and the scene BVH resident in HBM; L2 is flushed between steps by
         writing a 512 MiB buffer (outside the timed events).
  e2e    the same metric through the public C ABI call with HOST buffers
         (hsr_simulate_batch: pinned poses/budgets in, the normalised rows out,
         synchronised), wall-clock per step.
  roofline  dominant kernel k_wave (the traversal): algorithmic bytes = exact BVH node
         (64 B) and triangle (48 B) fetches of a counting launch over a quarter of the
         batch's poses (scaled by paths), divided by the kernel's CUDA-event time. The BVH
         (112 MB) is L2-resident, so the bound is the L2: peak = the L2 read bandwidth
         measured live (hsr_measure_l2_read); the HBM fraction is reported beside it.
  cpu_baseline  the oracle's FP32 restatement with its own BVH, on all host cores, on a
         bounded sample of the same workload.

--workload sphere: the sphere+ground configuration (icosphere level 6 on a 20 m ground
quad, 2^22 samples, 3 bounces, 512 bins) in the plain FP32 form with the reference's
33-bin splat. --workload serve: the serving loop (hsr_server_*): 8 resident scenes of
100 k .. 5 M triangles, a Poisson request stream (--rate req/s for --duration s);
p50/p99 latency and paths/s through the public API. --workload tte: time to -40 dB only.

--impl reference times the CPU restatement of the reference path (the reference itself
needs Embree/OptiX/Eigen, absent here) on the host cores with the same metric and config.
Multi-GPU: replicas (each rank traces its own disjoint Halton range of the same poses;
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
# DRAM bytes of one k_wave launch of the sphere bench (dram__bytes_read.sum +
# dram__bytes_write.sum from an ncu --set full capture of the first timed step of
# `bench.py --kernel-only`)
NCU_TRAFFIC = {"sphere": 4.415232e6 + 30.72e3}
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


def replica_range(rank, samples_per_rank):
    """Halton index range of one replica: rank r traces [r * S, (r + 1) * S), so the union
    over ranks is exactly the single-process sample set [0, world * S)."""
    return rank * samples_per_rank, samples_per_rank


def sum_frames(dist, frame):
    """Host-side sum of the replicas' raw frames (KB-sized; outside any timed region)."""
    if dist is None:
        return frame
    import torch
    t = torch.from_numpy(frame.astype(np.complex128).view(np.float64).copy())
    dist.all_reduce(t)
    return t.numpy().view(np.complex128).reshape(frame.shape)


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
        return {"sm_mhz": statistics.median(sm), "sm_min_mhz": min(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def l2_read_gbs(mib=32, sweeps=64):
    """Read bandwidth of an L2-resident `mib` MiB buffer (hsr_measure_l2_read: one launch
    of `sweeps` L2-cached passes, best of five): the L2 denominator for traversal, whose
    working set mostly stays in L2 (MEASURED_PEAKS.json holds HBM and tensor peaks)."""
    import ctypes

    from hussar_gb300 import _lib
    out = ctypes.c_double()
    _lib.check(_lib.lib().hsr_measure_l2_read(mib << 20, sweeps, ctypes.byref(out)))
    return out.value


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


BOXES_BATCH = 256  # poses per step of the batched configuration (4096 = 16 batches)
REF_POSES, REF_LOG2 = 4, 17  # the CPU arm's bounded sample per step: poses x samples


def run_reference(args, rank, world, dist):
    """--impl reference: the CPU restatement of the reference path on the host cores, on the
    GPU arm's workload. Each step is a bounded sample of one step's batch: the first
    REF_POSES poses of batch k mod 16 at 2^REF_LOG2 Halton samples each (sphere: 2^20 of
    the pose's 2^22); the metric is the same paths/s."""
    if rank != 0:
        return
    from hussar_gb300 import PathTracer
    from oracle import pyoracle
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
    w, desc = load_workload(args.workload)
    t = PathTracer()
    t.doGuiding = False
    t.maxDepth = w.max_depth
    ora = pyoracle.Scene(w.mesh)
    if args.workload == "boxes":
        def sample(k):
            b = (k % (len(w.tx) // BOXES_BATCH)) * BOXES_BATCH
            return [(w.tx[b + i], w.rx[b + i], 1 << REF_LOG2, 0) for i in range(REF_POSES)]
        what = "the first %d poses of step k's 256-pose batch, 2^%d Halton samples each" % (REF_POSES, REF_LOG2)
    else:
        def sample(k):
            return [(w.tx[0], w.rx[0], args.ref_samples, k * args.ref_samples)]
        what = "%d Halton samples of the pose per step (of 2^22)" % args.ref_samples

    def run(k, scale=1):
        n = 0
        for tx, rx, b, off in sample(k):
            ora.simulate(w.rf, w.frame, tx, rx, t, max(1, b // scale), offset=off, precision=32)
            n += max(1, b // scale)
        return n

    for k in range(args.warmup):
        run(k, 8)
    times, paths = [], 0
    for k in range(args.steps):
        t0 = time.perf_counter()
        paths += run(k)
        times.append(time.perf_counter() - t0)
    ms = 1000.0 * sum(times) / len(times)
    value = paths / sum(times)
    cores = os.cpu_count()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": desc, "samples_per_step": paths // args.steps, "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": value, "unit": "paths/s", "cores": cores, "kind": "port", "sample": what},
        "e2e": {"value": value, "unit": "paths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def load_workload(name, poses=None):
    """The bench workloads: the sphere+ground scene (the headline) or the boxes batch
    (4096 poses; --poses takes the first P of them)."""
    from hussar_gb300 import scenes
    if name == "boxes":
        w = scenes.boxes_workload()
        if poses:
            w.tx, w.rx, w.budget = w.tx[:poses], w.rx[:poses], w.budget[:poses]
        desc = ("boxes: %d triangles (83,334 random boxes) on a 100x100 m ground quad, %d poses at 1 m with random "
                "yaw, log-uniform budgets 2^16..2^22, 4 bounces, N=256" % (w.mesh.triangleCount(), len(w.tx)))
        return w, desc
    return scenes.sphere_ground_workload(samples=1 << 22), WORKLOAD


class DeviceBatch:
    """A workload's poses, budgets and output rows resident on the device."""

    def __init__(self, w, dev, rank, torch, _lib):
        P = len(w.tx)
        self.P, self.N = P, w.frame.samplesPerChirp
        self.paths = int(w.budget.sum())

        def to_dev(arr):
            return torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8).to(dev)

        self.h_tx = (_lib.AntennaC * P)(*[a.to_c() for a in w.tx])
        self.h_rx = (_lib.AntennaC * P)(*[a.to_c() for a in w.rx])
        self.d_tx, self.d_rx = to_dev(self.h_tx), to_dev(self.h_rx)
        self.d_budget = torch.from_numpy(w.budget.astype(np.int64)).to(dev)
        # each rank traces its own Halton range of every pose: replicas, weak scaling
        off = np.array([replica_range(rank, int(b))[0] for b in w.budget], np.int64)
        self.d_offset = torch.from_numpy(off).to(dev)
        self.h_budget = torch.from_numpy(w.budget.astype(np.int64)).pin_memory()
        self.h_offset = torch.from_numpy(off).pin_memory()
        self.d_rows = torch.zeros(2 * P * self.N, dtype=torch.float32, device=dev)
        self.h_rows = torch.zeros(2 * P * self.N, dtype=torch.float32).pin_memory()


def run_gb300(args, rank, world, local_rank, dist):
    import ctypes

    import torch

    from hussar_gb300 import PathTracer, _lib, gb300

    torch.cuda.set_device(local_rank)
    L = _lib.lib()
    w, desc = load_workload(args.workload, args.poses)
    t = PathTracer()
    t.doGuiding = False
    t.maxDepth = w.max_depth
    be = gb300.Backend(w.mesh, None)
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.current_stream(dev)
    B = DeviceBatch(w, dev, rank, torch, _lib)
    N, P = B.N, B.P
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    rf_c = w.rf.to_c()
    fl_c = t.flags_c()
    vp = ctypes.c_void_p

    def step(splat=_lib.HSR_SPLAT_DIRICHLET16, flags=fl_c):
        _lib.check(L.hsr_simulate_batch_device(
            be.handle, ctypes.byref(rf_c), N, ctypes.byref(flags), P, vp(B.d_tx.data_ptr()), vp(B.d_rx.data_ptr()),
            vp(B.d_budget.data_ptr()), vp(B.d_offset.data_ptr()), _lib.HSR_PHASE_REFERENCE_FP32, splat,
            vp(B.d_rows.data_ptr()), vp(stream.cuda_stream)))

    def timed(fn, steps):
        """Device time per step (CUDA events on the launching stream, L2 flushed between steps)."""
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for k in range(steps):
            flush.fill_(k & 0xff)  # > L2 (129 MB), outside the timed events
            ev[k][0].record(stream)
            fn()
            ev[k][1].record(stream)
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in ev]

    # the product's own autotuner picks the launch shape on a bounded sample of this batch
    # (at most 16 poses, budgets capped at 2^20); later plain runs on the scene use it
    sub = min(P, 16)
    if args.launch_config:  # a fixed shape (profiling runs reproduce the tuned one without tuning)
        vals = [int(x) for x in args.launch_config.split(",")] + [0]
        be.set_launch_config(*vals[:5])
        tuned = dict(zip(("tile", "ctas_per_sm", "queue_threshold", "field_on_hit", "coherent_order"), vals[:5]),
                     trace_ms=None, default_trace_ms=None)
    else:
        tuned = be.autotune(w.rf, N, t, w.tx[:sub], w.rx[:sub], np.minimum(w.budget[:sub], 1 << 20))
    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()

    clocks = ClockSampler(local_rank)
    barrier(dist)
    torch.cuda.synchronize()
    clocks.start()
    launches0 = L.hsr_launch_count()
    step_ms = timed(step, args.steps)
    launches = L.hsr_launch_count() - launches0
    barrier(dist)
    clk = clocks.stop()
    ms = max_over_ranks(dist, sum(step_ms) / len(step_ms))
    value = world * B.paths / (ms / 1000.0)

    if args.kernel_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world,
                              "steps": args.steps, "ms_per_step": ms, "kernel_only": True, "workload": desc,
                              "gpu_launches": int(launches), "clocks": clk}), flush=True)
        return

    # trace-kernel time alone (events around the kernel inside the library), for the roofline
    kms = ctypes.c_float()
    flush.fill_(1)
    step()
    _lib.check(L.hsr_last_kernel_ms(be.handle, ctypes.byref(kms)))
    trace_ms = kms.value

    # e2e through the public host-buffer API: pinned poses in, normalised rows out, synchronous
    e2e_times = []
    for k in range(args.steps):
        flush.fill_(k & 0xff)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _lib.check(L.hsr_simulate_batch(
            be.handle, ctypes.byref(rf_c), N, ctypes.byref(fl_c), P, ctypes.cast(B.h_tx, vp),
            ctypes.cast(B.h_rx, vp), vp(B.h_budget.data_ptr()), vp(B.h_offset.data_ptr()),
            _lib.HSR_PHASE_REFERENCE_FP32, _lib.HSR_SPLAT_DIRICHLET16, vp(B.h_rows.data_ptr()),
            vp(stream.cuda_stream)))
        e2e_times.append(time.perf_counter() - t0)
    e2e_ms = max_over_ranks(dist, 1000.0 * sum(e2e_times) / len(e2e_times))
    h2d = 2 * ctypes.sizeof(_lib.AntennaC) * P + 16 * P
    d2h = 8 * N * P

    # the other estimator forms on the same inputs: fine-histogram synthesis and guiding
    modes = {}
    for _ in range(2):  # warm-up: builds and caches the twiddle operand for N bins
        step(_lib.HSR_SPLAT_FINE_SYNTH)
    torch.cuda.synchronize()
    fine_ms = timed(lambda: step(_lib.HSR_SPLAT_FINE_SYNTH), max(2, args.steps // 2))
    fine_ms = max_over_ranks(dist, sum(fine_ms) / len(fine_ms))
    flush.fill_(2)
    step(_lib.HSR_SPLAT_FINE_SYNTH)
    _lib.check(L.hsr_last_kernel_ms(be.handle, ctypes.byref(kms)))
    fine_trace_ms = kms.value
    kk = 2 * 4 * 8 * N  # reduction length of the real synthesis GEMM (4 moments, 8 sub-bins)
    useful = 2.0 * P * (kk // 2) * (2 * N) * 2  # complex [P x 32N] x [32N x N]: 8 P (32N) N real flops
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    tc_peak = peaks.get("bf16_tflops", 1900.0)
    synth_ms = max(fine_ms - fine_trace_ms, 1e-6)
    modes["fine_synth"] = {"value": world * B.paths / (fine_ms / 1000.0), "unit": "paths/s", "ms_per_step": fine_ms,
                           "trace_ms": fine_trace_ms, "synthesis_ms": synth_ms,
                           "synthesis_gemm": {"bound": "tensor", "useful_tflop": useful / 1e12,
                                              "achieved_tflops": useful / (synth_ms / 1000.0) / 1e12,
                                              "peak_tflops": tc_peak,
                                              "note": "step time minus trace-kernel time; split-BF16 products "
                                                      "(6x) not counted as useful"}}
    if args.workload == "sphere":
        gfl = t.flags_c()
        gfl.doGuiding = 1
        step(_lib.HSR_SPLAT_DIRICHLET16, gfl)
        g_ms = timed(lambda: step(_lib.HSR_SPLAT_DIRICHLET16, gfl), 2)
        g_ms = max_over_ranks(dist, sum(g_ms) / len(g_ms))
        modes["guided"] = {"value": world * B.paths / (g_ms / 1000.0), "unit": "paths/s", "ms_per_step": g_ms,
                           "note": "PathTracer::run doubling schedule with device guiding over the same budget"}

    if rank != 0:
        return
    # exact traversal work of the same launch (counting instantiation); the boxes batch is
    # counted on a subsample of poses and scaled by paths
    if P == 1:
        counts = be.traversal_counts(w.rf, N, t, w.tx, w.rx, w.budget, [0])
        scale = 1.0
    else:
        sub = np.arange(0, P, max(1, P // 64))
        counts = be.traversal_counts(w.rf, N, t, [w.tx[i] for i in sub], [w.rx[i] for i in sub], w.budget[sub])
        scale = B.paths / float(w.budget[sub].sum())
    alg_bytes = counts["bytes"] * scale
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / (trace_ms / 1000.0) / 1e9
    l2_gbs = l2_read_gbs()
    cpu_val, cpu_cores, cpu_s = cpu_baseline(w, t, args.cpu_samples)
    line = {
        "metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": desc, "paths_per_step_per_gpu": B.paths, "poses": P, "max_bounces": w.max_depth,
                   "range_bins": N, "phase": "reference-fp32", "splat": "dirichlet16",
                   "l2": "flushed between steps (512 MiB write)", "parallelism": "replicas x%d" % world,
                   "launch_config": {k: tuned[k] for k in ("tile", "ctas_per_sm", "queue_threshold")},
                   "autotune_trace_ms": [tuned["default_trace_ms"], tuned["trace_ms"]]},
        "e2e": {"value": world * B.paths / (e2e_ms / 1000.0), "unit": "paths/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms},
        "roofline": {"bound": "l2", "achieved": achieved, "peak": l2_gbs, "unit": "GB/s",
                     "frac": achieved / l2_gbs,
                     "traffic": args.traffic if args.traffic is not None else NCU_TRAFFIC.get(args.workload),
                     "kernel": "k_wave",
                     "kernel_ms": trace_ms, "algorithmic_bytes": alg_bytes, "rays": counts["rays"] * scale,
                     "nodes": counts["nodes"] * scale, "tris": counts["tris"] * scale,
                     "peak_source": "L2 read bandwidth measured live (hsr_measure_l2_read, 32 MiB x 64 sweeps)",
                     "hbm_peak": peak, "hbm_peak_source": peak_kind, "frac_of_hbm": achieved / peak},
        "cpu_baseline": {"value": cpu_val, "unit": "paths/s", "cores": cpu_cores, "kind": "port",
                         "sample": "%d Halton samples of pose 0 (%.1f s wall)" % (args.cpu_samples, cpu_s)},
        "modes": modes,
        "time_to_minus40db": time_to_error() if not args.no_tte else None,
        "batch_graph": graph_overhead(torch, dev),
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def run_batched(args, rank, world, local_rank, dist):
    """The batched configuration (module docstring): 4096 poses resident on the device,
    one step = one 256-pose batch through a captured graph of the batched form."""
    import ctypes

    import torch

    from hussar_gb300 import HSR_PHASE_SPLIT_FP64, HSR_SPLAT_FINE_SYNTH, PathTracer, _lib, gb300

    torch.cuda.set_device(local_rank)
    L = _lib.lib()
    w, desc = load_workload("boxes", args.poses)
    if args.max_log2:  # profiling cases: budgets capped (say so in the line's config)
        w.budget = np.minimum(w.budget, 1 << args.max_log2)
        desc += ", budgets capped at 2^%d" % args.max_log2
    t = PathTracer()
    t.doGuiding = False
    t.maxDepth = w.max_depth
    be = gb300.Backend(w.mesh, None)
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.current_stream(dev)
    B = DeviceBatch(w, dev, rank, torch, _lib)  # every pose resident
    N, Q = B.N, min(BOXES_BATCH, B.P)
    nb = B.P // Q
    ant = ctypes.sizeof(_lib.AntennaC)
    # the graph's input slots (one batch) and its output rows
    s_tx = torch.empty(Q * ant, dtype=torch.uint8, device=dev)
    s_rx = torch.empty(Q * ant, dtype=torch.uint8, device=dev)
    s_budget = torch.empty(Q, dtype=torch.int64, device=dev)
    s_offset = torch.empty(Q, dtype=torch.int64, device=dev)
    s_rows = torch.zeros(2 * Q * N, dtype=torch.float32, device=dev)
    batch_paths = [int(w.budget[k * Q:(k + 1) * Q].sum()) for k in range(nb)]
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    vp = ctypes.c_void_p
    rf_c, fl_c = w.rf.to_c(), t.flags_c()
    phase, splat = HSR_PHASE_SPLIT_FP64, HSR_SPLAT_FINE_SYNTH

    # the product's autotuner picks the launch shape on a bounded sample of the batch (16
    # poses, budgets capped at 2^20); the graph below is captured with it
    if args.launch_config:  # a fixed shape (profiling runs reproduce the tuned one without tuning)
        vals = [int(x) for x in args.launch_config.split(",")] + [0]
        tile, ctas, thr, foh, coh = vals[:5]
        be.set_launch_config(tile, ctas, thr, foh, coh)
        tuned = dict(tile=tile, ctas_per_sm=ctas, queue_threshold=thr, field_on_hit=foh, coherent_order=coh,
                     trace_ms=None, default_trace_ms=None)
    else:
        tuned = be.autotune(w.rf, N, t, w.tx[:16], w.rx[:16], np.minimum(w.budget[:16], 1 << 20), phase_mode=phase,
                            splat_mode=splat)
    g = be.batch_graph(w.rf, N, t, Q, s_tx.data_ptr(), s_rx.data_ptr(), s_budget.data_ptr(), s_offset.data_ptr(),
                       s_rows.data_ptr(), phase_mode=phase, splat_mode=splat)

    def load_slot(k):
        b = (k % nb) * Q
        s_tx.copy_(B.d_tx[b * ant:(b + Q) * ant], non_blocking=True)
        s_rx.copy_(B.d_rx[b * ant:(b + Q) * ant], non_blocking=True)
        s_budget.copy_(B.d_budget[b:b + Q], non_blocking=True)
        s_offset.copy_(B.d_offset[b:b + Q], non_blocking=True)

    def step(k):
        load_slot(k)
        g.launch(stream.cuda_stream)

    for k in range(max(args.warmup, 3)):
        step(k)
    g.status()

    clocks = ClockSampler(local_rank)
    barrier(dist)
    torch.cuda.synchronize()
    clocks.start()
    launches0 = L.hsr_launch_count()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for k in range(args.steps):
        flush.fill_(k & 0xff)  # > L2 (129 MB), outside the timed events
        ev[k][0].record(stream)
        step(k)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    launches = L.hsr_launch_count() - launches0
    barrier(dist)
    clk = clocks.stop()
    g.status()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    timed_paths = sum(batch_paths[k % nb] for k in range(args.steps))
    total_ms = max_over_ranks(dist, sum(step_ms))
    ms = total_ms / args.steps
    value = world * timed_paths / (total_ms / 1000.0)

    if args.kernel_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world,
                              "steps": args.steps, "ms_per_step": ms, "kernel_only": True, "workload": desc,
                              "gpu_launches": int(launches), "clocks": clk}), flush=True)
        g.close()
        return

    # e2e through the public host-buffer API, the same batches and form: pinned poses in,
    # normalised rows out, synchronous
    h_tx = [(_lib.AntennaC * Q)(*[a.to_c() for a in w.tx[k * Q:(k + 1) * Q]]) for k in range(nb)]
    h_rx = [(_lib.AntennaC * Q)(*[a.to_c() for a in w.rx[k * Q:(k + 1) * Q]]) for k in range(nb)]
    h_rows = torch.zeros(2 * Q * N, dtype=torch.float32).pin_memory()

    def e2e_step(k):
        b = (k % nb) * Q
        _lib.check(L.hsr_simulate_batch(
            be.handle, ctypes.byref(rf_c), N, ctypes.byref(fl_c), Q, ctypes.cast(h_tx[k % nb], vp),
            ctypes.cast(h_rx[k % nb], vp), vp(B.h_budget[b:].data_ptr()), vp(B.h_offset[b:].data_ptr()), phase, splat,
            vp(h_rows.data_ptr()), vp(stream.cuda_stream)))

    e2e_step(0)
    e2e_times = []
    for k in range(args.steps):
        flush.fill_(k & 0xff)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step(k)
        e2e_times.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(dist, sum(e2e_times))
    h2d = (2 * ant + 16) * Q
    d2h = 8 * N * Q

    # the traversal kernel alone (events around it inside the library) on batch 0, direct call
    kms = ctypes.c_float()

    def direct(k, ph, sp_):
        b = (k % nb) * Q
        _lib.check(L.hsr_simulate_batch_device(
            be.handle, ctypes.byref(rf_c), N, ctypes.byref(fl_c), Q, vp(B.d_tx[b * ant:].data_ptr()),
            vp(B.d_rx[b * ant:].data_ptr()), vp(B.d_budget[b:].data_ptr()), vp(B.d_offset[b:].data_ptr()), ph, sp_,
            vp(B.d_rows.data_ptr()), vp(stream.cuda_stream)))

    flush.fill_(1)
    direct(0, phase, splat)
    flush.fill_(2)
    d0, d1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    d0.record(stream)
    direct(0, phase, splat)
    d1.record(stream)
    _lib.check(L.hsr_scene_status(be.handle, vp(stream.cuda_stream), None))
    _lib.check(L.hsr_last_kernel_ms(be.handle, ctypes.byref(kms)))
    trace_ms = kms.value
    torch.cuda.synchronize()
    direct_ms = d0.elapsed_time(d1)

    # the plain form on the same batches (reference FP32 phase, the reference's 33-bin
    # splat, direct calls): the parity form, for comparison
    modes = {}
    pl_ms = []
    for k in range(max(2, args.steps // 4)):
        flush.fill_(k & 0xff)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        direct(k, _lib.HSR_PHASE_REFERENCE_FP32, _lib.HSR_SPLAT_DIRICHLET16)
        e1.record(stream)
        torch.cuda.synchronize()
        pl_ms.append((batch_paths[k % nb], e0.elapsed_time(e1)))
    modes["plain_reference_fp32_splat16"] = {
        "value": world * sum(p for p, _ in pl_ms) / (max_over_ranks(dist, sum(m for _, m in pl_ms)) / 1000.0),
        "unit": "paths/s", "steps": len(pl_ms), "note": "direct calls, reference FP32 phase, Frame::splat<16>"}
    # the synthesis of batch 0: the direct call's time minus its traversal kernel's time
    synth_ms = direct_ms - trace_ms
    useful = 8.0 * Q * (32 * N) * N  # complex [Q x 32N] x [32N x N] in real flops
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    modes["synthesis_in_step"] = {"ms": synth_ms, "useful_tflop": useful / 1e12,
                                  "note": "one direct call on batch 0 minus its trace kernel (prefix, memsets, GEMM, "
                                          "rows); the GEMM's own roofline is bench.py --workload synth"}
    g.close()
    if rank != 0:
        return
    # exact traversal work of batch 0 (counting instantiation over every 4th pose, scaled by paths)
    sub = np.arange(0, Q, 4)
    counts = be.traversal_counts(w.rf, N, t, [w.tx[i] for i in sub], [w.rx[i] for i in sub], w.budget[sub])
    scale = batch_paths[0] / float(w.budget[sub].sum())
    alg_bytes = counts["bytes"] * scale
    hbm, peak_kind = measured_peaks()
    l2 = l2_read_gbs()
    achieved = alg_bytes / (trace_ms / 1000.0) / 1e9
    cpu_val, cpu_cores, cpu_s, cpu_what = cpu_baseline_boxes(w, t)
    line = {
        "metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": desc, "batch": "%d of the %d poses per step; step k traces batch k mod %d" % (Q, B.P, nb),
                   "paths_per_step_per_gpu": timed_paths / args.steps, "poses": B.P, "max_bounces": w.max_depth,
                   "range_bins": N, "phase": "split-fp64", "splat": "fine histogram + split-BF16 tcgen05 synthesis",
                   "launch": "captured CUDA graph (hsr_batch_graph_*), one persistent trace launch per step",
                   "l2": "flushed between steps (512 MiB write)", "parallelism": "replicas x%d" % world,
                   "launch_config": {k: tuned[k] for k in ("tile", "ctas_per_sm", "queue_threshold", "field_on_hit",
                                                           "coherent_order")},
                   "autotune_trace_ms": [tuned["default_trace_ms"], tuned["trace_ms"]]},
        "e2e": {"value": world * timed_paths / e2e_s, "unit": "paths/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": 1000.0 * e2e_s / args.steps,
                "call": "hsr_simulate_batch (host buffers, synchronous), split-FP64 phase, fine synthesis"},
        "roofline": {"bound": "l2", "achieved": achieved, "peak": l2, "unit": "GB/s", "frac": achieved / l2,
                     "traffic": args.traffic if args.traffic is not None else NCU_TRAFFIC.get("boxes"),
                     "kernel": "k_wave", "kernel_ms": trace_ms, "algorithmic_bytes": alg_bytes,
                     "rays": counts["rays"] * scale, "nodes": counts["nodes"] * scale, "tris": counts["tris"] * scale,
                     "peak_source": "L2 read bandwidth measured live (hsr_measure_l2_read, 32 MiB x 64 sweeps)",
                     "hbm_peak": hbm, "hbm_peak_source": peak_kind, "frac_of_hbm": achieved / hbm},
        "cpu_baseline": {"value": cpu_val, "unit": "paths/s", "cores": cpu_cores, "kind": "port",
                         "sample": "%s (%.1f s wall)" % (cpu_what, cpu_s)},
        "modes": modes,
        "time_to_minus40db": time_to_error(with_boxes=True) if not args.no_tte else None,
        "batch_graph": graph_overhead(torch, dev),
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def cpu_baseline_boxes(w, tracer):
    """The oracle's FP32 restatement on all host cores over a bounded sample of the batched
    configuration: the first REF_POSES poses at 2^REF_LOG2 samples each."""
    from oracle import pyoracle
    ora = pyoracle.Scene(w.mesh)
    t0 = time.perf_counter()
    for i in range(REF_POSES):
        ora.simulate(w.rf, w.frame, w.tx[i], w.rx[i], tracer, 1 << REF_LOG2, precision=32)
    dt = time.perf_counter() - t0
    return REF_POSES * (1 << REF_LOG2) / dt, os.cpu_count(), dt, \
        "the first %d poses at 2^%d Halton samples each" % (REF_POSES, REF_LOG2)


def graph_overhead(torch, dev, reps=50):
    """Per-batch device time of a small batch (the dihedral sweep, 91 poses x 2^12
    samples) through hsr_simulate_batch_device and through its captured CUDA graph
    (hsr_batch_graph_launch), CUDA events over `reps` back-to-back calls."""
    import ctypes

    from hussar_gb300 import PathTracer, _lib, gb300, scenes
    L = _lib.lib()
    w = scenes.dihedral_workload()
    t = PathTracer()
    t.doGuiding = False
    t.maxDepth = w.max_depth
    be = gb300.Backend(w.mesh, None)
    P, N = len(w.tx), w.frame.samplesPerChirp
    tx = (_lib.AntennaC * P)(*[a.to_c() for a in w.tx])
    rx = (_lib.AntennaC * P)(*[a.to_c() for a in w.rx])
    d_tx = torch.frombuffer(bytearray(bytes(tx)), dtype=torch.uint8).to(dev)
    d_rx = torch.frombuffer(bytearray(bytes(rx)), dtype=torch.uint8).to(dev)
    d_b = torch.full((P,), 1 << 12, dtype=torch.int64, device=dev)
    d_o = torch.zeros(P, dtype=torch.int64, device=dev)
    d_out = torch.zeros(2 * P * N, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    vp = ctypes.c_void_p
    rf_c, fl_c = w.rf.to_c(), t.flags_c()

    def direct():
        _lib.check(L.hsr_simulate_batch_device(be.handle, ctypes.byref(rf_c), N, ctypes.byref(fl_c), P,
                                               vp(d_tx.data_ptr()), vp(d_rx.data_ptr()), vp(d_b.data_ptr()),
                                               vp(d_o.data_ptr()), _lib.HSR_PHASE_REFERENCE_FP32,
                                               _lib.HSR_SPLAT_DIRICHLET16, vp(d_out.data_ptr()),
                                               vp(stream.cuda_stream)))

    g = be.batch_graph(w.rf, N, t, P, d_tx.data_ptr(), d_rx.data_ptr(), d_b.data_ptr(), d_o.data_ptr(),
                       d_out.data_ptr())
    out = {"workload": "dihedral, 91 poses x 2^12 samples", "reps": reps}
    for name, fn in (("direct_us", direct), ("graph_us", lambda: g.launch(stream.cuda_stream))):
        for _ in range(5):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        out[name] = 1000.0 * e0.elapsed_time(e1) / reps
    g.status()
    g.close()
    return out


TTE_TARGET = 1e-2  # -40 dB: relative L2 of the complex IF signal
# The converged reference of each scene (split-FP64 phase), per splat kernel: (guided,
# log2 samples per pose), and the largest budget measured. References trace Halton
# indices from TTE_REF_OFFSET, a set disjoint from the forms' (which start at 0), so their
# error is independent of the forms'. On the sphere the plain estimator is heavy-tailed
# (error ~ budget^-0.49 with rare grazing next-event spikes; still 10 % off at 2^32), so
# the reference there is the guided estimator (unbiased, same integrand) at 2^33: two
# independent 2^32 guided runs agree to 0.3-0.6 %.
TTE_SCENES = {"sphere_ground": (True, 33, 31), "dihedral_91": (False, 28, 26), "boxes_16": (False, 26, 23),
              "urban_mimo_12": (False, 25, 22)}
TTE_BOXES_POSES = 16  # the batched configuration's first 16 poses
TTE_ANCHOR = 1 << 16  # budget of the FP64-oracle anchor of each scene's converged reference
TTE_REF_OFFSET = 1_000_000_000_007


def fp64_anchor(w, be, tracer, poses):
    """How far the GPU's split-FP64 form is from the FP64 oracle on the SAME samples: the
    oracle in double precision fed the float Halton values of the FP32 run (precision 65),
    against the GPU's split-FP64 rows, TTE_ANCHOR Halton indices from 0, on `poses`.
    This is the part of a converged split-FP64 reference's distance to the FP64 oracle
    that does not shrink with more samples (the FP32 geometry), so each scene's
    time-to-error reference stands for the FP64 oracle to within it."""
    from hussar_gb300 import HSR_PHASE_SPLIT_FP64
    from oracle import pyoracle
    ora = pyoracle.Scene(w.mesh)
    N = w.frame.samplesPerChirp
    budget = np.full(len(poses), TTE_ANCHOR, np.int64)
    rows = be.simulate_batch(w.rf, N, tracer, [w.tx[i] for i in poses], [w.rx[i] for i in poses], budget,
                             phase_mode=HSR_PHASE_SPLIT_FP64).astype(np.complex128)
    ref = np.stack([ora.fetch_row(w.rf, N, w.tx[i], w.rx[i], tracer, TTE_ANCHOR, precision=65) for i in poses])
    return {"poses": [int(i) for i in poses], "samples_per_pose": TTE_ANCHOR,
            "rel_l2_split_fp64_vs_fp64_oracle": float(np.linalg.norm(rows - ref) / np.linalg.norm(ref))}


def time_to_error(with_boxes=False):
    """Time to -40 dB IF-signal error against the plain GPU form, on the sphere+ground pose,
    the 91-pose dihedral sweep and (with_boxes) the first 16 poses of the batched boxes
    configuration and the 12 channels of the urban MIMO array. Each form's rows at budget 2^k (Halton indices 0 .. 2^k-1, k = 10, 11,
    ...) are compared with a converged run of the same estimator (split-FP64 phase, Halton
    indices from TTE_REF_OFFSET: guided at 2^33 samples per pose for the sphere, plain at
    2^28 for the dihedral, 2^26 for the boxes and 2^25 for the urban channels; relative L2
    over all poses' rows), whose
    own distance to the FP64 oracle on identical samples is reported (fp64_anchor); the
    smallest such budget reaching 1e-2 is then timed through the host API (wall clock,
    synchronous calls, median of 3).
      plain_gpu            one pose per call, one-thread-per-sample kernel, FP32 phase of
                           the reference, Frame::splat<16> (the OptiX backend's form)
      batched_split        all poses in one wavefront launch, split-FP64 phase, splat<16>
      batched_split_synth  the same with the fine histogram and tensor-core synthesis of
                           the exact spectrum (its own estimator and reference)
      batched_split_guided[_synth]  the same with device path guiding (PathTracer::run's
                           doubling schedule; unbiased, the same reference)
      served_split         every pose a request to the serving loop (hsr_server_*, split-FP64
                           phase), all submitted at once and timed until the last row is on
                           the host; a served row is the batched split row up to summation
                           order (the same Halton samples), so it is timed at the budget the
                           batched split form needs, and its error there is reported
      served_split_guided  the same with guided requests (each runs the doubling schedule
                           across the server's ticks), from the batched guided form's budget,
                           doubled until its own rows reach the target
    A form that does not reach the target by the scene's largest budget (2^31 sphere,
    2^26 dihedral, 2^23 boxes, 2^22 urban) reports the budget extrapolated
    from the slope of its last six points (log error vs log budget) and the time for it
    at its measured throughput, marked "extrapolated"."""
    from hussar_gb300 import (HSR_PHASE_REFERENCE_FP32, HSR_PHASE_SPLIT_FP64, HSR_SPLAT_DIRICHLET16,
                              HSR_SPLAT_FINE_SYNTH, PathTracer, Server, _lib, gb300, scenes)
    L = _lib.lib()
    out = {"target_rel_l2": TTE_TARGET,
           "reference": "split-FP64 phase, same splat kernel, Halton indices from %d (disjoint from the forms'); "
                        "sphere: guided 2^%d samples per pose, dihedral: plain 2^%d, boxes: plain 2^%d, "
                        "urban: plain 2^%d" % (TTE_REF_OFFSET, TTE_SCENES["sphere_ground"][1],
                                               TTE_SCENES["dihedral_91"][1], TTE_SCENES["boxes_16"][1],
                                               TTE_SCENES["urban_mimo_12"][1]),
           "timing": "wall clock through hsr_simulate_batch, median of 3"}
    forms = {"plain_gpu": (1, HSR_PHASE_REFERENCE_FP32, HSR_SPLAT_DIRICHLET16, True, False),
             "batched_split": (0, HSR_PHASE_SPLIT_FP64, HSR_SPLAT_DIRICHLET16, False, False),
             "batched_split_synth": (0, HSR_PHASE_SPLIT_FP64, HSR_SPLAT_FINE_SYNTH, False, False),
             "batched_split_guided": (0, HSR_PHASE_SPLIT_FP64, HSR_SPLAT_DIRICHLET16, False, True),
             "batched_split_synth_guided": (0, HSR_PHASE_SPLIT_FP64, HSR_SPLAT_FINE_SYNTH, False, True)}
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    todo = [("sphere_ground", scenes.sphere_ground_workload()), ("dihedral_91", scenes.dihedral_workload())]
    if with_boxes:
        wb = scenes.boxes_workload()
        wb.tx, wb.rx, wb.budget = wb.tx[:TTE_BOXES_POSES], wb.rx[:TTE_BOXES_POSES], wb.budget[:TTE_BOXES_POSES]
        todo.append(("boxes_16", wb))
        # the urban MIMO array's 12 virtual channels (5 M triangles, 5 bounces)
        todo.append(("urban_mimo_12", scenes.urban_mimo_workload(samples=1 << 16)))
    for name, w in todo:
        ref_guided, ref_log2, max_log2 = TTE_SCENES[name]
        plain_t, guided_t = PathTracer(), PathTracer()
        plain_t.doGuiding = False
        guided_t.doGuiding = True
        plain_t.maxDepth = guided_t.maxDepth = w.max_depth
        be = gb300.Backend(w.mesh, None)
        N, P = w.frame.samplesPerChirp, len(w.tx)

        def run(form, S, offset=0):
            kernel, phase, splat, per_pose, guided = form
            t = guided_t if guided else plain_t
            L.hsr_set_path_kernel(kernel)
            try:
                if per_pose:
                    return np.concatenate([be.simulate_batch(w.rf, N, t, [w.tx[k]], [w.rx[k]], [S], [offset],
                                                             phase_mode=phase, splat_mode=splat) for k in range(P)])
                return be.simulate_batch(w.rf, N, t, w.tx, w.rx, np.full(P, S, np.int64), np.full(P, offset, np.int64),
                                         phase_mode=phase, splat_mode=splat)
            finally:
                L.hsr_set_path_kernel(0)

        refs = {s: run((0, HSR_PHASE_SPLIT_FP64, s, False, ref_guided), 1 << ref_log2,
                       TTE_REF_OFFSET).astype(np.complex128) for s in (HSR_SPLAT_DIRICHLET16, HSR_SPLAT_FINE_SYNTH)}
        res = {}
        be.set_launch_config(default=True)  # the plain GPU form runs with the default launch shape
        for fname, form in forms.items():
            if fname == "batched_split":
                # the batched forms use the product's autotuned shape (tuned on 2^20 samples per pose)
                res["launch_config"] = be.autotune(w.rf, N, plain_t, w.tx, w.rx, np.full(P, 1 << 20, np.int64),
                                                   phase_mode=HSR_PHASE_SPLIT_FP64)
            ref = refs[form[2]]
            curve, s40 = [], None
            for k in range(10, max_log2 + 1):
                rows = run(form, 1 << k).astype(np.complex128)
                err = float(np.linalg.norm(rows - ref) / np.linalg.norm(ref))
                curve.append([k, err])
                if err <= TTE_TARGET:
                    s40 = 1 << k
                    break
            entry = {"error_by_log2_budget": curve, "samples_per_pose": s40}
            timed_s = s40 or (1 << max_log2)
            run(form, timed_s)  # warm-up at this size
            times = []
            for _ in range(3):
                t0 = time.perf_counter()
                run(form, timed_s)
                times.append(time.perf_counter() - t0)
            sec = float(np.median(times))
            if s40:
                entry["seconds"] = sec
            else:
                k, e = np.array(curve[-6:]).T
                slope = float(np.polyfit(k, np.log2(e), 1)[0])  # log2 error per doubling
                if slope < -0.05:
                    extra = np.log2(e[-1] / TTE_TARGET) / -slope
                    entry["extrapolated"] = {"slope_per_doubling": slope, "samples_per_pose": timed_s * 2.0 ** extra,
                                             "seconds": sec * 2.0 ** extra}
            res[fname] = entry

        # the served form, at the budget the batched split form reaches the target with
        bs = res["batched_split"]
        s_budget = bs["samples_per_pose"] or (1 << max_log2)
        srv = Server(flags=plain_t, phase_mode=HSR_PHASE_SPLIT_FP64, max_slots=max(P, 1), max_samples_per_chirp=N)
        try:
            sid = srv.add_scene(be)

            def serve_all():
                reqs = [srv.submit(sid, w.rf, N, w.tx[k], w.rx[k], s_budget) for k in range(P)]
                return np.stack([r.result()[0] for r in reqs]).astype(np.complex128)

            rows = serve_all()
            ref = refs[HSR_SPLAT_DIRICHLET16]
            entry = {"samples_per_pose": bs["samples_per_pose"], "budget_timed": s_budget,
                     "error_at_budget": float(np.linalg.norm(rows - ref) / np.linalg.norm(ref))}
            # timed alternately with the batched split call at the same budget, so that both
            # see the same clock state
            times, batch_times = [], []
            for _ in range(3):
                t0 = time.perf_counter()
                serve_all()
                times.append(time.perf_counter() - t0)
                t0 = time.perf_counter()
                run(forms["batched_split"], s_budget)
                batch_times.append(time.perf_counter() - t0)
            sec = float(np.median(times))
            entry["batched_split_seconds_same_budget"] = float(np.median(batch_times))
            if bs["samples_per_pose"]:
                entry["seconds"] = sec
            elif bs.get("extrapolated"):
                scale = bs["extrapolated"]["samples_per_pose"] / s_budget
                entry["extrapolated"] = {"samples_per_pose": bs["extrapolated"]["samples_per_pose"],
                                         "seconds": sec * scale}
            entry["server"] = {k: v for k, v in srv.stats().items() if k in ("ticks", "max_batch", "device_ms")}
            res["served_split"] = entry
        finally:
            srv.close()

        # the served guided form: every pose a guided request (the doubling schedule runs
        # across the server's ticks). Its trees train on float sums in another order than
        # the batched guided form's, so its error at a budget differs: it starts at the
        # budget the batched guided form needs and doubles (at most twice) until it
        # reaches the target itself
        bg = res["batched_split_guided"]
        g_budget = bg["samples_per_pose"] or (1 << max_log2)
        srv = Server(flags=guided_t, phase_mode=HSR_PHASE_SPLIT_FP64, max_slots=max(P, 1), max_samples_per_chirp=N)
        try:
            sid = srv.add_scene(be)

            def serve_guided(budget):
                reqs = [srv.submit(sid, w.rf, N, w.tx[k], w.rx[k], budget) for k in range(P)]
                return np.stack([r.result()[0] for r in reqs]).astype(np.complex128)

            ref = refs[HSR_SPLAT_DIRICHLET16]
            curve, s40, budget = [], None, g_budget
            for _ in range(3 if bg["samples_per_pose"] else 1):
                rows = serve_guided(budget)
                err = float(np.linalg.norm(rows - ref) / np.linalg.norm(ref))
                curve.append([int(np.log2(budget)), err])
                if err <= TTE_TARGET:
                    s40 = budget
                    break
                budget *= 2
            entry = {"error_by_log2_budget": curve, "samples_per_pose": s40,
                     "budget_timed": s40 or g_budget}
            times = []
            for _ in range(3):
                t0 = time.perf_counter()
                serve_guided(s40 or g_budget)
                times.append(time.perf_counter() - t0)
            if s40:
                entry["seconds"] = float(np.median(times))
            entry["server"] = {k: v for k, v in srv.stats().items() if k in ("ticks", "max_batch", "device_ms")}
            res["served_split_guided"] = entry
        finally:
            srv.close()

        def seconds(e):
            return e.get("seconds") or (e.get("extrapolated") or {}).get("seconds")

        plain = seconds(res["plain_gpu"])
        for fname in list(forms) + ["served_split", "served_split_guided"]:
            if fname != "plain_gpu" and fname in res:
                sec = seconds(res[fname])
                res[fname]["speedup_vs_plain_gpu"] = (plain / sec) if (plain and sec) else None
        anchor_poses = list(range(0, P, max(1, P // 4)))[:4]
        out[name] = dict(res, poses=P, range_bins=N, triangles=w.mesh.triangleCount(), reference_log2=ref_log2,
                         reference_guided=ref_guided, fp64_anchor=fp64_anchor(w, be, plain_t, anchor_poses))
    out["clocks"] = clocks.stop()  # over the whole measurement
    return out


def run_urban_mimo(args, rank, world, local_rank, dist):
    """The guided urban MIMO configuration (scenes.urban_mimo_workload): the 3 TX x 4 RX
    array's 12 virtual channels traced as one guided batch (PathTracer::run's doubling
    schedule, 2^22 samples per channel: 8 iterations), split-FP64 phase, up to 5 bounces,
    each step one hsr_simulate_frame call returning the 128 x 256 x 12 radar cube
    [chirp][sample][channel] to the host. Replicas under torchrun."""
    import torch

    from hussar_gb300 import HSR_PHASE_SPLIT_FP64, PathTracer, _lib, gb300, scenes

    torch.cuda.set_device(local_rank)
    L = _lib.lib()
    w = scenes.urban_mimo_workload()
    be = gb300.Backend(w.mesh, None)
    P, N, C = len(w.tx), w.frame.samplesPerChirp, w.frame.chirpCount
    budget = int(w.budget[0])
    off = replica_range(rank, budget)[0]
    res = {}
    for name, guided in (("guided", True), ("plain", False)):
        t = PathTracer()
        t.doGuiding = guided
        t.maxDepth = w.max_depth

        def step():
            return be.simulate_frame(w.rf, w.frame, t, w.tx_array, w.rx_array, budget, index_offset=off,
                                     phase_mode=HSR_PHASE_SPLIT_FP64)

        for _ in range(max(args.warmup, 3) if guided else 1):
            step()
        barrier(dist)
        times = []
        n0 = L.hsr_launch_count()
        steps = args.steps if guided else 2
        for _ in range(steps):
            t0 = time.perf_counter()
            frame = step()
            times.append(time.perf_counter() - t0)
        ms = max_over_ranks(dist, 1000.0 * float(np.median(times)))
        res[name] = {"ms_per_step": ms, "paths_per_s": world * float(w.budget.sum()) / (ms / 1000.0),
                     "library_launches_per_step": (L.hsr_launch_count() - n0) / steps}
    if rank != 0:
        return
    g = res["guided"]
    line = {
        "metric": METRIC, "value": g["paths_per_s"], "unit": "paths/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": g["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "urban canyon %d triangles, 3 TX x 4 RX at lambda/2 (12 channels), %d chirps x %d "
                               "samples, guided (8 doubling iterations, 2^22 samples per channel), 5 bounces, "
                               "split FP64 phase" % (w.mesh.triangleCount(), C, N),
                   "frame_shape": [C, N, P], "l2": "inputs larger than L2 (%.0f MB scene)" % (be.footprint() / 1e6)},
        "e2e": {"value": g["paths_per_s"], "unit": "paths/s",
                "h2d_bytes_per_step": int((len(w.tx_array) + len(w.rx_array)) * 48 + P * 16),
                "d2h_bytes_per_step": int(C * N * P * 8),
                "note": "wall clock through hsr_simulate_frame (host radar cube out, synchronous)"},
        "modes": {"plain_same_budget": res["plain"]},
        "gpu_launches": int(round(g["library_launches_per_step"] * args.steps)),
    }
    print(json.dumps(line), flush=True)


def run_synth(args, rank, world, local_rank, dist):
    """The synthesis GEMM at batch scale: the 91 dihedral poses repeated to --poses (2048
    by default), 2^12 samples each, N = 256, HSR_SPLAT_FINE_SYNTH through
    hsr_simulate_batch_device; the step time minus the trace kernel's time is the
    synthesis (histogram clear, tcgen05 GEMM forming the BF16 terms of the histogram in
    its producer warps, rows). Replicas under torchrun."""
    import ctypes

    import torch

    from hussar_gb300 import PathTracer, _lib, gb300, scenes

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    L = _lib.lib()
    P = args.poses or 2048
    w = scenes.dihedral_workload()
    idx = np.arange(P) % len(w.tx)
    w.tx, w.rx = [w.tx[i] for i in idx], [w.rx[i] for i in idx]
    w.budget = np.full(P, 1 << 12, np.int64)
    t = PathTracer()
    t.doGuiding = False
    t.maxDepth = w.max_depth
    be = gb300.Backend(w.mesh, None)
    B = DeviceBatch(w, dev, rank, torch, _lib)
    N = B.N
    stream = torch.cuda.current_stream(dev)
    rf_c, fl_c = w.rf.to_c(), t.flags_c()
    vp = ctypes.c_void_p
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)

    def step(splat):
        _lib.check(L.hsr_simulate_batch_device(
            be.handle, ctypes.byref(rf_c), N, ctypes.byref(fl_c), P, vp(B.d_tx.data_ptr()), vp(B.d_rx.data_ptr()),
            vp(B.d_budget.data_ptr()), vp(B.d_offset.data_ptr()), _lib.HSR_PHASE_REFERENCE_FP32, splat,
            vp(B.d_rows.data_ptr()), vp(stream.cuda_stream)))

    res = {}
    for name, splat in (("fine_synth", _lib.HSR_SPLAT_FINE_SYNTH), ("dirichlet16", _lib.HSR_SPLAT_DIRICHLET16)):
        for _ in range(max(args.warmup, 3)):
            step(splat)
        ms, trace = [], []
        for k in range(args.steps):
            flush.fill_(k & 0xff)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step(splat)
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
            kms = ctypes.c_float()
            _lib.check(L.hsr_last_kernel_ms(be.handle, ctypes.byref(kms)))
            trace.append(kms.value)
        res[name] = {"ms_per_step": max_over_ranks(dist, float(np.median(ms))), "trace_ms": float(np.median(trace))}
    if rank != 0:
        return
    f = res["fine_synth"]
    synth_ms = max(f["ms_per_step"] - f["trace_ms"], 1e-6)
    useful = 8.0 * P * (32 * N) * N  # complex [P x 32N] x [32N x N] in real flops
    executed = 6 * 2.0 * P * (64 * N) * (2 * N)  # six BF16 products of the real [P x 64N] x [64N x 2N]
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    tc = peaks.get("bf16_tflops", 1900.0)
    line = {
        "metric": METRIC, "value": world * float(B.paths) / (f["ms_per_step"] / 1000.0), "unit": "paths/s",
        "n_gpus": world, "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": f["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "dihedral poses repeated to %d, 2^12 samples each, N=%d, fine-histogram synthesis"
                               % (P, N), "l2": "flushed between steps (512 MiB write)"},
        "roofline": {"bound": "tensor",
                     "kernel": "synthesis (histogram clear, k_umma_gemm with the BF16 split of the histogram fused "
                               "into its producer, k_synth_finalize)",
                     "achieved": useful / (synth_ms / 1000.0) / 1e12, "peak": tc, "unit": "TFLOP/s",
                     "frac": useful / (synth_ms / 1000.0) / 1e12 / tc, "traffic": None,
                     "executed_bf16_tflops": executed / (synth_ms / 1000.0) / 1e12, "synthesis_ms": synth_ms,
                     "note": "useful = the complex product's flops; the six BF16 split products execute 6x "
                             "the real product"},
        "modes": res,
        "e2e": None,
        "gpu_launches": None,
    }
    print(json.dumps(line), flush=True)


def run_serve(args, rank, world, local_rank, dist):
    """The serving workload (see the module docstring); replicas under torchrun: every rank
    serves its own request stream."""
    import torch

    from hussar_gb300 import HSR_PHASE_SPLIT_FP64, PathTracer, Server, gb300, scenes

    torch.cuda.set_device(local_rank)
    t = PathTracer()
    t.doGuiding = bool(args.guided)
    t.maxDepth = 4
    t0 = time.perf_counter()
    backends, posegens, tris = [], [], 0
    for i, (kind, n) in enumerate(scenes.SERVE_SCENES):
        mesh, pg = scenes.serve_scene(kind, n, 0xC5 + i)
        tris += mesh.triangleCount()
        backends.append(gb300.Backend(mesh, None))
        posegens.append(pg)
        del mesh
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    rng = np.random.default_rng(0xC5 + 101 * rank)
    n_req = max(1, int(round(args.rate * args.duration)))
    arrivals = np.cumsum(rng.exponential(1.0 / args.rate, n_req))
    sid = rng.integers(0, len(backends), n_req)
    budget = np.round(2.0 ** rng.uniform(16, 24, n_req)).astype(np.int64)
    bw = rng.uniform(1e9, 4e9, n_req)
    nbins = rng.choice([128, 256, 512], n_req)
    poses = [posegens[int(s)](1, 1000 + k)[0] for k, s in enumerate(sid)]
    srv = Server(flags=t, phase_mode=HSR_PHASE_SPLIT_FP64, max_slots=args.slots, max_samples_per_chirp=512,
                 tick_ms=args.tick_ms)
    ids = [srv.add_scene(be) for be in backends]

    def submit(k, offset=0, scale=1):
        rf = scenes.rf_chirp(bandwidth=float(bw[k]), samples=int(nbins[k]))
        return srv.submit(ids[int(sid[k])], rf, int(nbins[k]), poses[k], poses[k], max(1, int(budget[k]) // scale),
                          offset)

    # warm-up: every scene once at a small budget (kernel attributes, allocator, clocks)
    warm = [submit(int(np.nonzero(sid == s)[0][0]) if (sid == s).any() else 0, 1 << 30, 64)
            for s in range(len(backends))]
    for _ in range(max(args.warmup, 3) - 1):
        warm += [submit(k, 1 << 31, 64) for k in range(min(4, n_req))]
    for h in warm:
        h.result()
    srv.reset_stats()
    clocks = ClockSampler(local_rank)
    barrier(dist)
    clocks.start()
    start = time.perf_counter()
    handles = []
    for k in range(n_req):
        delay = start + arrivals[k] - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        handles.append(submit(k))
    infos = [h.result()[1] for h in handles]
    wall = time.perf_counter() - start
    barrier(dist)
    clk = clocks.stop()
    st = srv.stats()
    srv.close()
    # the error the served rows reach: a sample of requests against converged runs of the
    # same request (16x its budget, at most 2^27, on a disjoint Halton range, split phase)
    err_sample = []
    if rank == 0:
        for k in np.linspace(0, n_req - 1, min(8, n_req)).astype(int):
            row = handles[k].result()[0].astype(np.complex128)
            rf = scenes.rf_chirp(bandwidth=float(bw[k]), samples=int(nbins[k]))
            ref_budget = min(16 * int(budget[k]), 1 << 27)
            ref = backends[int(sid[k])].simulate_batch(rf, int(nbins[k]), t, [poses[k]], [poses[k]], [ref_budget],
                                                       index_offset=[TTE_REF_OFFSET],
                                                       phase_mode=HSR_PHASE_SPLIT_FP64)[0].astype(np.complex128)
            nr = np.linalg.norm(ref)
            if nr > 0:
                err_sample.append((int(budget[k]), float(np.linalg.norm(row - ref) / nr)))
    lat = np.array([i["latency_ms"] for i in infos])
    que = np.array([i["queue_ms"] for i in infos])
    paths = int(budget.sum())
    wall_max = max_over_ranks(dist, wall)
    value = world * paths / wall_max  # replicas: every rank served a stream of the same law
    offered = paths / float(arrivals[-1]) if n_req > 1 else float("nan")
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world, "steps": 1,
        "warmup": max(args.warmup, 3), "ms_per_step": 1000.0 * wall_max, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "serving: %d resident scenes (%s), %.0f req/s Poisson for %.1f s, budgets "
                               "2^16..2^24 log-uniform, bandwidth 1..4 GHz, N in {128,256,512}, 4 bounces, "
                               "split FP64 phase%s" % (len(backends), ", ".join("%s-%dk" % (k, n // 1000) for k, n in
                                                                                 scenes.SERVE_SCENES),
                                                       args.rate, args.duration,
                                                       ", guided requests (doubling schedule across ticks)"
                                                       if args.guided else ""),
                   "requests": n_req, "triangles": tris, "scene_bytes": st["scene_bytes"],
                   "max_slots": args.slots, "tick_ms": args.tick_ms, "setup_s": setup_s,
                   "l2": "inputs larger than L2 (%.2f GB of resident scenes)" % (st["scene_bytes"] / 1e9)},
        "serving": {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                    "max_ms": float(lat.max()), "queue_p50_ms": float(np.percentile(que, 50)),
                    "queue_p99_ms": float(np.percentile(que, 99)), "offered_paths_per_s": offered,
                    "device_paths_per_s": st["samples"] / (st["device_ms"] / 1000.0) if st["device_ms"] else None,
                    "device_busy_frac": st["device_ms"] / (1000.0 * wall), "ticks": st["ticks"],
                    "max_batch": st["max_batch"], "max_resident": st["max_resident"],
                    "admitted_while_busy": st["admitted_while_busy"], "failed": st["failed"],
                    "error_sample": {"requests": [{"budget": b, "rel_l2": e, "db": 20 * float(np.log10(e))}
                                                  for b, e in err_sample],
                                     "at_minus40db": sum(e <= TTE_TARGET for _, e in err_sample),
                                     "reference": "16x the request's budget (at most 2^27), disjoint Halton range"}},
        "e2e": {"value": value, "unit": "paths/s",
                "h2d_bytes_per_step": int(n_req * 152), "d2h_bytes_per_step": int(8 * nbins.sum()),
                "note": "wall clock from the first arrival to the last row on the host, through hsr_server_*"},
        "gpu_launches": int(st["ticks"]),
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
    ap.add_argument("--workload", default="boxes",
                    choices=["boxes", "sphere", "serve", "tte", "urban_mimo", "synth"])
    ap.add_argument("--poses", type=int, default=None, help="boxes workload: trace the first P poses")
    ap.add_argument("--launch-config", default=None,
                    help="boxes and sphere workloads: tile,ctas_per_sm,queue_threshold,field_on_hit[,coherent_order] "
                         "instead of autotuning")
    ap.add_argument("--max-log2", type=int, default=None,
                    help="boxes workload: cap every budget at 2^k (small profiling cases only)")
    ap.add_argument("--traffic", type=float, default=None,
                    help="DRAM bytes per trace launch from an ncu capture of the same workload (reported as-is)")
    ap.add_argument("--kernel-only", action="store_true",
                    help="timed steps only (no e2e, counting, CPU baseline): the profiling command")
    ap.add_argument("--no-tte", action="store_true", help="skip the time-to--40 dB measurement")
    ap.add_argument("--rate", type=float, default=200.0, help="serve: Poisson arrival rate (req/s)")
    ap.add_argument("--duration", type=float, default=2.0, help="serve: seconds of arrivals")
    ap.add_argument("--slots", type=int, default=256, help="serve: requests admitted at once")
    ap.add_argument("--tick-ms", type=float, default=4.0, help="serve: target device time per tick")
    ap.add_argument("--guided", action="store_true", help="serve: guided requests (PathTracer::run's schedule)")
    args = ap.parse_args()
    rank, world, local_rank = dist_env()
    dist = init_dist(world)
    if args.impl == "reference":
        run_reference(args, rank, world, dist)
    elif args.workload == "serve":
        run_serve(args, rank, world, local_rank, dist)
    elif args.workload == "synth":
        run_synth(args, rank, world, local_rank, dist)
    elif args.workload == "urban_mimo":
        run_urban_mimo(args, rank, world, local_rank, dist)
    elif args.workload == "tte":
        if rank == 0:
            import torch
            torch.cuda.set_device(local_rank)
            print(json.dumps({"time_to_minus40db": time_to_error(with_boxes=True)}), flush=True)
    elif args.workload == "boxes":
        run_batched(args, rank, world, local_rank, dist)
    else:
        run_gb300(args, rank, world, local_rank, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
