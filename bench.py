#!/usr/bin/env python3
"""k-means discretization throughput on GB300 (frames/s).

Workload (per GPU): one Lloyd iteration of k-means -- assignment of every
frame to its nearest center, float64 centroid update, inertia and the
convergence test -- on 2,000,000 frames x 528 float32 pairwise C-alpha
distances of a 33-bead chain, k = 2000.  The assignment runs on the tcgen05
tensor cores (FP16 operands, FP32 accumulation) with an exact FP32 recheck of
near ties (labels equal the plain FP32 kernel's bit for bit).  A "step" is one Lloyd iteration.

  value       frames/s over the timed steps, inputs resident in HBM, whole job
  e2e         the same metric through the public API (KmeansClustering.estimate
              with max_iter=1) from pinned host frames, copies inside the clock
  roofline    the tensor-core distance kernel: 2*N*k*d flops per launch over its
              CUDA-event launch time, against the measured sustained BF16 peak
              (FP16 and BF16 share the kind::f16 tensor rate)
  plain_fp32  the same Lloyd iteration with the exact FP32 CUDA-core kernel
  cpu_baseline  the CPU oracle (C/OpenMP restatement of the reference path) on
              a bounded sample, all host cores

--impl reference times the CPU restatement of the reference's
implementation on the host cores (bounded sample) with the same metric.

Multi-GPU (torchrun): each rank discretizes its own 2,000,000 frames (weak
scaling, no collective on the data path); value = all frames / max rank time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_FRAMES = 2_000_000
D = 528
K = 2000
SEED = 2026
METRIC = "k-means frames/s (Lloyd iteration: assign + centroid update + inertia)"
UNIT = "frames/s"


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--frames", type=int, default=N_FRAMES)
    p.add_argument("--no-fp32", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    return p.parse_args()


def config(args, extra=None):
    c = {"workload": "k-means Lloyd iteration on %d x %d float32 C-alpha pair distances (33-bead chain), "
                     "k=%d" % (args.frames, D, K),
         "n_frames_per_gpu": args.frames, "d": D, "k": K, "precision": "fp16 tensor cores + exact fp32 recheck",
         "l2": "inputs (%.1f GB of frames) larger than L2 (129 MB)" % (args.frames * D * 4 / 1e9),
         "parallelism": "frames sharded per GPU, no collective" if args.gpus > 1 else "single GPU"}
    if extra:
        c.update(extra)
    return c


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler(object):
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id):
        self.samples = []
        self.proc = None
        self.gpu_id = gpu_id
        self.mark = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", self.gpu_id, "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) == 8:
                self.samples.append((time.time(), parts))

    def window(self, t0, t1):
        return [p for t, p in self.samples if t0 <= t <= t1]

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0, t1):
        rows = self.window(t0, t1) or [p for _, p in self.samples]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no nvidia-smi samples"], "samples": 0}
        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[0]) for r in rows if num(r[0]) is not None]
        mx = [num(r[1]) for r in rows if num(r[1]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[4 + i].lower() == "active"})
        pw = [num(r[2]) for r in rows if num(r[2]) is not None]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "power_w_max": max(pw) if pw else None}


def gpu_id_for_smi(torch):
    try:
        return "GPU-" + str(torch.cuda.get_device_properties(torch.cuda.current_device()).uuid)
    except Exception:
        return "0"


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def profiled_traffic():
    """Per-launch DRAM bytes of the tensor-core kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "tc_assign_kernel_c3.md")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch_full_size:"):
                return float(line.split(":", 1)[1].strip())
    except OSError:
        pass
    return None


# ---------------------------------------------------------------------------
# CPU legs (oracle = C/OpenMP restatement of the reference path)
# ---------------------------------------------------------------------------
def cpu_lloyd_rate(X, C, target_s, threads):
    """Frames/s of one oracle Lloyd iteration on a sample sized for ~target_s."""
    from oracle import oracle
    n0 = min(len(X), 256)
    t = time.perf_counter()
    oracle.assign(X[:n0], C, n_threads=threads)
    per = (time.perf_counter() - t) / n0
    S = int(min(len(X), max(n0, target_s / max(per, 1e-9))))
    Xs = np.ascontiguousarray(X[:S])
    t = time.perf_counter()
    oracle.lloyd(Xs, C, 1, -1.0, n_threads=threads)
    dt = time.perf_counter() - t
    return S / dt, S, dt


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle
    from pyemma_gb300 import datasets
    threads = len(os.sched_getaffinity(0))
    oracle.lib()
    # Bounded sample of the same workload, sized so that W+K steps take a few minutes.
    X = datasets.calpha_distances(n_frames=60000, seed=SEED)
    rng = np.random.default_rng(SEED)
    C = X[rng.choice(len(X), K, replace=False)].copy()
    steps = max(1, args.steps)
    budget = 150.0 / (steps + args.warmup)
    n0 = 128
    t = time.perf_counter()
    oracle.assign(X[:n0], C, n_threads=threads)
    per = (time.perf_counter() - t) / n0
    S = int(min(len(X), max(n0, min(10.0, budget) / max(per, 1e-9))))
    Xs = np.ascontiguousarray(X[:S])
    for _ in range(args.warmup):
        oracle.lloyd(Xs, C, 1, -1.0, n_threads=threads)
    times = []
    for _ in range(steps):
        t = time.perf_counter()
        oracle.lloyd(Xs, C, 1, -1.0, n_threads=threads)
        times.append(time.perf_counter() - t)
    ms = 1e3 * sum(times) / len(times)
    value = S / (ms / 1e3)
    sample = "%d of %d frames (d=%d, k=%d), one Lloyd iteration per step" % (S, args.frames, D, K)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 distances, f64 sums", "data": "synthetic (seeded C-alpha distances)",
            "config": config(args, {"precision": "fp32 (CPU)"}), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_ours(args):
    import torch
    from pyemma_gb300 import _lib, datasets
    from pyemma_gb300.coordinates import KmeansClustering

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend="nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    _lib.load()
    n = args.frames
    X = datasets.calpha_distances(n_frames=n, seed=SEED + rank, device="cuda")
    rng = np.random.default_rng(SEED + rank)
    C0 = X[torch.from_numpy(rng.choice(n, K, replace=False)).cuda()].contiguous()
    torch.cuda.synchronize()

    sampler = ClockSampler(gpu_id_for_smi(torch)) if rank == 0 else None
    if sampler:
        sampler.start()

    # warm-up (also builds the one-time state of the library)
    C = C0.clone()
    _lib.lloyd(X, C, max(3, args.warmup), -1.0, precision="fp16")

    # ---- timed region: K Lloyd iterations, graph-launched ----
    C = C0.clone()
    _lib.profile_enable(True)
    barrier()
    t_wall0 = time.time()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    res = _lib.lloyd(X, C, args.steps, -1.0, precision="fp16")
    ev1.record()
    torch.cuda.synchronize()
    barrier()
    t_wall1 = time.time()
    ms = ev0.elapsed_time(ev1)
    prof = _lib.profile_read()
    _lib.profile_enable(False)
    assert res["n_iter"] == args.steps
    ms_max = ms
    if dist is not None:
        t = torch.tensor([ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_max = float(t.item())
    ms_per_step = ms_max / args.steps
    value = world * n * args.steps / (ms_max / 1e3)

    clocks = sampler.summary(t_wall0, t_wall1) if sampler else None

    # ---- roofline of the tensor-core distance kernel ----
    peaks, peak_kind = measured_peaks()
    tc_ms, tc_n = prof["tc"]
    flops = 2.0 * n * K * D
    achieved = flops / (tc_ms / tc_n / 1e3) / 1e12 if tc_n else None
    peak = float(peaks.get("bf16_tflops_sustained", 1700.0))
    roofline = {"bound": "tensor", "kernel": "tc_assign_kernel", "achieved": achieved, "peak": peak,
                "unit": "TFLOP/s", "frac": achieved / peak if achieved else None, "traffic": profiled_traffic(),
                "peak_source": "%s bf16_tflops_sustained (same kind::f16 rate as fp16)" % peak_kind,
                "launches": tc_n, "ms_per_launch": tc_ms / tc_n if tc_n else None,
                "flops_per_launch": flops,
                "step_breakdown_ms": {k: (v[0] / v[1] if v[1] else None) for k, v in prof.items()}}

    extra = {}
    if rank == 0:
        # assignment statistics and exactness against the plain FP32 kernel
        lab16, st = _lib.assign(X, C, precision="fp16")
        extra["recheck_fraction"] = (st["n_recheck"] + st["n_full"]) / float(n)
        extra["full_recheck_frames"] = st["n_full"]
        extra["flipped_ties"] = st["n_flipped"]
        if not args.no_fp32:
            lab32, _ = _lib.assign(X, C, precision="fp32")
            extra["dtrajs_identical_to_fp32"] = bool(torch.equal(lab16, lab32))
            del lab32
            # plain FP32 Lloyd iteration for the mixed-vs-FP32 ratio
            Cf = C0.clone()
            _lib.lloyd(X, Cf, 1, -1.0, precision="fp32")
            Cf = C0.clone()
            steps32 = 2
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            _lib.lloyd(X, Cf, steps32, -1.0, precision="fp32")
            e1.record()
            torch.cuda.synchronize()
            fp32_value = n * steps32 / (e0.elapsed_time(e1) / 1e3)
            extra["plain_fp32"] = {"value": fp32_value, "unit": UNIT, "steps": steps32}
            extra["mixed_vs_plain_fp32"] = (value / world) / fp32_value
        del lab16

    # ---- e2e through the public API from pinned host frames ----
    e2e = None
    if rank == 0 and not args.no_e2e:
        Xh = torch.empty((n, D), dtype=torch.float32, pin_memory=True)
        Xh.copy_(X)
        Xh_np = Xh.numpy()
        C0h = C0.cpu().numpy()
        del X  # the API makes its own device copy
        torch.cuda.empty_cache()
        km = KmeansClustering(n_clusters=K, max_iter=1, tolerance=-1.0, clustercenters=C0h, precision="fp16")
        km.estimate(Xh_np)  # warm-up
        e2e_steps = max(1, min(args.steps, 5))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            km = KmeansClustering(n_clusters=K, max_iter=1, tolerance=-1.0, clustercenters=C0h, precision="fp16")
            km.estimate(Xh_np)
            _ = km.clustercenters  # host result (already copied back by estimate)
        dt = (time.perf_counter() - t0) / e2e_steps
        e2e = {"value": n / dt, "unit": UNIT, "h2d_bytes_per_step": n * D * 4, "d2h_bytes_per_step": K * D * 4 + 8,
               "api": "KmeansClustering(n_clusters=2000, max_iter=1, clustercenters=C).estimate(pinned host X)",
               "steps": e2e_steps}

    # ---- CPU baseline (rank 0, N=1) ----
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = len(os.sched_getaffinity(0))
        Xc = datasets.calpha_distances(n_frames=40000, seed=SEED)
        rate, S, dt = cpu_lloyd_rate(Xc, C0.cpu().numpy(), 12.0, threads)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "%d C-alpha frames (d=%d) x k=%d centers, one oracle Lloyd iteration, %.1f s"
                         % (S, D, K, dt)}

    if sampler:
        sampler.stop()
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    if rank != 0:
        return
    launches_per_step = 11  # prep_centers, tc, 2 pair-recheck kernels, full recheck, 6 update kernels
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp16 distances (fp32 accumulate), fp32 recheck, f64 sums",
            "data": "synthetic (seeded C-alpha distances, generated on device)",
            "config": config(args), "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
            "gpu_launches": launches_per_step * args.steps + 2}
    line.update(extra)
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
