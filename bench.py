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
              with max_iter=1) from pinned host frames, copies inside the clock;
              a round of calls in which one call took more than twice the bare
              copy time (a disturbed host link) is kept as rejected and taken
              once more
  roofline    the tensor-core distance kernel: 2*N*k*d flops per launch over its
              CUDA-event launch time, against the measured BF16 peak (FP16 and
              BF16 share the kind::f16 tensor rate): the burst peak for a timed
              region under 2 s, the sustained one beyond; frac_issued counts
              the padded MMA work the kernel issues
  centers_rel_err_vs_fp64 / inertia_rel_err_vs_fp64
              one more Lloyd iteration against the float64 NumPy reference
              (member means and inertia of the GPU's labels, all frames)
  kmeans++    km_kmpp with k=2000 on all frames, timed with CUDA events
  plain_fp32  the same Lloyd iteration with the exact FP32 CUDA-core kernel
  cpu_baseline  the CPU oracle (C/OpenMP restatement of the reference path) on
              a bounded sample, all host cores

--impl reference times the CPU restatement of the reference's
implementation on the host cores (bounded sample) with the same metric.

--config selects the other measured workloads (each prints its own line):
  c1  100,000 x 2 mixture, k=50: kmeans++ + Lloyd to convergence + dtrajs
  c2  20 uneven AR(1) trajectories (~3.9M frames), d=10, k=1000, packed
  c4  precision sweep, 1M frames, d in {16,64,256,1024}, k in {100,1000,5000}
  c5  serving: Poisson arrivals (200 req/s) of trajectories of 1k-1M frames
      against 8 resident center sets, 40 GB admission budget, p50/p99

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
    p.add_argument("--steps", type=int, default=300)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--frames", type=int, default=N_FRAMES)
    p.add_argument("--no-fp32", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-fp64", action="store_true", help="skip the float64 reference check of the centers")
    p.add_argument("--no-kmpp", action="store_true", help="skip the kmeans++ timing")
    p.add_argument("--config", default="c3", choices=["c1", "c2", "c3", "c4", "c5", "minrmsd"])
    p.add_argument("--serve-seconds", type=float, default=10.0)
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
                                          "--format=csv,noheader,nounits", "-lms", "50"],
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
        with open(path) as fh:
            for line in fh:
                if line.startswith("traffic_bytes_per_launch_full_size:"):
                    return float(line.split(":", 1)[1].strip())
    except OSError:
        pass
    return None


# Timed regions at least this long are compared with the sustained (power-
# capped) bf16 peak; shorter ones with the burst peak.
SUSTAINED_AFTER_MS = 2000.0


def padded_mma_flops(n, k, d):
    """MMA work the tensor-core kernel issues per launch: frames padded to the
    256-row CTA-pair tile, centers to the 256-row B tile, and K to the 16-wide
    MMA steps that hold the d features plus the two norm columns."""
    n_pad = -(-n // 256) * 256
    k_pad = -(-k // 256) * 256
    k_steps = 16 * (-(-(d + 2) // 16))
    return 2.0 * n_pad * k_pad * k_steps


def tc_chunks(n):
    """Launches of one iteration's tensor-core pass: the library splits a
    Lloyd pass into KM_TC_CHUNKS (default 4) launches of at least 2^18
    frames each, so that each chunk's exact re-check runs beside the next."""
    want = max(1, min(int(os.environ.get("KM_TC_CHUNKS", "4")), 8))
    return max(1, min(want, n >> 18))


def tc_roofline(n, tc_ms, tc_n, timed_ms, k=K, d=D):
    """Roofline record of the tensor-core distance kernel: 2 n k d flops per
    launch over its mean CUDA-event launch time, against the measured bf16
    peak (FP16 and BF16 share the kind::f16 rate).  The burst peak applies
    unless the timed region ran long enough to settle under the power cap."""
    peaks, peak_kind = measured_peaks()
    flops = 2.0 * n * k * d
    issued = padded_mma_flops(n, k, d)
    t = tc_ms / tc_n / 1e3 if tc_n else None
    achieved = flops / t / 1e12 if t else None
    if timed_ms >= SUSTAINED_AFTER_MS:
        key, rule = "bf16_tflops_sustained", "timed region %.0f ms >= %.0f ms: sustained" % (timed_ms,
                                                                                             SUSTAINED_AFTER_MS)
    else:
        key, rule = "bf16_tflops", "timed region %.0f ms < %.0f ms: burst" % (timed_ms, SUSTAINED_AFTER_MS)
    peak = float(peaks.get(key, 1900.0 if key == "bf16_tflops" else 1700.0))
    return {"bound": "tensor", "kernel": "tc_assign_kernel", "achieved": achieved, "peak": peak,
            "unit": "TFLOP/s", "frac": achieved / peak if achieved else None, "traffic": profiled_traffic(),
            "peak_source": "%s %s of MEASURED_PEAKS.json (%s)" % (peak_kind, key, rule),
            "issued_tflops": issued / t / 1e12 if t else None,
            "frac_issued": issued / t / 1e12 / peak if t else None,
            "issued_flops_per_launch": issued,
            "launches": tc_n, "ms_per_launch": t * 1e3 if t else None, "flops_per_launch": flops}


def fp64_reference_check(X_host, labels, C_prev, C_new, inertia):
    """Centers and inertia of one GPU Lloyd iteration against the float64
    NumPy member means and inertia of the same labels (the oracle's
    centers_fp64 / inertia_fp64)."""
    from oracle import oracle
    mu, cnt = oracle.centers_fp64(X_host, labels, C_prev)
    ref_inertia = oracle.inertia_fp64(X_host, labels, mu)
    got = np.asarray(C_new, dtype=np.float64)
    rel = np.abs(got - mu) / np.maximum(np.abs(mu), 1e-30)
    return {"centers_rel_err_vs_fp64": float(rel.max()),
            "inertia_rel_err_vs_fp64": abs(inertia - ref_inertia) / ref_inertia,
            "fp64_reference": "oracle.centers_fp64 / inertia_fp64 on the GPU's labels of one Lloyd iteration "
                              "(all %d frames)" % len(labels),
            "empty_clusters": int((cnt == 0).sum())}


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


def max_over_ranks(ms, dist, device):
    """The slowest rank's time (every rank gets it); ms itself on one rank."""
    if dist is None:
        return float(ms)
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world, frames_per_rank, steps, ms_max):
    """Frames of all ranks per second over the slowest rank's time.  Every
    rank owns its own frames (weak scaling; no data-path collective)."""
    return world * frames_per_rank * steps / (ms_max / 1e3)


def rank_seed(rank):
    """Each rank's frames are drawn from their own seed."""
    return SEED + rank


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
    X = datasets.calpha_distances(n_frames=n, seed=rank_seed(rank), device="cuda")
    rng = np.random.default_rng(rank_seed(rank))
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
    ms_max = max_over_ranks(ms, dist, "cuda")
    ms_per_step = ms_max / args.steps
    value = whole_job_rate(world, n, args.steps, ms_max)

    clocks = sampler.summary(t_wall0, t_wall1) if sampler else None
    if sampler:
        # nvidia-smi's queries take driver locks: keep them out of the
        # end-to-end copies measured below
        sampler.stop()
        sampler = None

    # ---- roofline of the tensor-core distance kernel ----
    # In the step, one iteration's pass is tc_chunks(n) launches with the
    # exact re-check of each chunk beside the next: ms_per_launch is the span
    # from the first launch's start to the last one's end.  The same kernel
    # alone (one launch over all frames, the re-check after it) is timed
    # below as "isolated".
    tc_ms, tc_n = prof["tc"]
    roofline = tc_roofline(n, tc_ms, tc_n, ms)
    roofline["step_breakdown_ms"] = {k: (v[0] / v[1] if v[1] else None) for k, v in prof.items()}
    roofline["chunks_per_iteration"] = tc_chunks(n)
    roofline["span"] = ("ms_per_launch: one iteration's tensor-core pass, %d launches over consecutive frame "
                        "ranges, from the first start to the last end, each chunk's exact re-check running "
                        "beside the next launch" % tc_chunks(n))
    if rank == 0:
        old = os.environ.get("KM_TC_CHUNKS")
        os.environ["KM_TC_CHUNKS"] = "1"
        try:
            Ci = C0.clone()
            _lib.lloyd(X, Ci, 2, -1.0, precision="fp16")
            Ci = C0.clone()
            iso_steps = 20
            _lib.profile_enable(True)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            _lib.lloyd(X, Ci, iso_steps, -1.0, precision="fp16")
            e1.record()
            torch.cuda.synchronize()
            iprof = _lib.profile_read()
            _lib.profile_enable(False)
            iso = tc_roofline(n, iprof["tc"][0], iprof["tc"][1], e0.elapsed_time(e1))
            roofline["isolated"] = {key: iso[key] for key in ("achieved", "frac", "issued_tflops", "frac_issued",
                                                               "ms_per_launch", "launches", "peak_source")}
            roofline["isolated"]["ms_per_step"] = e0.elapsed_time(e1) / iso_steps
            roofline["isolated"]["how"] = ("the same kernel as one launch over all %d frames per iteration "
                                           "(KM_TC_CHUNKS=1), %d iterations" % (n, iso_steps))
            del Ci
        finally:
            if old is None:
                del os.environ["KM_TC_CHUNKS"]
            else:
                os.environ["KM_TC_CHUNKS"] = old

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
    if rank == 0 and not args.no_kmpp:
        # kmeans++ (k rounds of D^2 sampling) on the same frames
        _lib.kmpp(X[:65536].contiguous(), 8, 42)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        _, kidx = _lib.kmpp(X, K, 42)
        e1.record()
        torch.cuda.synchronize()
        kmpp_ms = e0.elapsed_time(e1)
        unpruned = float(K) * n * (4 * D + 8)
        extra["kmeans++"] = {"ms": kmpp_ms, "rounds": K, "ms_per_round": kmpp_ms / K,
                             "unpruned_bytes": unpruned,
                             "unpruned_bytes_per_s": unpruned / (kmpp_ms / 1e3),
                             "note": "km_kmpp, k=%d on all %d frames (seed 42); unpruned_bytes = k N (4d + 8), "
                                     "the bytes a pass without distance bounds would read" % (K, n)}
        del kidx

    # ---- e2e through the public API from pinned host frames ----
    e2e = None
    if rank == 0 and not args.no_e2e:
        Xh = torch.empty((n, D), dtype=torch.float32, pin_memory=True)
        Xh.copy_(X)
        Xh_np = Xh.numpy()
        C0h = C0.cpu().numpy()
        if not args.no_fp64:
            # centers and inertia of one more iteration (from the timed run's
            # centers) against the float64 reference on the same labels
            C_prev = C.clone()
            r1 = _lib.lloyd(X, C, 1, -1.0, precision="fp16")
            extra.update(fp64_reference_check(Xh_np, r1["labels"].cpu().numpy(), C_prev.cpu().numpy(),
                                              C.cpu().numpy(), float(r1["inertias"][0])))
            del r1, C_prev
        # the bare pinned host-to-device rate of this machine, for reading e2e
        # (the best of three copies: a single one has read low on a busy host)
        ec0, ec1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        X.copy_(Xh, non_blocking=True)
        copy_ms = []
        for _ in range(3):
            ec0.record()
            X.copy_(Xh, non_blocking=True)
            ec1.record()
            torch.cuda.synchronize()
            copy_ms.append(ec0.elapsed_time(ec1))
        link_gbs_engine = n * D * 4 / (min(copy_ms) / 1e3) / 1e9
        # the same bytes through the library's own host copy (km_lloyd_host
        # with no iteration: the copy kernel alone), best of three
        kernel_ms = []
        Cq = C0.clone()
        for _ in range(4):
            torch.cuda.synchronize()
            tk = time.perf_counter()
            _lib.lloyd_host([Xh_np], Cq, 0, -1.0, precision="fp16", X=X)
            torch.cuda.synchronize()
            kernel_ms.append((time.perf_counter() - tk) * 1e3)
        link_gbs_kernel = n * D * 4 / (min(kernel_ms[1:]) / 1e3) / 1e9
        link_gbs = max(link_gbs_engine, link_gbs_kernel)
        del X, Cq  # the API makes its own device copy
        torch.cuda.empty_cache()
        # Warm-up: the first passes over a freshly allocated multi-GB pinned
        # buffer run slower (32 against 21 ms per call here) while its pages
        # are first mapped for the device; W >= 3 calls precede the timing.
        e2e_warm = max(3, args.warmup)
        for _ in range(e2e_warm):
            KmeansClustering(n_clusters=K, max_iter=1, tolerance=-1.0, clustercenters=C0h,
                             precision="fp16").estimate(Xh_np)
        e2e_steps = max(1, min(args.steps, 8))
        copy_ms_best = n * D * 4 / (link_gbs * 1e9) * 1e3

        def e2e_round(frames):
            # e2e_steps calls, each with its own clock; the mean is the rate.
            # A call that took more than twice the bare copy of its frames met
            # a disturbed host link (other users' traffic on the shared host):
            # such a round is kept in the line as rejected and taken once more.
            rounds = []
            for _ in range(2):
                step = []
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                for _ in range(e2e_steps):
                    ts = time.perf_counter()
                    km = KmeansClustering(n_clusters=K, max_iter=1, tolerance=-1.0, clustercenters=C0h,
                                          precision="fp16")
                    km.estimate(frames)
                    _ = km.clustercenters  # host result (already copied back by estimate)
                    step.append((time.perf_counter() - ts) * 1e3)
                rounds.append(((time.perf_counter() - t0) / e2e_steps, step))
                if max(step) <= 2.0 * copy_ms_best:
                    break
            rejected = [{"step_ms": st, "reason": "a call took more than twice the bare copy (%.1f ms)"
                         % copy_ms_best} for _, st in rounds[:-1]]
            return rounds[-1][0], rounds[-1][1], rejected

        dt, step_ms, rejected = e2e_round(Xh_np)
        e2e = {"value": n / dt, "unit": UNIT, "h2d_bytes_per_step": n * D * 4, "d2h_bytes_per_step": K * D * 4 + 8,
               "api": "KmeansClustering(n_clusters=2000, max_iter=1, clustercenters=C).estimate(pinned host X)",
               "steps": e2e_steps, "warmup": e2e_warm, "step_ms": step_ms, "rejected_rounds": rejected,
               "h2d_link_gbs": link_gbs,
               "h2d_link_gbs_copy_engine": link_gbs_engine, "h2d_link_gbs_copy_kernel": link_gbs_kernel,
               "copy_bound_frames_per_s": link_gbs * 1e9 / (D * 4),
               "overlap": "frames copied in chunks on a side stream while the first iteration assigns "
                          "the chunks already copied (km_lloyd_host)"}
        # The same call with the frames in an ordinary (pageable) numpy
        # array, as PyEMMA callers hold them: where the GPU reads host memory
        # in place (Grace), a device kernel copies the chunks; elsewhere the
        # library stages them through page-locked buffers on worker threads.
        Xpg = np.empty_like(Xh_np)
        Xpg[...] = Xh_np
        del Xh, Xh_np
        for _ in range(e2e_warm):
            KmeansClustering(n_clusters=K, max_iter=1, tolerance=-1.0, clustercenters=C0h,
                             precision="fp16").estimate(Xpg)
        dtp, step_ms_pg, rejected_pg = e2e_round(Xpg)
        e2e["pageable"] = {"value": n / dtp, "unit": UNIT, "h2d_bytes_per_step": n * D * 4,
                           "d2h_bytes_per_step": K * D * 4 + 8, "vs_pinned": (n / dtp) / e2e["value"],
                           "step_ms": step_ms_pg, "rejected_rounds": rejected_pg,
                           "api": "KmeansClustering(max_iter=1, clustercenters=C).estimate(pageable numpy X)"}
        del Xpg
        # The same iteration from pinned host C-alpha coordinates: the 528
        # pair distances are never written out; every kernel that reads a
        # feature computes it from the coordinates (km_lloyd_pairs), so 396
        # bytes per frame cross the host link and no n x 528 matrix exists.
        from pyemma_gb300 import featurize
        xyz_d = datasets.calpha_coordinates(n_frames=n, seed=SEED + rank)
        xyz_h = torch.empty(tuple(xyz_d.shape), dtype=torch.float32, pin_memory=True)
        xyz_h.copy_(xyz_d)
        src = featurize.pair_distance_frames(xyz_d, excluded_neighbors=0)
        # Lloyd iterations on device-resident coordinates, for the step time
        Cp = C0.clone()
        _lib.lloyd_pairs(src.xyz, src.pairs, Cp, 2, -1.0, precision="fp16")
        Cp = C0.clone()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        _lib.lloyd_pairs(src.xyz, src.pairs, Cp, 5, -1.0, precision="fp16")
        e1.record()
        torch.cuda.synchronize()
        pair_ms = e0.elapsed_time(e1) / 5
        del src, xyz_d, Cp
        torch.cuda.empty_cache()
        for _ in range(e2e_warm):
            km = KmeansClustering(n_clusters=K, max_iter=1, tolerance=-1.0, clustercenters=C0h, precision="fp16")
            km.estimate(featurize.pair_distance_frames(xyz_h, excluded_neighbors=0))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            km = KmeansClustering(n_clusters=K, max_iter=1, tolerance=-1.0, clustercenters=C0h, precision="fp16")
            km.estimate(featurize.pair_distance_frames(xyz_h, excluded_neighbors=0))
            _ = km.clustercenters
        dtc = (time.perf_counter() - t0) / e2e_steps
        kp = 64 * (-(-(D + 2) // 64))
        e2e["from_coordinates"] = {
            "value": n / dtc, "unit": UNIT, "h2d_bytes_per_step": n * 33 * 3 * 4, "d2h_bytes_per_step": K * D * 4 + 8,
            "api": "KmeansClustering(max_iter=1).estimate(featurize.pair_distance_frames(pinned host xyz (n, 33, 3)))",
            "feature_matrix_bytes": 0,
            "device_lloyd_ms_per_iter": pair_ms,
            "hbm_bytes_per_iter": {"fp16_copy": n * kp * 2, "coordinates": n * 33 * 3 * 4,
                                   "dense_path_float32_features": n * D * 4},
            "workload": "same chain model, coordinates instead of precomputed distances; the features are computed "
                        "where they are read (km_lloyd_pairs)"}
        del xyz_h

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
    # Per iteration: prep_centers; per chunk of the tensor-core pass the
    # tensor-core launch (which also counts the members), 3 candidate
    # re-check kernels and 3 full re-check kernels (short list, tiled,
    # finalize); 6 centroid-update kernels (scan, scatter, segment sums,
    # flips, finalize, cost).  Once per km_lloyd call: shift, center norms,
    # scale, FP16 frame copy.
    launches_per_step = 1 + 7 * tc_chunks(n) + 6
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp16 distances (fp32 accumulate), fp32 recheck, f64 sums",
            "data": "synthetic (seeded C-alpha distances, generated on device)",
            "config": config(args), "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
            "gpu_launches": launches_per_step * args.steps + 4}
    line.update(extra)
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# other workloads (--config)
# ---------------------------------------------------------------------------
def _emit(line):
    print(json.dumps(line), flush=True)


def _fp32_sgemm_tflops(torch):
    """Measured FP32 (no TF32) GEMM rate of this GPU: the CUDA-core FMA peak proxy."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        a = torch.randn(8192, 8192, device="cuda")
        b = torch.randn(8192, 8192, device="cuda")
        for _ in range(2):
            a @ b
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(5):
            a @ b
        e1.record()
        torch.cuda.synchronize()
        return 5 * 2 * 8192.0 ** 3 / (e0.elapsed_time(e1) / 1e3) / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def _lloyd_rate(torch, _lib, X, C0, steps, precision):
    """(ms per Lloyd iteration, profile) over `steps` graph-launched iterations."""
    C = C0.clone()
    _lib.lloyd(X, C, 3, -1.0, precision=precision)
    C = C0.clone()
    _lib.profile_enable(True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    _lib.lloyd(X, C, steps, -1.0, precision=precision)
    e1.record()
    torch.cuda.synchronize()
    prof = _lib.profile_read()
    _lib.profile_enable(False)
    return e0.elapsed_time(e1) / steps, prof


def tile_tuning(torch, _lib, X, C0, steps):
    """The fixed tile plan's Lloyd iteration against the one km_tune_tiles
    picks for (d, k) on these frames; the table is cleared afterwards."""
    d, k = X.shape[1], C0.shape[0]
    _lib.tune_clear()
    fixed = _lib.tile_plan(d, k)
    ms_fixed, _ = _lloyd_rate(torch, _lib, X, C0, steps, "fp16")
    r = _lib.tune_tiles(X, C0)
    tuned = _lib.tile_plan(d, k)
    ms_tuned, _ = _lloyd_rate(torch, _lib, X, C0, steps, "fp16")
    lab_t, _ = _lib.assign(X, C0, precision="fp16")
    _lib.tune_clear()
    lab_f, _ = _lib.assign(X, C0, precision="fp16")
    return {"fixed_plan": fixed, "fixed_ms_per_iter": ms_fixed, "tuned_plan": tuned, "tuned_ms_per_iter": ms_tuned,
            "speedup": ms_fixed / ms_tuned, "labels_identical": bool(torch.equal(lab_t, lab_f)),
            "assign_ms_by_plan": [dict(t) for t in r["tried"]]}


def run_c1(args):
    """100,000 x 2, k=50, kmeans++ (fixed_seed=42), max_iter=100, tol 1e-5, then dtrajs."""
    import torch
    from oracle import oracle
    from pyemma_gb300 import _lib, datasets
    from pyemma_gb300.coordinates import cluster_kmeans
    _lib.load()
    X = datasets.small_mixture(seed=SEED)
    cluster_kmeans(X, k=50, max_iter=100, tolerance=1e-5, fixed_seed=42).dtrajs  # warm-up
    times, its = [], []
    for _ in range(max(3, args.steps // 10)):
        torch.cuda.synchronize()
        t = time.perf_counter()
        km = cluster_kmeans(X, k=50, max_iter=100, tolerance=1e-5, fixed_seed=42)
        dtrajs = km.dtrajs
        times.append(time.perf_counter() - t)
        its.append(int(len(km.inertias)))
    ms = 1e3 * statistics.median(times)
    threads = len(os.sched_getaffinity(0))
    t = time.perf_counter()
    C0, _ = oracle.kmpp(X, 50, 42, n_threads=threads)
    res = oracle.lloyd(X, C0, 100, 1e-5, n_threads=threads)
    oracle.assign(X, res["centers"], n_threads=threads)
    cpu_ms = 1e3 * (time.perf_counter() - t)
    _emit({"metric": "k-means wall time (kmeans++ + Lloyd to convergence + dtrajs)", "value": ms, "unit": "ms",
           "higher_is_better": False, "n_gpus": 1, "frames": len(X), "lloyd_iterations": its[-1],
           "frames_per_s_end_to_end": len(X) / (ms / 1e3),
           "config": {"workload": "c1: 100000 x 2 mixture of 10 Gaussians (sigma 0.5, means U[-5,5]^2), k=50, "
                                  "kmeans++ fixed_seed=42, max_iter=100, tol=1e-5, public API from host numpy"},
           "cpu_oracle_ms": cpu_ms, "cpu_cores": threads, "dtrajs_len": int(sum(len(d) for d in dtrajs)),
           "bound": "launch/latency (1.2 MB per pass); no roofline fraction"})


def run_c2(args):
    """20 uneven AR(1) trajectories, d=10, k=1000: packed Lloyd iterations."""
    import torch
    from pyemma_gb300 import _lib, datasets
    from pyemma_gb300.coordinates import KmeansClustering
    _lib.load()
    trajs = datasets.metastable_trajectories(n_traj=20, d=10, seed=SEED)
    n = sum(len(t) for t in trajs)
    X = torch.from_numpy(np.concatenate(trajs)).cuda()
    rng = np.random.default_rng(SEED)
    C0 = X[torch.from_numpy(rng.choice(n, 1000, replace=False)).cuda()].contiguous()
    # the library's own choice (precision "auto": FP16 tensor cores with the
    # exact re-check at d = 10, k = 1000) and the plain exact FP32 kernel
    ms, prof = _lloyd_rate(torch, _lib, X, C0, args.steps, "auto")
    ms32, prof32 = _lloyd_rate(torch, _lib, X, C0, args.steps, "fp32")
    lab_a, st_a = _lib.assign(X, C0, precision="auto")
    lab_32, _ = _lib.assign(X, C0, precision="fp32")
    same = bool(torch.equal(lab_a, lab_32))
    del lab_a, lab_32
    # tile shapes: the fixed plan against km_tune_tiles' choice for (10, 1000)
    tiles = tile_tuning(torch, _lib, X, C0, args.steps)
    flops = 2.0 * n * 1000 * 10
    fp32_ms = prof32["fp32"][0] / max(1, prof32["fp32"][1])
    peak = _fp32_sgemm_tflops(torch)
    achieved = flops / (fp32_ms / 1e3) / 1e12
    tc_ms = prof["tc"][0] / max(1, prof["tc"][1]) if prof["tc"][1] else None
    tpeak = float(measured_peaks()[0].get("bf16_tflops" if ms * args.steps < SUSTAINED_AFTER_MS
                                          else "bf16_tflops_sustained", 1900.0))
    # e2e: the public estimator on the 20 host trajectories (pinned), one iteration
    pinned = []
    for t in trajs:
        p = torch.empty(t.shape, dtype=torch.float32, pin_memory=True)
        p.numpy()[...] = t
        pinned.append(p.numpy())
    Ch = C0.cpu().numpy()
    for _ in range(max(3, args.warmup)):  # first passes over fresh pinned buffers run slower
        km = KmeansClustering(n_clusters=1000, max_iter=1, tolerance=-1.0, clustercenters=Ch)
        km.estimate(pinned)
    reps = 3
    t0 = time.perf_counter()
    for _ in range(reps):
        km = KmeansClustering(n_clusters=1000, max_iter=1, tolerance=-1.0, clustercenters=Ch)
        km.estimate(pinned)
        dtrajs = km.dtrajs
    e2e_s = (time.perf_counter() - t0) / reps
    # the next step of the pipeline: lag-10 transition counts of the 20 dtrajs
    packed = torch.from_numpy(np.concatenate(dtrajs).astype(np.int32)).cuda()
    offsets = np.concatenate([[0], np.cumsum([len(d) for d in dtrajs])]).astype(np.int64)
    _lib.count_matrix(packed, offsets, 10, 1000)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(10):
        counts = _lib.count_matrix(packed, offsets, 10, 1000)
    e1.record()
    torch.cuda.synchronize()
    cm_ms = e0.elapsed_time(e1) / 10
    _emit({"metric": "k-means frames/s (Lloyd iteration, packed uneven trajectories)", "value": n / (ms / 1e3),
           "unit": "frames/s", "n_gpus": 1, "steps": args.steps, "ms_per_step": ms, "higher_is_better": True,
           "dtype": "fp16 distances (fp32 accumulate) + exact fp32 recheck, f64 sums (precision auto)",
           "config": {"workload": "c2: 20 AR(1) metastable trajectories, lengths log-uniform [50k, 500k] "
                                  "(%d frames), d=10, k=1000, one CUDA graph per Lloyd iteration" % n,
                      "lengths": [len(t) for t in trajs]},
           "labels_identical_to_fp32": same, "recheck_fraction": st_a["n_recheck"] / float(n),
           "tile_tuning": tiles,
           "roofline": {"bound": "tensor-core epilogue: 1,000 accumulator columns per frame through tcgen05.ld and the "
                                 "candidate test; the MMA issues one 16-wide K step (10 features and 2 norm "
                                 "columns) per center tile",
                        "kernel": "tc_assign_kernel", "achieved": flops / (tc_ms / 1e3) / 1e12 if tc_ms else None,
                        "peak": tpeak, "unit": "TFLOP/s",
                        "frac": (flops / (tc_ms / 1e3) / 1e12) / tpeak if tc_ms else None,
                        "step_breakdown_ms": {k: (v[0] / v[1] if v[1] else None) for k, v in prof.items()}},
           "plain_fp32": {"value": n / (ms32 / 1e3), "ms_per_step": ms32, "kernel_ms": fp32_ms,
                          "kernel_tflops": achieved, "fp32_sgemm_tflops": peak, "frac_of_sgemm": achieved / peak,
                          "note": "exact distances take 3 instructions (sub, mul, add; no FMA) per 2 flops"},
           "e2e": {"value": n / e2e_s, "unit": "frames/s", "h2d_bytes_per_step": n * 40,
                   "d2h_bytes_per_step": n * 4 + 1000 * 40,
                   "api": "KmeansClustering(max_iter=1, clustercenters=C).estimate(20 pinned trajectories); dtrajs"},
           "dtrajs": len(dtrajs),
           "count_matrix": {"lag": 10, "ms": cm_ms, "frames_per_s": n / (cm_ms / 1e3), "counts": int(counts.sum()),
                            "note": "km_count_matrix on the 20 dtrajs, dense 1000 x 1000 int64 (memset included)"}})


def run_minrmsd(args):
    """minRMSD metric: 1,000,000 frames of 58 atoms (d=174), k=100."""
    import torch
    from pyemma_gb300 import _lib
    sys.path.insert(0, ROOT)
    from oracle import oracle
    _lib.load()
    n, n_atoms, k = 1_000_000, 58, 100
    g = torch.Generator(device="cuda").manual_seed(SEED)
    # 100 chain structures (random walks of 3.8-unit steps); every frame is a
    # noisy copy of one of them, randomly rotated and translated
    steps = torch.randn((k, n_atoms, 3), generator=g, device="cuda")
    base = torch.cumsum(3.8 * steps / steps.norm(dim=2, keepdim=True), dim=1)
    which = torch.randint(0, k, (n,), generator=g, device="cuda")
    q = torch.randn((n, 4), generator=g, device="cuda")
    q = q / q.norm(dim=1, keepdim=True)
    w, x, y, z = q.unbind(1)
    R = torch.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w),
                     2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w),
                     2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], dim=1).view(n, 3, 3)
    pos = base[which] + 0.8 * torch.randn((n, n_atoms, 3), generator=g, device="cuda")
    X = (torch.einsum("nij,naj->nai", R, pos) + 10.0 * torch.randn((n, 1, 3), generator=g, device="cuda"))
    X = X.reshape(n, 3 * n_atoms).contiguous()
    del pos, R, q, steps
    rng = np.random.default_rng(SEED)
    C0 = X[torch.from_numpy(rng.choice(n, k, replace=False)).cuda()].contiguous()
    _lib.assign_minrmsd(X, C0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 3
    e0.record()
    for _ in range(reps):
        lab = _lib.assign_minrmsd(X, C0)
    e1.record()
    torch.cuda.synchronize()
    assign_ms = e0.elapsed_time(e1) / reps
    C = C0.clone()
    _lib.lloyd_minrmsd(X, C, 1, -1.0)
    C = C0.clone()
    e0.record()
    res = _lib.lloyd_minrmsd(X, C, args.steps, -1.0)
    e1.record()
    torch.cuda.synchronize()
    lloyd_ms = e0.elapsed_time(e1) / args.steps
    assert res["n_iter"] == args.steps
    # parity and the CPU oracle on a sample
    sample = rng.choice(n, 20000, replace=False)
    Xs = X[torch.from_numpy(sample).cuda()].cpu().numpy()
    Ch = C0.cpu().numpy()
    threads = len(os.sched_getaffinity(0))
    t0 = time.perf_counter()
    lab_o = oracle.assign_minrmsd(Xs, Ch, n_threads=threads)
    cpu_s = time.perf_counter() - t0
    same = bool(np.array_equal(lab.cpu().numpy()[sample], lab_o))
    pairs = float(n) * k
    _emit({"metric": "minRMSD assignment frames/s", "value": n / (assign_ms / 1e3), "unit": "frames/s",
           "n_gpus": 1, "higher_is_better": True, "assign_ms": assign_ms,
           "pairs_per_s": pairs / (assign_ms / 1e3),
           "lloyd_ms_per_iter": lloyd_ms, "lloyd_frames_per_s": n / (lloyd_ms / 1e3), "steps": args.steps,
           "dtype": "f32 correlation sums (fused multiply-add), f64 QCP quartic",
           "labels_identical_to_oracle_on_sample": same,
           "cpu_baseline": {"value": len(sample) / cpu_s, "unit": "frames/s", "cores": threads, "kind": "port",
                            "sample": "20000 frames x k=100, oracle assign_minrmsd, %.1f s" % cpu_s},
           "config": {"workload": "minrmsd: 1,000,000 frames of 58 atoms (d=174), noisy rotated and translated "
                                  "copies of 100 chain structures; k=100 centers drawn from the frames",
                      "data": "synthetic (seeded, generated on the device)"}})


def run_c4(args):
    """Precision sweep: 1M frames, d x k grid, fp32 vs fp16 tensor cores."""
    import torch
    from pyemma_gb300 import _lib
    _lib.load()
    n = 1_000_000
    rows = []
    for d in (16, 64, 256, 1024):
        for k in (100, 1000, 5000):
            g = torch.Generator(device="cuda")
            g.manual_seed(SEED + 31 * d + k)
            means = (torch.rand((4 * k, d), device="cuda", generator=g) * 10.0 - 5.0)
            comp = torch.randint(0, 4 * k, (n,), device="cuda", generator=g)
            X = (means[comp] + 0.3 * torch.randn((n, d), device="cuda", generator=g)).contiguous()
            del means, comp
            C0 = X[torch.randperm(n, device="cuda", generator=g)[:k]].contiguous()
            row = {"d": d, "k": k}
            steps = 2
            for prec in ("fp32", "fp16", "bf16", "fp8"):
                try:
                    ms, prof = _lloyd_rate(torch, _lib, X, C0, steps, prec)
                    row[prec + "_ms_per_iter"] = ms
                except _lib.KmError as e:
                    row[prec + "_ms_per_iter"] = None
                    row[prec + "_error"] = str(e)
            if row.get("fp16_ms_per_iter") and row.get("fp32_ms_per_iter"):
                row["speedup"] = row["fp32_ms_per_iter"] / row["fp16_ms_per_iter"]
                lab16, st = _lib.assign(X, C0, precision="fp16")
                lab32, _ = _lib.assign(X, C0, precision="fp32")
                row["recheck_fraction"] = (st["n_recheck"] + st["n_full"]) / float(n)
                row["full_recheck_fraction"] = st["n_full"] / float(n)
                row["labels_identical"] = bool(torch.equal(lab16, lab32))
                row["tflops_fp16_iter"] = 2.0 * n * k * d / (row["fp16_ms_per_iter"] / 1e3) / 1e12
                for other in ("bf16", "fp8"):
                    if row.get(other + "_ms_per_iter"):
                        labb, stb = _lib.assign(X, C0, precision=other)
                        row[other + "_recheck_fraction"] = (stb["n_recheck"] + stb["n_full"]) / float(n)
                        row[other + "_full_recheck_fraction"] = stb["n_full"] / float(n)
                        row[other + "_labels_identical"] = bool(torch.equal(labb, lab32))
                        del labb
                tt = tile_tuning(torch, _lib, X, C0, steps)
                row["tile_tuning"] = {key: tt[key] for key in ("fixed_plan", "fixed_ms_per_iter", "tuned_plan",
                                                               "tuned_ms_per_iter", "speedup", "labels_identical")}
            rows.append(row)
            del X, C0
            torch.cuda.empty_cache()
    _emit({"metric": "Lloyd iteration time per precision (precision sweep)", "unit": "ms", "n_gpus": 1,
           "higher_is_better": False,
           "config": {"workload": "c4: 1,000,000 frames, 4k Gaussian clusters (sigma 0.3, means U[-5,5]^d), "
                                  "d in {16,64,256,1024}, k in {100,1000,5000}; fp32 exact vs fp16, bf16 and fp8 "
                                  "(e4m3, per-frame scales) tensor cores with exact recheck"},
           "rows": rows})


def run_c5(args):
    """Serving: Poisson arrivals against 8 resident center sets."""
    import torch
    from pyemma_gb300 import _lib, datasets
    _lib.load()
    rng = np.random.default_rng(SEED)
    specs = [(2, 100), (2, 500), (10, 1000), (10, 5000), (528, 500), (528, 1000), (528, 2000), (528, 5000)]
    pool_n = {2: 2_000_000, 10: 2_000_000, 528: 1_000_000}
    pools = {}
    src = {2: datasets.gaussian_mixture(pool_n[2], 2, 10, 0.5, 5.0, SEED),
           10: np.concatenate(datasets.metastable_trajectories(n_traj=12, d=10, lmin=150_000, lmax=300_000,
                                                               seed=SEED))[:pool_n[10]]}
    for d, a in src.items():
        pool_n[d] = len(a)
        t = torch.empty(a.shape, dtype=torch.float32, pin_memory=True)
        t.numpy()[...] = a
        pools[d] = t
    Xd528 = datasets.calpha_distances(n_frames=pool_n[528], seed=SEED, device="cuda")
    pools[528] = torch.empty(tuple(Xd528.shape), dtype=torch.float32, pin_memory=True)
    pools[528].copy_(Xd528)
    srv = _lib.Server(hbm_budget_bytes=40 << 30)
    sets = []
    for d, k in specs:
        if d == 528:
            C = Xd528[torch.from_numpy(rng.choice(pool_n[d], k, replace=False)).cuda()].contiguous()
        else:
            C = torch.from_numpy(pools[d].numpy()[rng.choice(pool_n[d], k, replace=False)]).cuda()
        cs = _lib.Centers(C, precision="auto")
        sets.append((srv.add_centers(cs), cs, d, k))
    del Xd528
    torch.cuda.empty_cache()
    # schedule
    rate, dur = 200.0, float(args.serve_seconds)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=int(rate * dur * 2)))
    arrivals = arrivals[arrivals < dur]
    m = len(arrivals)
    lengths = np.exp(rng.uniform(np.log(1e3), np.log(1e6), size=m)).astype(np.int64)
    which = rng.integers(0, len(specs), size=m)
    starts = [int(rng.integers(0, pool_n[specs[w][0]] - L + 1)) for w, L in zip(which, lengths)]
    total = int(lengths.sum())
    arena_t = torch.empty(total, dtype=torch.int32, pin_memory=True)
    arena = arena_t.numpy()
    offs = np.concatenate([[0], np.cumsum(lengths)])
    # warm-up: three host-to-device passes over every pinned pool (the first
    # passes over freshly pinned memory run slower; a production server's
    # buffers are warm), then one small request per set
    h2d_gbs = None
    for d in pools:
        tmp = torch.empty(tuple(pools[d].shape), dtype=torch.float32, device="cuda")
        for _ in range(3):
            tmp.copy_(pools[d], non_blocking=True)
        torch.cuda.synchronize()
        if d == 528:
            # this process's pinned host-to-device rate, for reading the latencies
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            tmp.copy_(pools[d], non_blocking=True)
            e1.record()
            torch.cuda.synchronize()
            h2d_gbs = pools[d].numel() * 4 / (e0.elapsed_time(e1) / 1e3) / 1e9
        del tmp
    tmp = torch.zeros(total, dtype=torch.int32, device="cuda")  # and over the label arena, device to host
    for _ in range(3):
        arena_t.copy_(tmp, non_blocking=True)
    torch.cuda.synchronize()
    del tmp
    torch.cuda.empty_cache()
    for sid, cs, d, k in sets:
        t, _ = srv.submit(sid, pools[d].numpy()[:4096])
        srv.poll(t)
    infos = [None] * m
    tickets = [None] * m

    def poller():
        for i in range(m):
            while tickets[i] is None:
                time.sleep(0.0002)
            infos[i] = srv.poll(tickets[i])

    th = threading.Thread(target=poller)
    th.start()
    t0 = time.perf_counter()
    for i in range(m):
        now = time.perf_counter() - t0
        if arrivals[i] > now:
            time.sleep(arrivals[i] - now)
        sid, cs, d, k = sets[which[i]]
        Xr = pools[d].numpy()[starts[i]:starts[i] + lengths[i]]
        tickets[i] = srv.submit(sid, Xr, arena[offs[i]:offs[i + 1]])[0]
    th.join()
    t_end = time.perf_counter() - t0
    lat = np.array([x["total_ms"] for x in infos])
    qlat = np.array([x["queue_ms"] for x in infos])
    st = srv.stats()
    # the same requests alone (one per set, first occurrence) against the mixed results
    same = True
    checked = 0
    for w in range(len(specs)):
        idx = np.nonzero(which == w)[0]
        if len(idx) == 0:
            continue
        i = int(idx[0])
        sid, cs, d, k = sets[w]
        Xr = pools[d].numpy()[starts[i]:starts[i] + lengths[i]]
        alone, _ = cs.assign(torch.from_numpy(np.ascontiguousarray(Xr)).cuda())
        same &= bool(np.array_equal(alone.cpu().numpy(), arena[offs[i]:offs[i + 1]]))
        checked += 1
    srv.shutdown()
    flops = sum(2.0 * L * specs[w][1] * specs[w][0] for w, L in zip(which, lengths))
    per_d = {}
    for dd in (2, 10, 528):
        sel = np.array([specs[w][0] == dd for w in which])
        if sel.any():
            per_d[str(dd)] = {"requests": int(sel.sum()), "p50_ms": float(np.percentile(lat[sel], 50)),
                              "p99_ms": float(np.percentile(lat[sel], 99))}
    per_size = {}
    for name, lo_, hi_ in (("<10k", 0, 10_000), ("10k-100k", 10_000, 100_000), (">=100k", 100_000, 1 << 62)):
        sel = (lengths >= lo_) & (lengths < hi_)
        if sel.any():
            per_size[name] = {"requests": int(sel.sum()), "p50_ms": float(np.percentile(lat[sel], 50)),
                              "p99_ms": float(np.percentile(lat[sel], 99)),
                              "queue_p99_ms": float(np.percentile(qlat[sel], 99))}
    _emit({"metric": "serving frames/s with p50/p99 request latency", "value": total / t_end, "unit": "frames/s",
           "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
           "max_ms": float(lat.max()), "queue_p99_ms": float(np.percentile(qlat, 99)), "n_gpus": 1,
           "requests": m, "frames": total, "offered_frames_per_s": total / dur,
           "offered_tflops": flops / dur / 1e12, "wall_s": t_end, "server": st,
           "labels_same_alone_and_mixed": same, "checked_requests": checked, "per_d": per_d,
           "per_request_frames": per_size, "h2d_gbs_pinned_pool": h2d_gbs,
           "config": {"workload": "c5: Poisson arrivals at %.0f req/s for %.0f s, lengths log-uniform [1k, 1M], "
                                  "8 resident center sets (d, k) = %s, 40 GB admission budget, pinned host "
                                  "buffers, copies included" % (rate, dur, specs)}})


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.config == "c1":
        run_c1(args)
    elif args.config == "c2":
        run_c2(args)
    elif args.config == "minrmsd":
        run_minrmsd(args)
    elif args.config == "c4":
        run_c4(args)
    elif args.config == "c5":
        run_c5(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
