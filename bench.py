#!/usr/bin/env python
"""Benchmark: exact LOF fit_predict at n=200,000, d=8, k=20 (contamination 0.01).

One step = one LOF(n_neighbors=20, contamination=0.01).fit_predict of the whole
synthetic data set (5 Gaussian clusters + 1% uniform outliers, seed 1) through
the engine's C ABI: centre, norms, exact k-NN, LRD, scores, the contamination
offset and the labels.

* value: pair-distances per second, n^2 / t, with the input already in HBM;
  t is the CUDA-event time of one step on the launching stream; L2 (129 MB)
  is flushed with a 256 MiB write between steps, outside the timed events.
* e2e: the same metric through culof_context_fit_predict with pinned host
  buffers: host->device copy of X, the pipeline and the device->host copy of
  nof + labels + offset, every step (wall time of the synchronous call).
* roofline: the distance sweep kernel (the dominant kernel): the algorithmic
  work, 2d FLOP for each of the n (n - 640) pairs outside the rows' seed
  windows (the own tile and its four nearest Morton neighbour tiles, which
  the seed kernel covers; one evaluation per pair), over its event time,
  against the measured FP32 FMA peak. The kernel skips column tiles that a bounding-box test proves
  farther than every k-th neighbour; the pairs it actually evaluated, the
  pruned fraction and its FLOP rate on the evaluated pairs are reported
  beside it (executed_tflops, executed_frac).
* cpu_baseline: one whole fit_predict of the same workload (centre, exact
  k-NN of all n rows, LRD, scores, offset, labels) by the CPU oracle, a C
  restatement of the same exact algorithm, on all host threads.

``--impl reference`` times the reference's CPU implementation of this path
instead: whole fit_predict steps of the CPU port of its algorithm (oracle/),
on all host threads, the mean of the timed steps. The reference's own CPU
comparison path (scikit-learn) is not on the GPU host and its CUDA build does
not run there. That arm never loads the engine's library: the workload
generator is loaded by path.

Under torchrun with N > 1 every rank runs an independent replica on its own
GPU (no collective on the data path); value sums the ranks' work over the
slowest rank's time.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L2_FLUSH_BYTES = 256 << 20


PATH_NAMES = ["auto", "fast", "general", "tensor"]

# DRAM traffic of one sweep_kernel launch, measured by one ncu capture of this
# very workload (dram__bytes_read.sum + dram__bytes_write.sum); other
# workloads report null.
MEASURED_SWEEP_TRAFFIC = {
    ("clusters", 200_000, 8, 20): (16_110_000 + 10_360_000,
                                   "ncu: 16.11 MB read + 10.36 MB written per sweep_kernel launch at this workload "
                                   "(the isolated rows' pass beside it: 7.79 MB read)"),
}


def tensor_peak():
    """Dense 16-bit tensor peak: the measured cuBLAS bf16 burst figure (f16
    runs at the same rate) when present, else the fallback figure."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"]), "of measured: cuBLAS bf16 burst (MEASURED_PEAKS.json)"
    except (OSError, KeyError, ValueError):
        return 1900.0, "of fallback: 1.9 PFLOP/s bf16 burst"


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=30)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--n", type=int, default=200_000)
    p.add_argument("--d", type=int, default=8)
    p.add_argument("--k", type=int, default=20)
    p.add_argument("--contamination", type=float, default=0.01)
    p.add_argument("--seed", type=int, default=1)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--path", choices=["auto", "fast", "general", "tensor"], default="auto")
    p.add_argument("--suite", action="store_true",
                   help="report harness: one JSON line per benchmark workload (five) with an agreement gate")
    p.add_argument("--batched", type=int, default=0, metavar="N",
                   help="the batched problem mix (d = 16, k 10-40, n log-uniform in [128, 16384]) with N problems, "
                        "batched call against single calls")
    p.add_argument("--autotune-table", action="store_true",
                   help="the batched autotuner's variant times and choice for a grid of batch layouts")
    p.add_argument("--backward", action="store_true",
                   help="the gradient workload alone (mixture, --n/--d/--k): forward + sparse backward timing")
    p.add_argument("--scaling", action="store_true",
                   help="the reference benchmark's n and d sweeps through culof_gb300.lof, gated bit-exact on the oracle")
    p.add_argument("--workload", choices=["clusters", "factor", "mixture"], default="clusters",
                   help="clusters: 5 clusters + 1%% outliers; factor: rank-16 factor model + 5.0 shift + 0.5%% noisy "
                        "rows; mixture: 8 clusters + 1%% outliers")
    return p.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def load_synthetic():
    """culof_gb300/synthetic.py by path (numpy only): importing the package
    would load the engine's library, which the CPU arm must not touch."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("culof_gb300_synthetic",
                                                  os.path.join(ROOT, "culof_gb300", "synthetic.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def workload(args):
    synthetic = load_synthetic()
    if args.workload == "factor":
        return synthetic.factor_model(args.n, args.d, seed=args.seed)
    if args.workload == "mixture":
        return synthetic.gradient_mixture(args.n, args.d, seed=args.seed)
    return synthetic.clusters_with_outliers(args.n, args.d, seed=args.seed)


GENERATORS = {
    "clusters": "5 isotropic Gaussian clusters (centres U[-10,10]^d, sigma U[0.5,2]) + 1% U[-15,15]^d",
    "factor": "rank-16 Gaussian factor model (loadings N(0,1/16)) + N(0,0.1^2) noise + 5.0 shift, 0.5% rows + U[-3,3]^d",
    "mixture": "8 Gaussian clusters (centres U[-8,8]^d, sigma U[0.5,1.5]) + 1% U[-12,12]^d",
}


def config_dict(args, extra=None):
    cfg = {
        "workload": f"exact LOF fit_predict n={args.n} d={args.d} k={args.k} contamination={args.contamination}",
        "n": args.n,
        "d": args.d,
        "k": args.k,
        "contamination": args.contamination,
        "generator": GENERATORS[args.workload] + ", seed " + str(args.seed),
        "l2": "256 MiB write between timed steps, outside the events (X is 6.4 MB < L2)",
        "parallelism": "replicas" if int(os.environ.get("WORLD_SIZE", "1")) > 1 else "single GPU",
    }
    if extra:
        cfg.update(extra)
    return cfg


# ----------------------------------------------------------------- clocks


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = (
        "timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
        "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
        "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"
    )

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"],
                stdout=self.file, stderr=subprocess.DEVNULL,
            )
        except (OSError, FileNotFoundError):
            self.proc = None

    def window(self, t0: float, t1: float):
        self.t0, self.t1 = t0, t1

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        self.file.seek(0)
        rows = [r.split(",") for r in self.file.read().strip().splitlines() if r.strip()]
        os.unlink(self.file.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        t0, t1 = getattr(self, "t0", None), getattr(self, "t1", None)

        def in_window(stamp: str) -> bool:
            if t0 is None:
                return True
            try:
                import datetime

                ts = datetime.datetime.strptime(stamp.strip(), "%Y/%m/%d %H:%M:%S.%f").timestamp()
            except ValueError:
                return True
            return t0 - 0.25 <= ts <= t1 + 0.25

        rows_in = [r for r in rows if r and in_window(r[0])] or rows
        for r in rows_in:
            r = r[1:]
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() in ("active", "1"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(mx) if mx else None,
            "reasons": sorted(reasons),
            "samples": len(sm),
        }


# ----------------------------------------------------------------- CPU legs


def cpu_fit_predict_s(args, X) -> float:
    """Wall time of one whole fit_predict by the CPU oracle on all host threads."""
    import oracle

    oracle.build()
    t0 = time.perf_counter()
    oracle.fit_predict(X, args.k, args.contamination)
    return time.perf_counter() - t0


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    import oracle

    oracle.build()
    X = workload(args)
    n = X.shape[0]
    cores = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_fit_predict_s(args, X)
    step_s = [cpu_fit_predict_s(args, X) for _ in range(args.steps)]
    mean_s = statistics.mean(step_s)
    value = float(n) * n / mean_s
    line = {
        "impl": "reference",
        "metric": "pair-dists/s",
        "value": value,
        "unit": "pair-dists/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": mean_s * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": config_dict(args),
        "fit_predict_s": mean_s,
        "cpu_baseline": {
            "value": value,
            "unit": "pair-dists/s",
            "cores": cores,
            "kind": "port",
            "sample": f"every step one whole fit_predict of all {n} rows (centre, exact k-NN, LRD, scores, offset, "
            f"labels) by the C port of the reference algorithm on {cores} threads; mean of {args.steps} timed "
            "steps. The reference's CPU comparison path (scikit-learn) is not installed on the GPU host and its "
            "CUDA build cannot run there",
        },
        "e2e": {"value": value, "unit": "pair-dists/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------- GPU leg


def run_ours(args):
    import torch

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from culof_gb300 import _culof

    X = workload(args)
    n, d, k, c = X.shape[0], X.shape[1], args.k, args.contamination
    pairs = float(n) * float(n)
    stream = torch.cuda.Stream()
    ctx = _culof.Context()
    ctx.set_stream(stream.cuda_stream)
    ctx.set_path({"auto": 0, "fast": 1, "general": 2, "tensor": 3}[args.path])
    ctx.set_timing(True)

    with torch.cuda.stream(stream):
        dX = torch.from_numpy(X).cuda()
        d_nof = torch.empty(n, dtype=torch.float32, device="cuda")
        d_lab = torch.empty(n, dtype=torch.int64, device="cuda")
        d_off = torch.empty(1, dtype=torch.float64, device="cuda")
        flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    stream.synchronize()

    def step():
        ctx.fit_predict_device(dX.data_ptr(), n, d, k, False, c, d_nof.data_ptr(), d_lab.data_ptr(), d_off.data_ptr())

    for _ in range(args.warmup):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        step()
    ctx.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(1.0)  # nvidia-smi start-up, so samples cover the timed region
    barrier()
    wall0 = time.time()
    launches0 = _culof.kernel_launch_count()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    stage_acc = {}
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(i))
        starts[i].record(stream)
        step()
        ends[i].record(stream)
        for name, ms in ctx.stage_times().items():  # synchronises; outside the events
            stage_acc.setdefault(name, []).append(ms)
        ev_pairs, unpruned_pairs = ctx.pair_stats()
    barrier()
    sampler.window(wall0, time.time())
    launches = _culof.kernel_launch_count() - launches0
    ctx.synchronize()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    mean_ms = statistics.mean(step_ms)
    clocks = sampler.stop()

    # e2e through the C ABI with pinned host buffers (copies inside the region)
    hX = torch.from_numpy(X).pin_memory()
    h_nof = torch.empty(n, dtype=torch.float32).pin_memory()
    h_lab = torch.empty(n, dtype=torch.int64).pin_memory()
    h_off = torch.empty(1, dtype=torch.float64).pin_memory()

    def e2e_step():
        ctx.fit_predict_host_ptr(hX.data_ptr(), n, d, k, False, c, h_nof.data_ptr(), h_lab.data_ptr(), h_off.data_ptr())

    for _ in range(max(1, args.warmup)):
        e2e_step()
    e2e_ms = []
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(i))
        stream.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_mean = statistics.mean(e2e_ms)

    # parity guard on the benchmarked output: labels agree with the offset
    nof = d_nof.cpu().numpy()
    lab = d_lab.cpu().numpy()
    off = float(d_off.item())
    assert np.array_equal(lab, np.where(nof < np.float32(off), -1, 1)), "labels disagree with offset"
    assert np.array_equal(h_nof.numpy(), nof) and float(h_off.item()) == off, "e2e output differs"

    if world > 1:
        t = torch.tensor([mean_ms, e2e_mean], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        mean_ms, e2e_mean = float(t[0]), float(t[1])
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return 0

    stages = {name: statistics.mean(v) for name, v in stage_acc.items()}
    fp32_peak = max(_culof.probe_fp32_tflops(True), _culof.probe_fp32_tflops(False))
    # the sweep evaluates every pair outside the rows' seed window: the own
    # 128-point tile (tensor and wide paths), or the own tile and its four
    # nearest Morton neighbour tiles (small-d path, d <= 8)
    nt = (n + 127) // 128
    window = min(nt, 5) if (ctx.last_path() == _culof.PATH_FAST and d <= 8) else 1
    sweep_pairs = float(n) * float(n - min(n, 128 * window)) if nt > window else 0.0
    sweep_ms = stages.get("sweep")
    roofline = None
    if sweep_ms and sweep_pairs > 0 and ctx.last_path() == _culof.PATH_TENSOR:
        # the f16 Gram of every pair on the tensor cores (K = d padded to 64/128)
        kp = 64 if d <= 64 else 128
        peak, peak_src = tensor_peak()
        achieved = 2.0 * kp * sweep_pairs / (sweep_ms * 1e-3) / 1e12
        roofline = {
            "bound": "tensor",
            "kernel": "tc_sweep_kernel (f16 tcgen05 Gram filter + exact FP32 rescoring)",
            "achieved": achieved,
            "peak": peak,
            "unit": "TFLOP/s",
            "frac": achieved / peak,
            "traffic": None,
            "peak_source": peak_src,
            "algorithmic_flop_per_pair": 2 * kp,
            "pairs_per_launch": sweep_pairs,
            "sweep_share_of_step": sweep_ms / mean_ms,
        }
    elif sweep_ms and sweep_pairs > 0 and ctx.last_path() == _culof.PATH_FAST:
        # algorithmic work: 2d FLOP for every pair past the row's seed window
        # (one evaluation per pair); the kernel itself evaluates only the
        # pairs of column tiles a bounding-box test cannot rule out, and its
        # efficiency on those is reported beside it
        achieved = 2.0 * d * sweep_pairs / (sweep_ms * 1e-3) / 1e12
        executed = 2.0 * d * (ev_pairs if unpruned_pairs > 0 else sweep_pairs) / (sweep_ms * 1e-3) / 1e12
        traffic, traffic_src = MEASURED_SWEEP_TRAFFIC.get((args.workload, n, d, k), (None, None))
        roofline = {
            "bound": "fp32",
            "kernel": "sweep_kernel (fused distance + filtered exact select)",
            "achieved": achieved,
            "peak": fp32_peak,
            "unit": "TFLOP/s",
            "frac": achieved / fp32_peak,
            "traffic": traffic,
            "peak_source": "measured FP32 FMA throughput (culof_probe_fp32_tflops, best of scalar/packed)",
            "algorithmic_flop_per_pair": 2 * d,
            "pairs_per_launch": sweep_pairs,
            "evaluated_pairs_per_launch": ev_pairs if unpruned_pairs > 0 else sweep_pairs,
            "pruned_fraction": (1.0 - ev_pairs / unpruned_pairs) if unpruned_pairs > 0 else 0.0,
            "executed_tflops": executed,
            "executed_frac": executed / fp32_peak,
            "traffic_source": traffic_src,
            "sweep_share_of_step": sweep_ms / mean_ms,
        }
    cpu = None
    if not args.no_cpu_baseline:
        dt = cpu_fit_predict_s(args, X)
        cpu = {
            "value": pairs / dt,
            "unit": "pair-dists/s",
            "cores": os.cpu_count() or 1,
            "kind": "port",
            "sample": f"one whole fit_predict of all {n} rows ({dt:.2f} s): the C port of the same algorithm",
        }
    value = world * pairs / (mean_ms * 1e-3)
    line = {
        "metric": "pair-dists/s",
        "value": value,
        "unit": "pair-dists/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": mean_ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": config_dict(args),
        "path": PATH_NAMES[ctx.last_path()],
        "fit_predict_s": mean_ms * 1e-3,
        "e2e": {
            "value": world * pairs / (e2e_mean * 1e-3),
            "unit": "pair-dists/s",
            "fit_predict_s": e2e_mean * 1e-3,
            "h2d_bytes_per_step": int(X.nbytes),
            "d2h_bytes_per_step": int(n * 4 + n * 8 + 8),
        },
        "roofline": roofline,
        "cpu_baseline": cpu,
        "clocks": clocks,
        "gpu_launches": int(launches),
        "stages_ms": stages,
        "device": _culof.device_info(),
        "published_reference": {"lof_s_n200000_d8_k20": 1.409, "hardware": "RTX A6000", "source": "README.md:50"},
    }
    print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


# ----------------------------------------------------------------- report suite


def _time_calls(fn, stream, warm=2, reps=5):
    """Mean ms per call of fn (queued on stream), CUDA events around reps calls."""
    import torch

    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def batched_case(count, stream, emit, label, fp64=False):
    """The batched problem mix with `count` problems: one batched call (CUDA
    graph replay after the first call) against a loop of single calls, and
    the scores of both compared bit for bit."""
    import torch

    from culof_gb300 import _culof, synthetic

    probs, ks = synthetic.batched_problems(count, 16, seed=0)
    Xb = np.concatenate(probs).astype(np.float32)
    offs = np.zeros(len(probs) + 1, np.int64)
    offs[1:] = np.cumsum([len(p) for p in probs])
    ctx = _culof.Context()
    ctx.set_stream(stream.cuda_stream)
    dX = torch.from_numpy(Xb).cuda()
    ds = torch.empty(len(Xb), device="cuda")
    t0 = time.perf_counter()
    ctx.lof_batched_device(offs, ks, dX.data_ptr(), 16, False, ds.data_ptr())
    ctx.synchronize()
    first_s = time.perf_counter() - t0
    ms_b = _time_calls(lambda: ctx.lof_batched_device(offs, ks, dX.data_ptr(), 16, False, ds.data_ptr()), stream)
    dps = [dX[offs[i]:offs[i + 1]] for i in range(len(probs))]
    outs = torch.empty_like(ds)

    def loop():
        for i in range(len(probs)):
            ctx.lof_device(dps[i].data_ptr(), len(probs[i]), 16, ks[i], False, outs[offs[i]:offs[i + 1]].data_ptr())

    ms_l = _time_calls(loop, stream, warm=1, reps=2)
    scores = ds.cpu().numpy()
    same = bool(np.array_equal(scores.view(np.uint32), outs.cpu().numpy().view(np.uint32)))
    line = {"suite": label, "problems": len(probs), "points": int(offs[-1]), "d": 16,
            "pairs": float(sum(float(len(p)) ** 2 for p in probs)),
            "batched_s": ms_b * 1e-3, "loop_of_single_calls_s": ms_l * 1e-3, "speedup_vs_loop": ms_l / ms_b,
            "first_call_s_plan_autotune_capture": first_s,
            "agreement": {"bit_exact_vs_single_calls": same}}
    if fp64:
        import oracle

        # FP64 error over a seeded sample of up to 64 problems
        pick = np.sort(np.random.default_rng(64).choice(len(probs), min(64, len(probs)), replace=False))
        rel = []
        for i in pick:
            ref = oracle.lof_f64(probs[i], ks[i])
            rel.append(np.abs(scores[offs[i]:offs[i + 1]].astype(np.float64) - ref) / ref)
        rel = np.concatenate(rel)
        line["fp64_err"] = {"median": float(np.median(rel)), "p99": float(np.quantile(rel, 0.99)),
                            "max": float(rel.max()), "over": f"every score of {len(pick)} seeded problems"}
    emit(line)
    ctx.close()


def run_suite(args):
    """One JSON line per benchmark workload, each with its timing and an
    agreement gate against the oracle or an independent exact path (the
    speed and accuracy columns come from the same run)."""
    import torch

    import oracle
    from culof_gb300 import _culof, synthetic
    from oracle import backward as ob

    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    dev = _culof.device_info()

    def emit(line):
        line["device"] = dev
        print(json.dumps(line), flush=True)

    def fit_predict_case(name, X, k, c, path, rows_checked):
        n, d = X.shape
        ctx = _culof.Context()
        ctx.set_stream(stream.cuda_stream)
        ctx.set_path(path)
        dX = torch.from_numpy(X).cuda()
        nof = torch.empty(n, device="cuda")
        lab = torch.empty(n, dtype=torch.int64, device="cuda")
        off = torch.empty(1, dtype=torch.float64, device="cuda")
        ms = _time_calls(lambda: ctx.fit_predict_device(dX.data_ptr(), n, d, k, False, c, nof.data_ptr(),
                                                        lab.data_ptr(), off.data_ptr()), stream)
        # k-NN of a seeded block of rows against the oracle, bit for bit
        idx = torch.empty((k, n), dtype=torch.int32, device="cuda")
        d2 = torch.empty((k, n), device="cuda")
        kd = torch.empty(n, device="cuda")
        ctx.knn_device(dX.data_ptr(), n, d, k, False, idx.data_ptr(), d2.data_ptr(), kd.data_ptr())
        ctx.synchronize()
        b = int(np.random.default_rng(n).integers(0, n - rows_checked + 1))
        Xc, _, _ = oracle.center(X)
        t0 = time.perf_counter()
        oi, od, ok = oracle.knn(Xc, k, rows=(b, b + rows_checked))
        cpu_s = time.perf_counter() - t0
        gi, gd, gk = idx.cpu().numpy(), d2.cpu().numpy(), kd.cpu().numpy()
        agree = bool(np.array_equal(gi[:, b:b + rows_checked], oi[:, b:b + rows_checked])
                     and np.array_equal(gd[:, b:b + rows_checked].view(np.uint32), od[:, b:b + rows_checked].view(np.uint32))
                     and np.array_equal(gk[b:b + rows_checked].view(np.uint32), ok[b:b + rows_checked].view(np.uint32)))
        res = {"suite": name, "n": n, "d": d, "k": k, "path": PATH_NAMES[ctx.last_path()],
               "fit_predict_s": ms * 1e-3, "pair_dists_per_s": float(n) * n / (ms * 1e-3),
               "agreement": {"knn_rows_checked": rows_checked, "bit_exact_vs_oracle": agree},
               "cpu_oracle_knn_rows_per_s": rows_checked / cpu_s}
        ctx.close()
        return res, nof.cpu().numpy()

    # clusters, d = 8, k = 20, c = 0.01, at n = 20k and 200k; the scores'
    # relative error against the FP64 brute force of all n points
    for name, n in (("clusters_n20000_d8_k20", 20_000), ("clusters_n200000_d8_k20", 200_000)):
        X = synthetic.clusters_with_outliers(n, 8, seed=1)
        res, nof = fit_predict_case(name, X, 20, 0.01, 0, 2000)
        res["fp64_err"] = dict(oracle.fp64_error(-nof, X, 20), over=f"all {n} scores")
        emit(res)
    # factor model, n = 200k, d = 128, k = 50: tensor path against the FP32
    # sweep; FP64 error of the LOF of a seeded 5,000-row subsample
    X = synthetic.factor_model(200_000, 128, seed=1)
    tres, tnof = fit_predict_case("factor_n200000_d128_k50", X, 50, 0.01, 3, 500)
    fres, fnof = fit_predict_case("factor_n200000_d128_k50_fp32", X, 50, 0.01, 1, 1)
    tres["fp32_fit_predict_s"] = fres["fit_predict_s"]
    tres["speedup_vs_fp32"] = fres["fit_predict_s"] / tres["fit_predict_s"]
    tres["agreement"]["nof_bit_exact_vs_fp32_path"] = bool(np.array_equal(tnof.view(np.uint32), fnof.view(np.uint32)))
    Xs = np.ascontiguousarray(X[np.sort(np.random.default_rng(5000).choice(len(X), 5000, replace=False))])
    with _culof.Context() as ctx:
        ctx.set_path(_culof.PATH_TENSOR)
        s_sub = ctx.lof(Xs, 50)
    tres["fp64_err"] = dict(oracle.fp64_error(s_sub, Xs, 50), over="LOF of a seeded 5,000-row subsample")
    emit(tres)
    # sparse backward, mixture, n = 50,000, d = 32, k = 20
    from culof_gb300.autograd import lof_scores

    X = synthetic.gradient_mixture(50_000, 32, seed=1)
    w = torch.from_numpy(np.random.default_rng(3).standard_normal(len(X))).cuda()
    Xt = torch.from_numpy(X).cuda()

    def fwd_bwd():
        Xg = Xt.clone().requires_grad_(True)
        (lof_scores(Xg, 20).double() * w).sum().backward()
        return Xg.grad

    ms_fb = _time_calls(fwd_bwd, stream)
    ms_f = _time_calls(lambda: lof_scores(Xt, 20), stream)
    g = fwd_bwd().double()
    with _culof.Context() as ctx:
        idx = torch.empty((20, len(X)), dtype=torch.int32, device="cuda")
        d2 = torch.empty((20, len(X)), device="cuda")
        kd = torch.empty(len(X), device="cuda")
        ctx.knn_device(Xt.data_ptr(), len(X), 32, 20, False, idx.data_ptr(), d2.data_ptr(), kd.data_ptr())
        ctx.synchronize()
    X64 = Xt.double().requires_grad_(True)
    (ob.lof_fixed(X64, idx.long(), False) * w).sum().backward()
    rel = float((g - X64.grad).abs().max() / X64.grad.abs().max())
    fwd = lof_scores(Xt, 20).cpu().numpy()
    emit({"suite": "mixture_n50000_d32_k20_backward", "n": len(X), "d": 32, "k": 20, "forward_s": ms_f * 1e-3,
          "backward_s": (ms_fb - ms_f) * 1e-3, "forward_backward_s": ms_fb * 1e-3,
          "agreement": {"grad_max_rel_err_vs_fp64_autograd": rel, "float32_result": True},
          "fp64_err": dict(oracle.fp64_error(fwd, X, 20), over="all 50000 forward scores")})
    # 2,048 problems in one batched call against a loop of single calls
    batched_case(2048, stream, emit, "batched_2048_problems_d16", fp64=True)
    return 0


def run_scaling(args):
    """The reference benchmark's two sweeps (benchmarks/benchmark.py:187-205):
    sample count n in {1k .. 200k} at d = 8, and dimensionality d in
    {2, 8, 32, 128} at n = 20k, k = 20. Each row times the public host API
    `culof_gb300.lof(X, k)` (fastest of 5 calls after one warm-up, wall clock,
    host copies included, as benchmark.py:69-84 times `culof.lof`) and the
    oracle on all host cores (one call), and gates on the scores: bit-exact
    against the oracle, and the top-1% rank sets identical
    (benchmark.py:101-116 allows 5% relative error against scikit-learn)."""
    import torch

    import culof_gb300
    import oracle
    from culof_gb300 import synthetic

    torch.cuda.set_device(0)
    culof_gb300.lof(synthetic.clusters_with_outliers(1000, 8, seed=0), 20)  # context init, excluded
    rows = [("samples", n, 8) for n in (1_000, 2_000, 5_000, 10_000, 20_000, 50_000, 100_000, 200_000)]
    rows += [("features", 20_000, d) for d in (2, 8, 32, 128)]
    k = args.k
    failed = False
    for sweep, n, d in rows:
        X = synthetic.clusters_with_outliers(n, d, seed=args.seed)
        culof_gb300.lof(X, k)
        best = float("inf")
        for _ in range(5):
            t0 = time.perf_counter()
            s_gpu = culof_gb300.lof(X, k)
            best = min(best, time.perf_counter() - t0)
        t0 = time.perf_counter()
        s_cpu = oracle.lof(X, k)
        t_cpu = time.perf_counter() - t0
        rel = float(np.max(np.abs(s_gpu.astype(np.float64) - s_cpu) / np.maximum(np.abs(s_cpu), 1e-9)))
        top = max(1, n // 100)
        agree = len(set(np.argsort(-s_gpu, kind="stable")[:top]) & set(np.argsort(-s_cpu, kind="stable")[:top])) / top
        exact = bool(np.array_equal(s_gpu.view(np.uint32), np.asarray(s_cpu, np.float32).view(np.uint32)))
        failed |= not exact or agree < 1.0
        print(json.dumps({"scaling": sweep, "n": n, "d": d, "k": k, "lof_s": best,
                          "pair_dists_per_s": float(n) * n / best, "oracle_s": t_cpu,
                          "oracle_threads": os.cpu_count(), "speedup_vs_oracle": t_cpu / best,
                          "max_rel_err": rel, "rank_agreement": agree, "bit_exact_vs_oracle": exact}), flush=True)
    return 1 if failed else 0


def run_batched(args):
    """The batched problem mix alone, with --batched problems (a small count
    keeps an ncu capture of the batched kernel short)."""
    import torch

    from culof_gb300 import _culof

    torch.cuda.set_device(0)
    dev = _culof.device_info()

    def emit(line):
        line["device"] = dev
        print(json.dumps(line), flush=True)

    batched_case(args.batched, torch.cuda.current_stream(), emit, "batched")
    return 0


def run_backward(args):
    """The gradient workload alone (8-cluster mixture, --n points, --d dims,
    --k neighbours): forward and sparse backward of sum_i w_i LOF_i through
    the autograd function, timed with CUDA events, the gradient compared with
    FP64 autograd of the same fixed-neighbour LOF."""
    import torch

    from culof_gb300 import _culof
    from culof_gb300.autograd import lof_scores
    from oracle import backward as ob

    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    X = load_synthetic().gradient_mixture(args.n, args.d, seed=args.seed)
    w = torch.from_numpy(np.random.default_rng(3).standard_normal(len(X))).cuda()
    Xt = torch.from_numpy(X).cuda()

    def fwd_bwd():
        Xg = Xt.clone().requires_grad_(True)
        (lof_scores(Xg, args.k).double() * w).sum().backward()
        return Xg.grad

    ms_fb = _time_calls(fwd_bwd, stream, warm=args.warmup, reps=args.steps)
    ms_f = _time_calls(lambda: lof_scores(Xt, args.k), stream, warm=args.warmup, reps=args.steps)
    g = fwd_bwd().double()
    with _culof.Context() as ctx:
        idx = torch.empty((args.k, len(X)), dtype=torch.int32, device="cuda")
        d2 = torch.empty((args.k, len(X)), device="cuda")
        kd = torch.empty(len(X), device="cuda")
        ctx.knn_device(Xt.data_ptr(), len(X), args.d, args.k, False, idx.data_ptr(), d2.data_ptr(), kd.data_ptr())
        ctx.synchronize()
    X64 = Xt.double().requires_grad_(True)
    (ob.lof_fixed(X64, idx.long(), False) * w).sum().backward()
    rel = float((g - X64.grad).abs().max() / X64.grad.abs().max())
    print(json.dumps({"workload": f"gradient mixture n={len(X)} d={args.d} k={args.k}", "forward_s": ms_f * 1e-3,
                      "backward_s": (ms_fb - ms_f) * 1e-3, "forward_backward_s": ms_fb * 1e-3,
                      "grad_max_rel_err_vs_fp64_autograd": rel, "device": _culof.device_info()}), flush=True)
    return 0


def run_autotune_table(args):
    """The batched autotuner's record per batch layout: the batched problem
    mix (3 clusters + 2% outliers per problem, n log-uniform in [128, 16384],
    k in 10..40) with several problem counts and dimensions; one line per
    layout with every variant's time and the variant chosen."""
    import torch

    from culof_gb300 import _culof

    torch.cuda.set_device(0)
    synthetic = load_synthetic()
    layouts = [(c, d) for d in (4, 8, 16) for c in (64, 256, 2048)] + [(c, d) for d in (32, 64) for c in (64, 256)]
    for count, d in layouts:
        probs, ks = synthetic.batched_problems(count, d, seed=0)
        Xb = np.concatenate(probs).astype(np.float32)
        offs = np.zeros(len(probs) + 1, np.int64)
        offs[1:] = np.cumsum([len(p) for p in probs])
        with _culof.Context() as ctx:
            dX = torch.from_numpy(Xb).cuda()
            ds = torch.empty(len(Xb), device="cuda")
            ctx.lof_batched_device(offs, ks, dX.data_ptr(), d, False, ds.data_ptr())
            ctx.synchronize()
            tune = ctx.batched_tuning()
        print(json.dumps({"problems": count, "points": int(offs[-1]), "d": d, **tune,
                          "device": _culof.device_info()}), flush=True)
    return 0


def main():
    args = parse_args()
    if args.autotune_table:
        return run_autotune_table(args)
    if args.suite:
        return run_suite(args)
    if args.batched:
        return run_batched(args)
    if args.backward:
        return run_backward(args)
    if args.scaling:
        return run_scaling(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
