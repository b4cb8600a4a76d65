#!/usr/bin/env python3
"""RI-MP2 energy benchmark (one JSON line on rank 0).

Workload: the synthetic RI-MP2 energy at nocc=40, nvir=360, naux=1200 with
B^Q_ia = G_Qia 0.05 exp(-Q/400), G ~ N(0,1), eps_occ ~ U[-1.5,-0.3],
eps_vir ~ U[0.05,3.0] (seeded, numpy PCG64).  A step is one full RI-MP2 energy
evaluation from the FP64 B tensor: slice pre-pass, fused tcgen05 energy kernel
and the FP64 reduction.  Throughput is the algorithmic count
F = 2 nocc^2 nvir^2 naux per step (the reference's full-(i,j) count,
src/POSTHF/can_mp2.cc:82-88) over the device time.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision split_fp16]
  python bench.py --impl reference ...   # the reference's CPU path on host cores

With N > 1 (torchrun, one rank per GPU) every rank runs an independent replica
of the workload; value = N * F * K / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = ("RI-MP2 time-to-E_corr & TFLOP/s, split-BF16 vs FP64 GPU at |ΔE|≤1 µEh")
NOCC, NVIR, NAUX, SEED = 40, 360, 1200, 2024
FLOPS = 2.0 * NOCC * NOCC * NVIR * NVIR * NAUX
WORKLOAD = (f"RI-MP2 energy nocc={NOCC} nvir={NVIR} naux={NAUX}; synthetic B = G diag(s_Q), "
            f"s_Q = 0.05 exp(-Q/400), seed {SEED}")
FALLBACK_PEAK_BF16 = 1900.0
L2_FLUSH_BYTES = 256 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="split_fp16",
                    choices=["split_fp16", "split_bf16", "fp64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-cluster", action="store_true",
                    help="leave the water-cluster time-to-E_corr block out of the line "
                         "(profiling runs of the energy kernel)")
    ap.add_argument("--batch-count", type=int, default=256,
                    help="instances of the batched workload (256 by default)")
    ap.add_argument("--workload", default="rimp2",
                    choices=["rimp2", "batch256", "ri_pipeline", "cluster", "dgemm_tc",
                             "adjoint"],
                    help="batch256: 256 uneven RI-MP2 instances in one batched launch; "
                         "ri_pipeline: time-to-E_corr from the 3-index integrals")
    ap.add_argument("--nbf", type=int, default=480, help="ri_pipeline: basis functions")
    ap.add_argument("--nocc", type=int, default=100, help="ri_pipeline: occupied orbitals")
    ap.add_argument("--naux", type=int, default=1520, help="ri_pipeline: auxiliary functions")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, gpu):
        self.rows = []
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "20", "-i", str(gpu)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def wait_first(self, timeout=20.0):
        """nvidia-smi start-up takes driver locks; let it finish before timing."""
        t0 = time.time()
        while self.proc is not None and not self.rows and time.time() - t0 < timeout:
            time.sleep(0.05)

    def mark(self):
        self.start_row = len(self.rows)

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        rows = self.rows[getattr(self, "start_row", 0):] or self.rows[-1:]
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": len(rows)}
        try:
            sm = [float(r[1]) for r in rows]
            mx = [float(r[2]) for r in rows]
            if sm:
                out["sm_mhz"] = statistics.median(sm)
                out["sm_max_mhz"] = max(mx)
            reasons = set()
            for r in rows:
                for k, name in enumerate(self.NAMES):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(name)
            out["reasons"] = sorted(reasons)
        except Exception:
            pass
        return out


# ---------------------------------------------------------------------------
# CPU baseline: the reference's algorithm on the host cores
# ---------------------------------------------------------------------------
def blas_threads():
    try:
        from threadpoolctl import threadpool_info

        n = [i.get("num_threads") for i in threadpool_info() if i.get("user_api") == "blas"]
        if n:
            return int(max(n))
    except Exception:
        pass
    return os.cpu_count() or 1


def cpu_energy_fn():
    """The reference's RI-MP2 energy on the host: its own compiled code
    (oracle/_ref) when present on this machine, else the oracle's restatement
    (same BLAS calls).  Returns (fn(B, eps, nocc, nvir), kind)."""
    from oracle import oracle as O

    try:
        from oracle import refwrap

        if os.path.exists(refwrap.SO):
            refwrap.lib()
            return refwrap.rimp2_energy, "reference"
    except Exception:
        pass
    return O.rimp2_energy, "port"


def cpu_sample(B, eps, nocc_s, min_seconds=10.0, max_reps=50):
    """Time the reference's RI-MP2 loop on the first nocc_s occupied orbitals
    (nocc_s^2 of the workload's nocc^2 pair GEMMs, same nvir and naux).
    Uses the reference's own compiled code (oracle/_ref) when it is present
    on this machine, else the oracle's restatement (same BLAS calls).
    Returns (tflops, kind, seconds, reps)."""
    import numpy as np

    from oracle import oracle as O

    fn, kind = cpu_energy_fn()
    Bs = np.ascontiguousarray(B[:, :nocc_s, :])
    es = np.concatenate([eps[:nocc_s], eps[NOCC:]])
    fn(Bs, es, nocc_s, NVIR)  # warm
    t0 = time.perf_counter()
    reps = 0
    while reps < max_reps:
        fn(Bs, es, nocc_s, NVIR)
        reps += 1
        if time.perf_counter() - t0 >= min_seconds:
            break
    dt = time.perf_counter() - t0
    f = 2.0 * nocc_s * nocc_s * NVIR * NVIR * NAUX * reps
    return f / dt / 1e12, kind, dt, reps


def read_traffic():
    """DRAM bytes per launch of the energy kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "energy_tc_o40v360x1200.md")
    try:
        for line in open(path):
            if line.strip().startswith("dram_bytes_per_launch"):
                return float(line.split("=")[1].split()[0])
    except Exception:
        pass
    return None


def read_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        return FALLBACK_PEAK_BF16, "fallback"


# ---------------------------------------------------------------------------
def run_reference(args):
    """The reference's RI-MP2 energy (can_mp2.cc:53-132) on the host cores:
    one full evaluation of the workload per step (all nocc^2 pair GEMMs)."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from corr_gb300 import workloads as W

    B, eps = W.synth_rimp2(NOCC, NVIR, NAUX, SEED)
    fn, kind = cpu_energy_fn()
    for _ in range(max(1, min(args.warmup, 2))):
        fn(B, eps, NOCC, NVIR)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        fn(B, eps, NOCC, NVIR)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    value = FLOPS * len(times) / tot / 1e12
    sample = (f"the full workload every step: all {NOCC * NOCC} pair GEMMs of nocc={NOCC}, "
              f"nvir={NVIR}, naux={NAUX}")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "TFLOP/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": tot / len(times) * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "precision": "fp64 (reference CPU path)",
                   "parallelism": "host cores"},
        "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": blas_threads(),
                         "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def time_to_ecorr_c3(ctx, reps=3):
    """RI-MP2 time-to-E_corr of the 20-water cluster (def2-SVP / def2-SVP-RI,
    N=480, nocc=100, naux=1520): its geometry and basis shells
    (tests/golden/systems.npz) and the MO coefficients and orbital energies of
    its RHF (tests/golden/config3_cluster.npz).  On the GPU: (P|Q) and
    (P|mu nu) (corr_ri_integrals), then the (P|ia) transform, RI metric,
    B = J^-1/2 (P|ia) and the energy (corr_rimp2_energy_from_3index) in each
    precision form against the FP64 form; the FP64 energy is compared with the
    reference's for the same orbitals (golden_molecules.json)."""
    import numpy as np
    import torch

    import corr_gb300

    gold = os.path.join(ROOT, "tests", "golden")
    sysd = np.load(os.path.join(gold, "systems.npz"))
    basis = [corr_gb300.Basis(*(sysd[f"c3_{k}_{n}"]
                                for n in ("l", "nprim", "poff", "center", "exps", "coefs")))
             for k in ("obs", "aux")]
    fx = np.load(os.path.join(gold, "config3_cluster.npz"))
    with open(os.path.join(gold, "golden_molecules.json")) as f:
        e_ref = json.load(f)["config3"]["ri_mp2"][2]
    mos = torch.from_numpy(fx["mos"]).cuda()
    eps = torch.from_numpy(fx["eps"]).cuda()
    nroe = 200
    ctx.ri_integrals(*basis)  # warm
    ts = []
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        J, P = ctx.ri_integrals(*basis)
        ts.append((time.perf_counter() - t0) * 1e3)
    t_int = statistics.median(ts)
    out = {"workload": "20-water cluster, def2-SVP/def2-SVP-RI (N=480, nocc=100, naux=1520), "
                       "RHF orbitals of tests/golden/config3_cluster.npz; integrals computed on the "
                       "GPU", "integrals_ms": t_int}
    e = {}
    for prec in ("split_fp16", "split_bf16", "fp64"):
        ctx.rimp2_energy_from_3index(nroe, mos, eps, J, P, prec)  # warm (sizes the workspace)
        ts = []
        for _ in range(reps if prec != "fp64" else 1):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r, ncut = ctx.rimp2_energy_from_3index(nroe, mos, eps, J, P, prec)
            ts.append((time.perf_counter() - t0) * 1e3)
        e[prec] = r.e_total
        out[f"{prec}_pipeline_ms"] = statistics.median(ts)
        out[f"{prec}_time_to_ecorr_ms"] = t_int + statistics.median(ts)
    for prec in ("split_fp16", "split_bf16"):
        out[f"{prec}_speedup_vs_fp64"] = out["fp64_pipeline_ms"] / out[f"{prec}_pipeline_ms"]
        out[f"{prec}_abs_dE_vs_fp64"] = abs(e[prec] - e["fp64"])
        out[f"{prec}_within_1uEh"] = abs(e[prec] - e["fp64"]) <= 1e-6
    out["e_fp64"] = e["fp64"]
    out["e_reference"] = e_ref
    out["abs_dE_fp64_vs_reference"] = abs(e["fp64"] - e_ref)
    out["metric_path"] = "cholesky" if ncut == 0 else f"jacobi, {ncut} cut"
    del J, P
    return out


def run_ours(args):
    import numpy as np
    import torch

    import corr_gb300
    from corr_gb300 import workloads as W

    ws, rank, local = dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        torch.cuda.set_device(0)
    dev = torch.cuda.current_device()
    stream = torch.cuda.current_stream()

    B, eps = W.synth_rimp2(NOCC, NVIR, NAUX, SEED)
    Bd = torch.from_numpy(B).to(dev)
    ed = torch.from_numpy(eps).to(dev)
    ctx = corr_gb300.Context(dev, stream=stream)
    ctx.set_timing(True)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    prec = args.precision

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    clocks = ClockSampler(dev) if rank == 0 else None
    if clocks:
        clocks.wait_first()
    for _ in range(max(3, args.warmup)):
        e_split = ctx.rimp2_energy(Bd, ed, NOCC, NVIR, NAUX, prec)

    # One step = one RI-MP2 energy evaluation from the resident FP64 B tensor,
    # enqueued through the asynchronous entry point and captured once into a
    # CUDA graph, so the timed region holds only device work.
    out_e = torch.zeros(4, dtype=torch.float64, device=dev)
    ctx.rimp2_energy_async(Bd, ed, NOCC, NVIR, NAUX, prec, out_e)
    ctx.sync()
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(stream)
    cap0 = ctx.timing().launches_total
    with torch.cuda.graph(graph, stream=side):
        ctx.set_stream(side)
        ctx.rimp2_energy_async(Bd, ed, NOCC, NVIR, NAUX, prec, out_e)
    per_step = ctx.timing().launches_total - cap0  # library kernels in one step
    ctx.set_stream(stream)
    graph.replay()
    torch.cuda.synchronize()
    ctx.sync()

    # ---- timed region: device time per step, L2 flushed between steps
    if clocks:
        clocks.mark()
    barrier()
    evs = []
    for _ in range(args.steps):
        flush.fill_(1)  # outside the timed interval
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        graph.replay()
        t1.record(stream)
        evs.append((t0, t1))
    barrier()
    ctx.sync()
    clk = clocks.stop() if clocks else None
    step_ms = [a.elapsed_time(b) for a, b in evs]
    # graph replays bypass the library's launch counter: the captured step's count
    launches = per_step * args.steps
    e_graph = out_e.cpu().tolist()
    total_ms = sum(step_ms)
    if dist is not None:
        t = torch.tensor([total_ms], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = ws * FLOPS * args.steps / (total_ms * 1e-3) / 1e12
    ms_step = total_ms / args.steps

    # ---- dominant-kernel duration for the roofline (CUDA events inside the
    # library around the energy kernel, on the context stream)
    kern_ms = []
    for _ in range(min(args.steps, 20)):
        flush.fill_(1)
        e_split = ctx.rimp2_energy(Bd, ed, NOCC, NVIR, NAUX, prec)
        kern_ms.append(ctx.timing().kernel_ms)

    # ---- the other precision form (same job, library device timing)
    alt = "split_bf16" if prec != "split_bf16" else "split_fp16"
    e_alt = ctx.rimp2_energy(Bd, ed, NOCC, NVIR, NAUX, alt)
    alt_ms = []
    for _ in range(5):
        flush.fill_(1)
        e_alt = ctx.rimp2_energy(Bd, ed, NOCC, NVIR, NAUX, alt)
        alt_ms.append(ctx.timing().total_ms)

    # ---- FP64 GPU form of the same job (the comparison form)
    ctx.rimp2_energy(Bd, ed, NOCC, NVIR, NAUX, "fp64")
    f64_ms = []
    for _ in range(2):
        flush.fill_(1)
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        e64 = ctx.rimp2_energy(Bd, ed, NOCC, NVIR, NAUX, "fp64")
        t1.record(stream)
        t1.synchronize()
        f64_ms.append(t0.elapsed_time(t1))
    f64 = statistics.median(f64_ms)

    # ---- the metric's time-to-E_corr leg at the water-cluster sizes
    c3 = None if args.no_cluster else time_to_ecorr_c3(ctx)

    # ---- end to end through the public API with host buffers
    Bh = torch.from_numpy(B).pin_memory()
    eh = torch.from_numpy(eps).pin_memory()
    ctx.rimp2_energy(Bh, eh, NOCC, NVIR, NAUX, prec)
    n_e2e = max(3, min(args.steps, 10))
    barrier()
    t0 = time.perf_counter()
    for _ in range(n_e2e):
        e_host = ctx.rimp2_energy(Bh, eh, NOCC, NVIR, NAUX, prec)
    e2e_s = (time.perf_counter() - t0) / n_e2e
    if dist is not None:
        t = torch.tensor([e2e_s], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    h2d = B.nbytes + eps.nbytes
    d2h = 72  # the library's result block (energies + device status word)

    if rank != 0:
        dist.destroy_process_group()
        return

    peak, peak_kind = read_peak()
    kmean = statistics.mean(kern_ms)
    achieved = FLOPS / (kmean * 1e-3) / 1e12
    traffic = read_traffic()
    cpu = None
    if ws == 1 and not args.no_cpu_baseline:
        tf, kind, dt, reps = cpu_sample(B, eps, NOCC, min_seconds=10.0, max_reps=20)
        cpu = {"value": tf, "unit": "TFLOP/s", "cores": blas_threads(), "kind": kind,
               "sample": f"{reps} full RI-MP2 energy evaluation(s) of the workload, "
                         f"{dt:.1f} s"}
    line = {
        "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16" if prec == "split_bf16" else ("f16" if prec == "split_fp16" else "f64"),
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "precision": prec, "global_batch": 1,
                   "parallelism": "replicas" if ws > 1 else "single GPU",
                   "l2": "FP64 input 138 MB > L2 (129 MB); 256 MB L2 flush between timed "
                         "steps, outside the timed region"},
        "time_to_ecorr_ms": ms_step,
        "time_to_ecorr_c3": c3,
        "graph_energy_matches": e_graph[2] == e_split.e_total,
        "energy": {"split": [e_split.e_ss, e_split.e_os, e_split.e_total],
                   "fp64": [e64.e_ss, e64.e_os, e64.e_total],
                   "abs_err_vs_fp64": abs(e_split.e_total - e64.e_total),
                   "rel_err_vs_fp64": abs(e_split.e_total - e64.e_total) / abs(e64.e_total),
                   "host_api_matches": e_host.e_total == e_split.e_total},
        "fp64_form": {"ms_per_step": f64, "tflops": FLOPS / (f64 * 1e-3) / 1e12,
                      "split_speedup": f64 / ms_step},
        "other_split_form": {"precision": alt, "device_ms": statistics.median(alt_ms),
                             "tflops": FLOPS / (statistics.median(alt_ms) * 1e-3) / 1e12,
                             "rel_err_vs_fp64": abs(e_alt.e_total - e64.e_total)
                             / abs(e64.e_total)},
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "kernel": "energy_tc_kernel", "kernel_ms": kmean,
                     "peak_source": f"{peak_kind} bf16 dense (burst)",
                     "flops_per_launch": FLOPS},
        "cpu_baseline": cpu,
        "e2e": {"value": FLOPS / e2e_s / 1e12 * ws, "unit": "TFLOP/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_s * 1e3},
        "gpu_launches": launches,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def run_batch(args):
    """256 independent RI-MP2 instances, nocc ~ U{5..60}, nvir = nocc * U{4..8},
    naux = round(3.5 nvir), B and eps distributed as in the main workload
    (generated on the GPU from a seeded torch generator).  The batched
    precision-form launch is autotuned, captured into a CUDA graph and
    replayed; the FP64 form of every instance gives per-instance |dE|."""
    import torch

    import corr_gb300
    from corr_gb300 import workloads as W

    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    sizes = W.synth_batch_sizes(256, 5005)[:max(1, min(256, args.batch_count))]
    g = torch.Generator(device="cuda")
    g.manual_seed(5006)
    items = []
    flops = 0.0
    for (o, v, X) in sizes:
        s = 0.05 * torch.exp(-torch.arange(X, device="cuda", dtype=torch.float64) / 400.0)
        B = (torch.randn((X, o, v), generator=g, device="cuda", dtype=torch.float64)
             * s[:, None, None]).contiguous()
        eo = torch.sort(torch.rand(o, generator=g, device="cuda", dtype=torch.float64) * 1.2 - 1.5)[0]
        ev = torch.sort(torch.rand(v, generator=g, device="cuda", dtype=torch.float64) * 2.95
                        + 0.05)[0]
        items.append((B, torch.cat([eo, ev]).contiguous(), o, v))
        flops += 2.0 * o * o * v * v * X
    ctx = corr_gb300.Context(0, stream=stream)
    prec = args.precision if args.precision != "fp64" else "split_fp16"
    order, stages, tiles, tune_ms = ctx.batch_autotune(items, prec)
    out = torch.zeros(4 * len(items), dtype=torch.float64, device="cuda")
    ctx.rimp2_energy_batched_async(items, prec, out)
    ctx.sync()
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(stream)
    with torch.cuda.graph(graph, stream=side):
        ctx.set_stream(side)
        ctx.rimp2_energy_batched_async(items, prec, out)
    ctx.set_stream(stream)
    for _ in range(max(3, args.warmup)):
        graph.replay()
    torch.cuda.synchronize()
    steps = max(3, min(args.steps, 20))
    evs = []
    for _ in range(steps):
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        graph.replay()
        t1.record(stream)
        evs.append((t0, t1))
    torch.cuda.synchronize()
    ctx.sync()
    ms = statistics.median(a.elapsed_time(b) for a, b in evs)
    split = out.view(-1, 4)[:, 2].cpu().numpy()
    t0 = time.perf_counter()
    f64 = ctx.rimp2_energy_batched(items, "fp64")
    f64_s = time.perf_counter() - t0
    e64 = [x.e_total for x in f64]
    import numpy as np

    e64 = np.array(e64)
    dE = np.abs(split - e64)
    cpu = None
    if not args.no_cpu_baseline:
        # the reference's CPU energy on the instances in order until ~10 s of
        # work, as a flop rate, scaled to the whole batch
        fn, kind = cpu_energy_fn()
        done = 0
        fdone = 0.0
        t0 = time.perf_counter()
        for (B, e, o, v) in items:
            fn(B.cpu().numpy(), e.cpu().numpy(), o, v)
            done += 1
            fdone += 2.0 * o * o * v * v * B.shape[0]
            if time.perf_counter() - t0 >= 10.0:
                break
        dt = time.perf_counter() - t0
        rate = fdone / dt
        cpu = {"value": len(items) * rate / flops, "unit": "instances/s",
               "cores": blas_threads(), "kind": kind,
               "sample": f"the first {done} instances of the batch ({fdone / 1e12:.2f} TFLOP "
                         f"in {dt:.1f} s, {rate / 1e12:.3f} TFLOP/s), scaled by flops to all "
                         f"{len(items)}"}
    line = {
        "metric": f"batched RI-MP2 instances/s ({len(items)} uneven instances)",
        "value": len(items) / (ms * 1e-3), "unit": "instances/s", "n_gpus": 1,
        "steps": steps, "warmup": max(3, args.warmup), "ms_per_step": ms,
        "higher_is_better": True, "dtype": "bf16" if prec == "split_bf16" else "f16",
        "data": "synthetic",
        "config": {"workload": f"{len(items)} instances, nocc~U{{5..60}}, nvir=nocc*U{{4..8}}, "
                               "naux=round(3.5 nvir), seed 5005/5006",
                   "precision": prec, "policy": {"order": order, "stages": stages,
                                                 "tiles": "128",
                                                 "autotune_ms": tune_ms},
                   "b_bytes": int(sum(B.numel() * 8 for B, _, _, _ in items))},
        "tflops_algorithmic": flops / (ms * 1e-3) / 1e12,
        "fp64_form": {"seconds": f64_s, "instances_per_s": len(items) / f64_s,
                      "split_speedup": f64_s / (ms * 1e-3)},
        "per_instance_abs_err_vs_fp64": {"max": float(dE.max()), "median": float(np.median(dE))},
        "per_instance_rel_err_vs_fp64_max": float((dE / np.abs(e64)).max()),
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)


def cpu_pipeline(mos, eps, J, P, o):
    """The same job on the host cores, as the reference computes it: the
    transform_ri contractions (ri.cc:147-172, BLAS), J^-1/2 by LAPACK's
    eigendecomposition with the cutoff (ri.cc:50-69), B = J^-1/2 (P|ia) and
    the RI-MP2 energy (can_mp2.cc:53-132) on the first nocc_s occupied
    orbitals, scaled by (nocc / nocc_s)^2.  Returns the cpu_baseline object
    (time-to-E_corr in ms)."""
    import numpy as np

    from oracle import oracle as O

    mos, eps, J, P = (t.cpu().numpy() for t in (mos, eps, J, P))
    X, N = P.shape[0], P.shape[1]
    v = N - o
    t0 = time.perf_counter()
    pia = O.transform_ri_np(o, mos, P)
    t1 = time.perf_counter()
    jm, _ = O.ri_metric_inv_sqrt(J)
    B = np.ascontiguousarray((jm @ pia.reshape(X, -1)).reshape(X, o, v))
    t2 = time.perf_counter()
    fn, kind = cpu_energy_fn()
    nocc_s = max(1, min(o, 30))
    es = np.concatenate([eps[:nocc_s], eps[o:]])
    te = time.perf_counter()
    fn(np.ascontiguousarray(B[:, :nocc_s, :]), es, nocc_s, v)
    t3 = time.perf_counter()
    energy_ms = (t3 - te) * 1e3 * (o / nocc_s) ** 2
    total = (t2 - t0) * 1e3 + energy_ms
    return {"value": total, "unit": "ms", "cores": blas_threads(), "kind": kind,
            "sample": f"transform {1e3 * (t1 - t0):.0f} ms + J^-1/2 and B {1e3 * (t2 - t1):.0f} ms "
                      f"(numpy/LAPACK, all cores) + RI-MP2 energy on {nocc_s} of {o} occupied "
                      f"orbitals scaled by (nocc/{nocc_s})^2: {energy_ms:.0f} ms"}


def run_pipeline(args):
    """RI-MP2 time-to-E_corr from the 3-index integrals, by default at the
    water-cluster sizes (nbf=480, nocc=100, naux=1520): (P|ia) transform, metric (Cholesky
    under the inertia certificate, else Jacobi), energy.  Inputs are seeded
    synthetic stand-ins resident on the GPU (corr_gb300.workloads); the
    tests run the same pipeline on the molecular integrals.  Split form vs
    FP64 form of the same call."""
    import torch

    import corr_gb300
    from corr_gb300 import workloads as W

    torch.cuda.set_device(0)
    N, o, X = args.nbf, args.nocc, args.naux
    v = N - o
    mos, eps, J, P = W.synth_ri_pipeline(N, o, X, 303)
    ctx = corr_gb300.Context(0)
    prec = args.precision if args.precision != "fp64" else "split_fp16"
    for _ in range(max(3, args.warmup)):
        e_split, ncut = ctx.rimp2_energy_from_3index(2 * o, mos, eps, J, P, prec)
    steps = max(3, min(args.steps, 10))
    ts = []
    for _ in range(steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e_split, ncut = ctx.rimp2_energy_from_3index(2 * o, mos, eps, J, P, prec)
        ts.append(time.perf_counter() - t0)
    ms = statistics.median(ts) * 1e3
    t0 = time.perf_counter()
    e64, _ = ctx.rimp2_energy_from_3index(2 * o, mos, eps, J, P, "fp64")
    f64_ms = (time.perf_counter() - t0) * 1e3
    flops = (2.0 * X * N * N * o + 2.0 * X * o * v * N + 1.0 * X * X * o * v
             + 2.0 * o * o * v * v * X)
    cpu = None
    if not args.no_cpu_baseline:
        cpu = cpu_pipeline(mos, eps, J, P, o)
    line = {
        "metric": "RI-MP2 time-to-E_corr from 3-index integrals"
                  + (" (water-cluster sizes)" if (N, o, X) == (480, 100, 1520) else ""),
        "value": ms, "unit": "ms", "n_gpus": 1, "steps": steps, "warmup": max(3, args.warmup),
        "ms_per_step": ms, "higher_is_better": False,
        "dtype": "bf16" if prec == "split_bf16" else "f16", "data": "synthetic",
        "config": {"workload": f"nbf={N} nocc={o} naux={X}, seeded synthetic J, (P|mn), C, eps "
                               "resident on the GPU (seed 303)", "precision": prec,
                   "metric_path": "cholesky" if ncut == 0 else f"jacobi, {ncut} cut"},
        "tflops_algorithmic": flops / (ms * 1e-3) / 1e12,
        "fp64_form": {"ms": f64_ms, "split_speedup": f64_ms / ms},
        "energy": {"split": e_split.e_total, "fp64": e64.e_total,
                   "abs_err_vs_fp64": abs(e_split.e_total - e64.e_total)},
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)


def run_cluster(args):
    """Config-3 time-to-E_corr from the basis, as one process runs it: (P|Q) and
    (P|mu nu) on the GPU (corr_ri_integrals) for the 20-water cluster's shells,
    then corr_rimp2_energy_from_3index in the precision form, per step; the
    orbitals are the cluster's RHF orbitals (tests/golden)."""
    import numpy as np
    import torch

    import corr_gb300

    torch.cuda.set_device(0)
    gold = os.path.join(ROOT, "tests", "golden")
    sysd = np.load(os.path.join(gold, "systems.npz"))
    basis = [corr_gb300.Basis(*(sysd[f"c3_{k}_{n}"]
                                for n in ("l", "nprim", "poff", "center", "exps", "coefs")))
             for k in ("obs", "aux")]
    fx = np.load(os.path.join(gold, "config3_cluster.npz"))
    mos = torch.from_numpy(fx["mos"]).cuda()
    eps = torch.from_numpy(fx["eps"]).cuda()
    ctx = corr_gb300.Context(0)
    prec = args.precision if args.precision != "fp64" else "split_fp16"

    def step():
        J, P = ctx.ri_integrals(*basis)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        e, ncut = ctx.rimp2_energy_from_3index(200, mos, eps, J, P, prec)
        return e, ncut, t1

    for _ in range(max(3, args.warmup)):
        step()
    steps = max(3, min(args.steps, 20))
    tot, ints = [], []
    for _ in range(steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e, ncut, t1 = step()
        t2 = time.perf_counter()
        tot.append((t2 - t0) * 1e3)
        ints.append((t1 - t0) * 1e3)
    ms = statistics.median(tot)
    line = {
        "metric": "RI-MP2 time-to-E_corr from the basis (20-water cluster)",
        "value": ms, "unit": "ms", "n_gpus": 1, "steps": steps, "warmup": max(3, args.warmup),
        "ms_per_step": ms, "higher_is_better": False,
        "dtype": "bf16" if prec == "split_bf16" else "f16", "data": "molecular",
        "config": {"workload": "20 H2O, def2-SVP/def2-SVP-RI, N=480 nocc=100 naux=1520, shells of "
                               "tests/golden/systems.npz, RHF orbitals of config3_cluster.npz",
                   "precision": prec, "metric_path": "cholesky" if ncut == 0 else f"jacobi, {ncut} cut"},
        "integrals_ms": statistics.median(ints),
        "pipeline_ms": ms - statistics.median(ints),
        "energy": e.e_total,
    }
    print(json.dumps(line), flush=True)


def run_dgemm(args):
    """The FP64-accurate digit GEMM (corr_dgemm_tc) on the (P|ia) transform's
    shape for 304 auxiliary functions (M = 304 x 100 rows, N = 384, K = 480),
    device operands, against the FP64-pipe GEMM (corr_dgemm) of the same call;
    value = FP64-equivalent TFLOP/s of the whole call (slicing included)."""
    import numpy as np
    import torch

    import corr_gb300

    torch.cuda.set_device(0)
    M, N, K = 30400, 384, 480
    r = np.random.default_rng(5)
    A = torch.from_numpy(r.standard_normal((M, K))).cuda()
    B = torch.from_numpy(r.standard_normal((N, K))).cuda()
    ctx = corr_gb300.Context(0)

    def timed(tc, n):
        for _ in range(max(3, args.warmup)):
            C = ctx.dgemm(A, B, transb=True, tensor_cores=tc)
        torch.cuda.synchronize()
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record()
        for _ in range(n):
            C = ctx.dgemm(A, B, transb=True, tensor_cores=tc)
        s1.record()
        torch.cuda.synchronize()
        return s0.elapsed_time(s1) / n, C

    steps = max(3, min(args.steps, 50))
    ms, C = timed(True, steps)
    ms64, C64 = timed(False, 3)
    flop = 2.0 * M * N * K
    line = {
        "metric": "FP64-accurate GEMM on the tensor cores, FP64-equivalent TFLOP/s",
        "value": flop / (ms * 1e-3) / 1e12, "unit": "TFLOP/s", "n_gpus": 1, "steps": steps,
        "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True,
        "dtype": "f64 (bf16 digits)", "data": "synthetic",
        "config": {"workload": f"C[{M}][{N}] = A[{M}][{K}] B[{N}][{K}]^T, normal random, seed 5"},
        "fp64_pipe_gemm": {"ms": ms64, "tflops": flop / (ms64 * 1e-3) / 1e12,
                           "speedup": ms64 / ms},
        "max_abs_diff_vs_fp64_gemm": float((C - C64).abs().max()),
    }
    print(json.dumps(line), flush=True)


def run_adjoint(args):
    """The RI-MP2 adjoint (dE/dB, dE/deps) at nocc=64, nvir=512, naux=2048
    (config-2 distributions, seeded), device arrays: the tensor-core form
    (corr_rimp2_gradient_tc) per step, timed with CUDA events, and one call of
    the FP64 form (corr_rimp2_gradient) beside it."""
    import numpy as np
    import torch

    import corr_gb300
    from corr_gb300 import workloads as W

    torch.cuda.set_device(0)
    o, v, X = 64, 512, 2048
    B, eps = W.synth_rimp2(o, v, X, 4004)
    Bd, ed = torch.from_numpy(B).cuda(), torch.from_numpy(eps).cuda()
    ctx = corr_gb300.Context(0)

    def timed(tc, n):
        for _ in range(1 if not tc else max(1, args.warmup)):
            r = ctx.rimp2_gradient(Bd, ed, o, v, X, tensor_cores=tc)
        torch.cuda.synchronize()
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record()
        for _ in range(n):
            r = ctx.rimp2_gradient(Bd, ed, o, v, X, tensor_cores=tc)
        s1.record()
        torch.cuda.synchronize()
        return s0.elapsed_time(s1) / n, r

    steps = max(1, min(args.steps, 10))
    ms, (E, dB, de) = timed(True, steps)
    line = {
        "metric": "RI-MP2 adjoint (dE/dB, dE/deps) time", "value": ms, "unit": "ms",
        "n_gpus": 1, "steps": steps, "warmup": max(1, args.warmup), "ms_per_step": ms,
        "higher_is_better": False, "dtype": "f64 (bf16 digits)", "data": "synthetic",
        "config": {"workload": f"nocc={o} nvir={v} naux={X}, B = G diag(s_Q), seed 4004"},
        "energy": E,
    }
    if not args.no_cpu_baseline:
        ms64, (E64, dB64, de64) = timed(False, 1)
        line["fp64_form"] = {"ms": ms64, "speedup": ms64 / ms,
                             "max_rel_dB": float((dB - dB64).abs().max() / dB64.abs().max()),
                             "max_rel_deps": float((de - de64).abs().max() / de64.abs().max())}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.workload == "adjoint":
        run_adjoint(args)
        return
    if args.workload == "cluster":
        run_cluster(args)
        return
    if args.workload == "dgemm_tc":
        run_dgemm(args)
        return
    if args.workload == "batch256":
        run_batch(args)
        return
    if args.workload == "ri_pipeline":
        run_pipeline(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
