"""Benchmark: detrend + masked BLS on Kepler-like light curves (one GB300).

Workload (per GPU): 1024 curves x 65,536 samples at 29.4-min cadence with per-curve
jittered times, 5% masked in contiguous gaps, sinusoid + quadratic trends, noise 5e-4 and
box transits in a quarter of the curves; median detrend with a 49-sample window, offsets,
then BLS over 16,384 frequencies (1/200 .. 2 per day) with nb = 2048 bins, qmi = 0.005,
qma = 0.1 (kma = 205, kmi = 10, kkmi = 327), then per-curve peak statistics.

A step is that whole pipeline over the batch: gfilter -> offset -> geebls -> blsstat.
``value`` is (curve x trial-frequency) evaluations per second with the inputs resident
in HBM (inputs are 512 MiB, larger than L2).  ``e2e`` repeats the step through the
tensor API with host buffers: pinned host -> device copies of the light curves and a
device -> host read of the spectrum and peak statistics inside the timed region.

``--impl reference`` times the reference's algorithm on the host CPU (the FP64 C
restatement of geebls with scipy's median filter, all host threads) on a bounded
sample of the same workload and prints the same metric.

Multi-GPU: one process per GPU (torchrun); every rank processes its own batch of
curves (weak scaling, no data-path collective); the time is the max over ranks.
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

METRIC = "BLS/TLS (curve x freq) evals/sec vs plain; served p50/p99 at SR rel err<=1e-4"
UNIT = "evals/s"

NQ, N, NF, NB, R_MEDIAN = 1024, 65536, 16384, 2048, 24
QMI, QMA = 0.005, 0.1


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--nq", type=int, default=NQ, help="curves per GPU (default: the workload's 1024)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    return p.parse_args()


def workload_config(nq):
    return {"workload": "detrend+masked BLS, Kepler-like: %d curves x %d samples, 29.4-min cadence, "
                        "5%% masked gaps, median window 49, nf=%d (1/200..2 /d), nb=%d, qmi=%g, qma=%g"
                        % (nq, N, NF, NB, QMI, QMA),
            "curves_per_gpu": nq, "samples": N, "nf": NF, "nb": NB, "kma": int(QMA * NB) + 1,
            "kmi": int(QMI * NB), "kkmi": int(N * QMI), "median_window": 2 * R_MEDIAN + 1,
            "phase": "exact 64-bit fixed point", "l2": "inputs 512 MiB per GPU exceed L2 (no flush needed)"}


def make_data(nq, seed):
    from gtrap_gb300 import synth
    lc, tu, ntrue, grid, inj = synth.kepler_like(nq=nq, n=N, nf=NF, nb=NB, qmi=QMI, qma=QMA, seed=seed)
    return lc, tu, ntrue, grid


# ----------------------------------------------------------------------------- clocks

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


# ----------------------------------------------------------------------------- CPU legs

def cpu_pipeline_sample(lc, tu, ntrue, grid, n_curves, n_freqs, threads):
    """Reference algorithm on the host: scipy medfilt residual, masked mean offset and
    the FP64 BLS restatement, for ``n_curves`` curves x ``n_freqs`` frequencies."""
    import oracle
    sub_lc = np.ascontiguousarray(lc[:, :n_curves])
    sub_tu = np.ascontiguousarray(tu[:, :n_curves])
    t0 = time.perf_counter()
    resid = oracle.medfilt_residual(sub_lc, R_MEDIAN)
    off = oracle.offset(resid, sub_tu).astype(np.float32)
    oracle.bls(resid, sub_tu, n_freqs, grid["nb"], grid["kma"], grid["kmi"], grid["kkmi"],
               grid["fmin"], grid["df"], offset=off, ntrue=ntrue[:n_curves], nthreads=threads)
    dt = time.perf_counter() - t0
    return n_curves * n_freqs / dt, dt


def cpu_baseline(lc, tu, ntrue, grid):
    threads = os.cpu_count() or 1
    n_curves, n_freqs = 2, 256 * threads
    value, dt = cpu_pipeline_sample(lc, tu, ntrue, grid, n_curves, n_freqs, threads)
    return {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d curves x %d frequencies of the workload (medfilt + offset + FP64 BLS), %.1f s"
                      % (n_curves, n_freqs, dt)}


def run_reference(args, rank, world):
    if rank != 0:
        return
    lc, tu, ntrue, grid = make_data(4, 2000)
    threads = os.cpu_count() or 1
    n_curves, n_freqs = 1, 128 * threads
    if args.warmup > 0:
        cpu_pipeline_sample(lc, tu, ntrue, grid, 1, threads, threads)
    vals, total = [], 0.0
    for _ in range(args.steps):
        v, dt = cpu_pipeline_sample(lc, tu, ntrue, grid, n_curves, n_freqs, threads)
        vals.append(v)
        total += dt
    value = float(np.median(vals))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": workload_config(NQ),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "per step %d curve x %d frequencies (medfilt + offset + FP64 BLS)"
                                       % (n_curves, n_freqs)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- GPU legs

def run_ours(args, rank, world, local_rank):
    import torch
    import torch.distributed as dist
    from gtrap_gb300 import _build, api

    _build.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    nq = args.nq
    lc, tu, ntrue, grid = make_data(nq, 2000 + 100000 * rank)
    d_lc = torch.from_numpy(lc).to(dev)
    d_tu = torch.from_numpy(tu).to(dev)
    d_nt = torch.from_numpy(ntrue.astype(np.int32)).to(dev)
    stream = torch.cuda.current_stream(dev)
    kma, kmi, kkmi = grid["kma"], grid["kmi"], grid["kkmi"]
    bls_time = []

    def step(x_lc, x_tu, x_nt, timed_bls=False):
        resid = api.gfilter(x_lc, R_MEDIAN)
        off = api.offset(resid, x_tu)
        if timed_bls:
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
        blsp, p1, p2 = api.geebls(resid, x_tu, off, x_nt, NF, NB, kma, kmi, kkmi, grid["fmin"], grid["df"])
        if timed_bls:
            e.record(stream)
            bls_time.append((s, e))
        stats = api.blsstat(blsp, p1, p2, grid["df"], grid["fmin"])
        return blsp, stats

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize(dev)

    for _ in range(args.warmup):
        step(d_lc, d_tu, d_nt)
    barrier()
    clocks = ClockSampler(local_rank)
    clocks.start()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    start.record(stream)
    for _ in range(args.steps):
        step(d_lc, d_tu, d_nt, timed_bls=True)
    end.record(stream)
    barrier()
    clk = clocks.stop()
    ms = start.elapsed_time(end) / args.steps
    bls_ms = float(np.mean([s.elapsed_time(e) for s, e in bls_time]))
    t = torch.tensor([ms, bls_ms], device=dev, dtype=torch.float64)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms, bls_ms = float(t[0]), float(t[1])
    evals = nq * NF * world
    value = evals / (ms / 1e3)

    # e2e through the tensor API with pinned host buffers
    e2e = None
    if not args.no_e2e:
        h_lc = torch.from_numpy(lc).pin_memory()
        h_tu = torch.from_numpy(tu).pin_memory()
        h_nt = torch.from_numpy(ntrue.astype(np.int32)).pin_memory()
        h_out = torch.empty((nq, NF), dtype=torch.float32).pin_memory()
        h_stat = torch.empty((2, nq), dtype=torch.float64).pin_memory()

        def e2e_step():
            x_lc = h_lc.to(dev, non_blocking=True)
            x_tu = h_tu.to(dev, non_blocking=True)
            x_nt = h_nt.to(dev, non_blocking=True)
            blsp, (pest, sde, b1, b2) = step(x_lc, x_tu, x_nt)
            h_out.copy_(blsp, non_blocking=True)
            h_stat[0].copy_(pest, non_blocking=True)
            h_stat[1].copy_(sde, non_blocking=True)

        for _ in range(max(1, args.warmup // 2)):
            e2e_step()
        barrier()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        for _ in range(args.steps):
            e2e_step()
        e.record(stream)
        barrier()
        ems = torch.tensor([s.elapsed_time(e) / args.steps], device=dev, dtype=torch.float64)
        if world > 1:
            dist.all_reduce(ems, op=dist.ReduceOp.MAX)
        h2d = lc.nbytes + tu.nbytes + ntrue.nbytes
        d2h = h_out.numel() * 4 + h_stat.numel() * 8
        e2e = {"value": evals / (float(ems[0]) / 1e3), "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": float(ems[0])}

    if rank != 0:
        return
    # roofline of the dominant kernel (the BLS call: prep + fold/scan), FP32-pipe bound
    sink, flops = api.fp32_peak_probe(iters=4096)
    torch.cuda.synchronize(dev)
    ps, pe = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ps.record(stream)
    for _ in range(3):
        api.fp32_peak_probe(iters=4096)
    pe.record(stream)
    torch.cuda.synchronize(dev)
    peak = flops * 3 / (ps.elapsed_time(pe) / 1e3) / 1e12
    cand = NB * (kma - max(kmi, 1))            # accepted windows per evaluation
    flop_per_eval = 7.0 * cand                  # s, kk, N-kk, den, s^2 and an FMA compare
    achieved = flop_per_eval * nq * NF / (bls_ms / 1e3) / 1e12
    traffic = None
    prof = os.path.join(ROOT, "profiles", "bls_fold_scan_traffic.json")
    if os.path.exists(prof):
        try:
            with open(prof) as f:
                traffic = json.load(f).get("dram_bytes_per_launch_full_workload")
        except Exception:
            traffic = None
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+i64", "data": "synthetic",
            "config": workload_config(nq) | {"parallelism": "replicas x%d (curves sharded)" % world},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "geebls (prep + bls_fold_scan_kernel)", "kernel_ms": bls_ms,
                         "peak_source": "live FP32 FMA-chain probe on this GPU (MEASURED_PEAKS.json has no FP32 figure)",
                         "flop_per_eval": flop_per_eval},
            "gpu_launches": 6 * args.steps,
            "clocks": clk}
    if e2e:
        line["e2e"] = e2e
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(lc, tu, ntrue, grid)
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    try:
        run_ours(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
