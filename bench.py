"""Benchmark of the batched transit search on one GB300 (one process per GPU).

Default workload (``--workload ragged``): the uneven mixed batch.  10,000 curves per GPU
whose lengths are log-uniform on [2,000, 70,000] samples, each at 2-min or 29.4-min cadence,
10% masked in contiguous gaps (t = -1000, zig-zag filled flux), three sinusoids plus a
quadratic trend, box (BLS) or trapezoid (GTLS) signals in a quarter of the curves; half the
curves are BLS requests (nb = 2048, qmi = 0.005, qma = 0.1 -> kma = 205, kmi = 10,
kkmi = int(n*qmi); nf = clip(next_pow2(8 * baseline_days), 2048, 32768), fmin = 2/baseline,
fmax = 2 per day) and half GTLS requests (8 widths from 8 h to 0.5 h, 16 ingress widths,
nsc = wmax/cadence + 3, every sample an epoch).  Every curve is detrended with a 49-sample
running median first.  A step is the whole batch: packed detrend -> offsets -> encoding ->
one persistent BLS launch -> one persistent GTLS launch, replayed from CUDA graphs with the
inputs resident in HBM (5-7 GB, far above L2).  ``value`` is evaluations per second:
(curve, trial frequency) pairs of the BLS requests plus (curve, epoch) pairs of the GTLS
requests.  ``plain`` is the same requests through the plain per-curve entry points (one
launch sequence per curve); ``e2e`` repeats the step with the light curves copied from
pinned host memory and every spectrum copied back inside the timed region.

``--workload masked``: 1024 Kepler-like curves x 65,536 samples, detrend + masked BLS over
16,384 frequencies (the plain image entry points).  ``--workload plain``: plain BLS on 64
curves x 4096 samples, 4096 frequencies, nb 1024 (geebls_simple).  ``--workload tls``: GTLS
in the reference's semantics on 4096 TESS-like curves x 18,000 epochs (8 widths x 16 ingress
widths per epoch).  ``--workload tlsfold``: the folded trapezoid search (an extension) on the
same curves: 8192 periods (0.5 .. 12 d) x 8 durations (0.5 .. 8 h) x 2048 phase bins.
``--workload served``: the continuous-batching server under Poisson arrivals (p50/p99
latency per offered load).  ``--workload lone``: single requests (BLS and GTLS of about 5k, 20k
and 60k samples) through an idle server and through the plain path, the latency floor of
both.  ``--workload mock``: mock transit injection as the TESS mock driver
does it (one drawn planet per curve, lc *= 2 - model, plus trends) on 4096 x 18,000 samples.
``--workload tlsfit``: the reference's CPU trapezoid fit (gtrap/tls.py tlsfit) on one TESS-like
curve over 8 widths x 8 ingress lengths x 4320 epochs, in FP64.  ``--tls-kind fold`` sends the
TLS half of the ragged and served mixes through the folded search instead of GTLS.

``--impl reference`` times the reference's algorithm on the host CPU (the FP64 C
restatement of geebls and gtls with scipy's median filter, all host threads) on a bounded
sample of the same workload and prints the same metric.

Multi-GPU: one process per GPU (torchrun); every rank processes its own batch of curves
(weak scaling, no data-path collective); times are the max over ranks.
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

# masked workload
NQ, N, NF, NB, R_MEDIAN = 1024, 65536, 16384, 2048, 24
QMI, QMA = 0.005, 0.1
# ragged workload
NCURVES = 10000
KMA, KMI = int(QMA * NB) + 1, int(QMI * NB)
NW, NL = 8, 16


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="ragged",
                   choices=["ragged", "masked", "served", "lone", "plain", "tls", "tlsfold", "mock", "tlsfit",
                            "epilogue"])
    p.add_argument("--nq", type=int, default=None,
                   help="curves per GPU (default: 10,000 ragged, 1024 masked)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-plain", action="store_true")
    p.add_argument("--no-parity", action="store_true", help="ragged workload: skip the oracle sample")
    p.add_argument("--no-served", action="store_true", help="ragged workload: skip the served block")
    p.add_argument("--peaks-only", action="store_true",
                   help="served workload: requests return only their statistics records (fused epilogue)")
    p.add_argument("--tls-kind", default="gtls", choices=["gtls", "fold"],
                   help="ragged workload: search the TLS-kind curves with GTLS (reference semantics) or "
                        "the folded trapezoid search")
    return p.parse_args()


def masked_config(nq):
    return {"workload": "detrend+masked BLS, Kepler-like: %d curves x %d samples, 29.4-min cadence, "
                        "5%% masked gaps, median window 49, nf=%d (1/200..2 /d), nb=%d, qmi=%g, qma=%g"
                        % (nq, N, NF, NB, QMI, QMA),
            "curves_per_gpu": nq, "samples": N, "nf": NF, "nb": NB, "kma": KMA,
            "kmi": KMI, "kkmi": int(N * QMI), "median_window": 2 * R_MEDIAN + 1,
            "phase": "exact 64-bit fixed point", "l2": "inputs 512 MiB per GPU exceed L2 (no flush needed)"}


def ragged_config(nc, bat=None, tls_kind="gtls"):
    if tls_kind == "fold":
        tls_desc = ("TLS curves through the folded trapezoid search (nb %d, 8 durations 0.5..8 h, ingress 0.2, "
                    "longest template %d bins) on the BLS frequency rule" % (TF_NB, TF_DMAX))
    else:
        tls_desc = "GTLS nw=%d nl=%d (W 8 h..0.5 h), every sample an epoch" % (NW, NL)
    cfg = {"workload": "uneven mixed BLS/%s batch: %d curves, n log-uniform [2000, 70000], cadence 2 or "
                       "29.4 min, 10%% masked, median window 49; BLS nb=%d kma=%d kmi=%d kkmi=n*%g, "
                       "nf=clip(next_pow2(8*baseline_d), 2048, 32768) from 2/baseline to 2 /d; %s; one "
                       "persistent launch per search kind, CUDA graphs, autotuned tiles"
                       % ("folded TLS" if tls_kind == "fold" else "GTLS", nc, NB, KMA, KMI, QMI, tls_desc),
           "curves_per_gpu": nc, "nb": NB, "kma": KMA, "kmi": KMI, "nw": NW, "nl": NL,
           "median_window": 2 * R_MEDIAN + 1, "phase": "exact 64-bit fixed point",
           "l2": "inputs of several GB per GPU exceed L2 (no flush needed)"}
    if bat is not None:
        cfg.update({"bls_curves": bat.n_bls, "tls_curves": bat.n_tls, "bls_evals": bat.bls_evals,
                    "tls_evals": bat.tls_evals, "fold_curves": bat.n_fold, "fold_evals": bat.fold_evals,
                    "samples_total": bat.total,
                    "tile_frequencies": bat.F, "bls_blocks": bat.bls_blocks, "tls_blocks": bat.tls_blocks})
    return cfg


def _profile(name):
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return None


def smem_atomic_peak(dev):
    """Shared-memory atomic peak in fold updates per second (two 32-bit adds per update)."""
    import bench_probes
    return bench_probes.smem_atomic_updates(dev)


def smem_load_peak(dev):
    """Shared-memory load bandwidth of this GPU in bytes/s (conflict-free 64-bit loads)."""
    import bench_probes
    return bench_probes.smem_load_bytes(dev)


def fp32_peak_tflops(dev):
    """FP32 FMA issue peak of this GPU, measured live (MEASURED_PEAKS.json has no FP32 figure)."""
    import bench_probes
    return bench_probes.fp32_tflops(dev)


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


# ----------------------------------------------------------------------------- masked workload

def make_data(nq, seed):
    from gtrap_gb300 import synth
    lc, tu, ntrue, grid, inj = synth.kepler_like(nq=nq, n=N, nf=NF, nb=NB, qmi=QMI, qma=QMA, seed=seed)
    return lc, tu, ntrue, grid


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


def masked_cpu_baseline(lc, tu, ntrue, grid):
    threads = os.cpu_count() or 1
    n_curves, n_freqs = 2, 256 * threads
    value, dt = cpu_pipeline_sample(lc, tu, ntrue, grid, n_curves, n_freqs, threads)
    return {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d curves x %d frequencies of the workload (medfilt + offset + FP64 BLS), %.1f s"
                      % (n_curves, n_freqs, dt)}


def run_masked_reference(args, rank, world):
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
            "data": "synthetic", "config": masked_config(NQ),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "per step %d curve x %d frequencies (medfilt + offset + FP64 BLS)"
                                       % (n_curves, n_freqs)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_masked(args, rank, world, local_rank):
    import torch
    import torch.distributed as dist
    from gtrap_gb300 import _build, api

    _build.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    nq = args.nq or NQ
    lc, tu, ntrue, grid = make_data(nq, 2000 + 100000 * rank)
    d_lc = torch.from_numpy(lc).to(dev)
    d_tu = torch.from_numpy(tu).to(dev)
    d_nt = torch.from_numpy(ntrue.astype(np.int32)).to(dev)
    stream = torch.cuda.current_stream(dev)
    kma, kmi, kkmi = grid["kma"], grid["kmi"], grid["kkmi"]
    bls_time = []
    gf_time = []

    def step(x_lc, x_tu, x_nt, timed_bls=False):
        if timed_bls:
            g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            g0.record(stream)
        resid = api.gfilter(x_lc, R_MEDIAN)
        if timed_bls:
            g1.record(stream)
            gf_time.append((g0, g1))
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
    gf_ms = float(np.mean([s.elapsed_time(e) for s, e in gf_time]))
    t = torch.tensor([ms, bls_ms, gf_ms], device=dev, dtype=torch.float64)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms, bls_ms, gf_ms = float(t[0]), float(t[1]), float(t[2])
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
    peak = fp32_peak_tflops(dev)
    # the exhaustive scan's work per evaluation: nb * kma windows at ~5 FP32 operations each
    flop_per_eval = 5.0 * NB * kma
    achieved = flop_per_eval * nq * NF / (bls_ms / 1e3) / 1e12
    traffic = None
    prof = _profile("bls_fold_scan_traffic.json")
    if prof:
        traffic = prof.get("dram_bytes_per_launch_full_workload")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+i64", "data": "synthetic",
            "config": masked_config(nq) | {"parallelism": "replicas x%d (curves sharded)" % world},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "geebls (prep + bls_fold_scan_kernel)", "kernel_ms": bls_ms,
                         "peak_source": "live FP32 FMA-chain probe on this GPU (MEASURED_PEAKS.json has no FP32 figure)",
                         "flop_per_eval": flop_per_eval,
                         "work": "exhaustive-scan equivalent: nb*kma windows x 5 FP32 ops per evaluation"},
            "gpu_launches": 6 * args.steps,
            "clocks": clk}
    # the detrend of the same image (gfilter, r = 24): its HBM roofline (8 B a sample read
    # and written) beside its rate; the sorted-window updates in shared memory bind it
    hbm, hbm_src = _hbm_peak_gbs()
    samples = lc.shape[0] * lc.shape[1]
    gbs = 8.0 * samples / (gf_ms / 1e3) / 1e9
    line["gfilter"] = {"ms": gf_ms, "samples_per_s": samples / (gf_ms / 1e3),
                       "hbm": {"achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                               "peak_source": hbm_src, "bytes_per_sample": 8},
                       "bound": "compute: per-sample sorted-window updates in shared memory (binary search "
                                "and shifts), not HBM"}
    if e2e:
        line["e2e"] = e2e
    if not args.no_cpu_baseline:
        # full-size outputs against the FP64 oracle: 2 curves x every 8th frequency (a
        # stride of 8 in j is df' = 8 df, which keeps the exact phases)
        import oracle
        blsp = step(d_lc, d_tu, d_nt)[0].cpu().numpy()
        r2 = oracle.medfilt_residual(lc[:, :2], R_MEDIAN)
        o2 = oracle.offset(r2, tu[:, :2]).astype(np.float32)
        ref = oracle.bls(r2, np.ascontiguousarray(tu[:, :2]), NF // 8, NB, kma, kmi, kkmi, grid["fmin"],
                         grid["df"] * 8, offset=o2, ntrue=ntrue[:2], nthreads=os.cpu_count() or 1)[0]
        got = blsp[:2, ::8]
        ok = ref > 0
        line["parity"] = {"sample": "2 curves x %d frequencies (every 8th; scipy medfilt + offset + FP64 geebls)"
                                    % (NF // 8), "sr_max_rel_err": float(np.max(np.abs(got[ok] - ref[ok]) / ref[ok]))}
        line["cpu_baseline"] = masked_cpu_baseline(lc, tu, ntrue, grid)
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- ragged workload

def make_mix(nc, seed):
    from gtrap_gb300 import synth
    return synth.ragged_mix(nc, seed=seed)


def fold_grid(c):
    """Frequency grid of a TLS-kind curve sent to the folded search: the BLS rule,
    nf = clip(next_pow2(8 * baseline_d), 2048, 32768) from 2/baseline to 2 per day."""
    from gtrap_gb300 import synth
    T = float(c["t"].max())
    nf = int(min(32768, max(2048, synth.next_pow2(8.0 * T))))
    fmin = 2.0 / T
    return nf, float(np.float32(fmin)), float(np.float32((2.0 - fmin) / (nf - 1)))


def build_batch(mix, dev_index, tls_kind="gtls"):
    from gtrap_gb300 import batch as B
    bat = B.RaggedBatch(B.BlsSpec(nb=NB, kma=KMA, kmi=KMI), B.TlsSpec(nw=NW, nl=NL),
                        detrend_r=R_MEDIAN, device=dev_index,
                        fold=B.FoldSpec(nb=TF_NB, durations=tuple(float(w) for w in TF_DURS), lfrac=TF_LFRAC,
                                        dmax=TF_DMAX))
    for c in mix:
        if c["kind"] == "bls":
            bat.add_bls(c["t"], c["x"], c["nf"], c["fmin"], c["df"], kkmi=c["kkmi"])
        elif tls_kind == "fold":
            bat.add_fold(c["t"], c["x"], *fold_grid(c))
        else:
            bat.add_tls(c["t"], c["x"], c["nsc"], c["wmax"], c["dw"], c["deltat"])
    return bat.build()


def cpu_mix_rates(mix, threads, seconds, tls_kind="gtls"):
    """The reference's algorithm on the host for a bounded sample of the mix: scipy's median
    filter, get_offset and the FP64 restatements of geebls and gtls (or of the folded search,
    for ``tls_kind`` "fold"), each kind run over curves until ``seconds`` have passed.
    Returns per-kind rates and a description."""
    import oracle
    oracle.medfilt_residual(np.zeros((64, 1), np.float32), R_MEDIAN)  # imports outside the timing
    bls = [c for c in mix if c["kind"] == "bls"]
    tls = [c for c in mix if c["kind"] == "tls"] if tls_kind == "gtls" else []
    fold = [c for c in mix if c["kind"] == "tls"] if tls_kind == "fold" else []
    t_med = n_med = 0.0
    t_b = e_b = 0.0
    t_t = e_t = 0.0
    nb_c = nt_c = 0
    for c in bls:
        t0 = time.perf_counter()
        resid = oracle.medfilt_residual(c["x"][:, None], R_MEDIAN)
        t1 = time.perf_counter()
        off = oracle.offset(resid, c["t"][:, None]).astype(np.float32)
        ntrue = np.array([np.count_nonzero(c["t"] >= 0)], np.uint32)
        nf = min(c["nf"], 64 * threads)
        oracle.bls(resid, c["t"][:, None], nf, NB, KMA, KMI, c["kkmi"], c["fmin"], c["df"],
                   offset=off, ntrue=ntrue, nthreads=threads)
        t2 = time.perf_counter()
        t_med += t1 - t0
        n_med += c["x"].size
        t_b += t2 - t1
        e_b += nf
        nb_c += 1
        if t_b >= seconds:
            break
    for c in tls:
        t0 = time.perf_counter()
        resid = oracle.medfilt_residual(c["x"][:, None], R_MEDIAN)
        t1 = time.perf_counter()
        nt = min(c["x"].size, 512 * threads)
        oracle.gtls(resid, c["t"][:, None], nt, NW, NL, c["nsc"], c["wmax"], c["dw"], c["deltat"],
                    nthreads=threads)
        t2 = time.perf_counter()
        t_med += t1 - t0
        n_med += c["x"].size
        t_t += t2 - t1
        e_t += nt
        nt_c += 1
        if t_t >= seconds:
            break
    t_f = e_f = 0.0
    nf_c = 0
    for c in fold:  # frequencies spread over the curve's grid, OpenMP over frequencies
        t0 = time.perf_counter()
        resid = oracle.medfilt_residual(c["x"][:, None], R_MEDIAN)
        t1 = time.perf_counter()
        off = oracle.offset(resid, c["t"][:, None]).astype(np.float32)
        nf, fmin, df = fold_grid(c)
        nfs = 2 * threads
        oracle.tls_fold(resid, c["t"][:, None], off, nfs, TF_NB, np.float32(fmin), np.float32(df * (nf // nfs)),
                        TF_DURS, lfrac=TF_LFRAC, dmax=TF_DMAX)
        t2 = time.perf_counter()
        t_med += t1 - t0
        n_med += c["x"].size
        t_f += t2 - t1
        e_f += nfs
        nf_c += 1
        if t_f >= seconds:
            break
    rates = {"bls": e_b / t_b, "medfilt_samples": n_med / t_med}
    if tls:
        rates["tls"] = e_t / t_t
        desc = ("%d BLS curves x <=%d frequencies and %d GTLS curves x <=%d epochs of the mix "
                "(scipy medfilt + get_offset + FP64 geebls/gtls restatements), %.1f s"
                % (nb_c, 64 * threads, nt_c, 512 * threads, t_med + t_b + t_t))
    else:
        rates["fold"] = e_f / t_f
        desc = ("%d BLS curves x <=%d frequencies and %d folded-search curves x %d frequencies of the mix "
                "(scipy medfilt + get_offset + FP64 geebls and folded-search restatements), %.1f s"
                % (nb_c, 64 * threads, nf_c, 2 * threads, t_med + t_b + t_f))
    return rates, desc, t_med + t_b + t_t + t_f


def cpu_mix_value(mix, rates):
    """Evaluations per second of the whole mix at the sampled per-kind CPU rates."""
    bls_ev = sum(c["nf"] for c in mix if c["kind"] == "bls")
    if "fold" in rates:  # TLS-kind curves through the folded search: (curve, frequency) evals
        tls_ev = sum(fold_grid(c)[0] for c in mix if c["kind"] == "tls")
        r_tls = rates["fold"]
    else:
        tls_ev = sum(c["x"].size for c in mix if c["kind"] == "tls")
        r_tls = rates["tls"]
    samples = sum(c["x"].size for c in mix)
    t = bls_ev / rates["bls"] + tls_ev / r_tls + samples / rates["medfilt_samples"]
    return (bls_ev + tls_ev) / t


def ragged_cpu_baseline(mix, seconds=6.0, tls_kind="gtls"):
    threads = os.cpu_count() or 1
    rates, desc, _ = cpu_mix_rates(mix, threads, seconds, tls_kind)
    return {"value": cpu_mix_value(mix, rates), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": desc, "rates": rates}


def run_ragged_reference(args, rank, world):
    if rank != 0:
        return
    nc = args.nq or NCURVES
    mix = make_mix(nc, 4000)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_mix_rates(mix[:40], threads, 0.2, args.tls_kind)
    vals, total = [], 0.0
    desc = ""
    for k in range(args.steps):
        rates, desc, dt = cpu_mix_rates(mix[200 * k:], threads, 1.5, args.tls_kind)
        vals.append(cpu_mix_value(mix, rates))
        total += dt
    value = float(np.median(vals))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": ragged_config(nc, None, args.tls_kind),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "per step: " + desc},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def per_kind(bat, stage_ms, ms):
    """Evaluations per second of each search kind over its own stage of the step (CUDA events
    between the stage replays), and the prep stage's share."""
    out = {"prep_ms": stage_ms.get("prep"), "step_ms": ms}
    if bat.n_bls:
        out["bls"] = {"unit": "(curve, frequency) evals/s", "evals": bat.bls_evals, "stage_ms": stage_ms["bls"],
                      "value": bat.bls_evals / (stage_ms["bls"] / 1e3)}
    if bat.n_fold:
        out["fold"] = {"unit": "(curve, frequency) evals/s", "evals": bat.fold_evals, "stage_ms": stage_ms["fold"],
                       "value": bat.fold_evals / (stage_ms["fold"] / 1e3)}
    if bat.n_tls:
        out["gtls"] = {"unit": "(curve, epoch) evals/s", "evals": bat.tls_evals, "stage_ms": stage_ms["tls"],
                       "value": bat.tls_evals / (stage_ms["tls"] / 1e3)}
    return out


def ragged_parity(mix, bat, n_curves=16, fstride=8):
    """The headline run's outputs against the FP64 oracle on a sample of its full-length
    curves: ``n_curves`` BLS requests spread over the batch at every ``fstride``-th frequency
    and ``n_curves`` GTLS requests at every epoch (each from the raw curve through scipy's
    median filter; the BLS offset is the device's get_offset, itself checked against FP64).
    Tolerances: SR relative error <= 1e-4; best bins identical or tie-equivalent (the
    oracle's power of the GPU's window within 1e-5 of the maximum); GTLS S/N within 1e-4
    (relative, absolute below 1)."""
    import oracle
    from gtrap_gb300 import batch as B
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    bls_curves = [c for c in mix if c["kind"] == "bls"]
    tls_curves = [c for c in mix if c["kind"] == "tls"]
    dev_table = np.frombuffer(bat.bls_curves.cpu().numpy().tobytes(), B.BLS_CURVE)
    out = {"tolerance": "SR rel err <= 1e-4 vs FP64, best bins identical or tie-equivalent (FP64 power "
                        "within 1e-5 of the maximum); GTLS S/N rel err <= 1e-4 (absolute below 1)"}
    if bat.n_bls:
        ks = sorted(set(np.linspace(0, bat.n_bls - 1, min(n_curves, bat.n_bls)).astype(int).tolist()))
        err = off_err = 0.0
        evals = same = ties = bad = best_same = best_tie = best_bad = 0
        for k in ks:
            c, row = bls_curves[k], bat.bls_table[k]
            x, t = c["x"].astype(np.float32), c["t"].astype(np.float32)
            resid = oracle.medfilt_residual(x[:, None], R_MEDIAN)
            off64 = oracle.offset(resid, t[:, None])[0]
            off = np.array([dev_table[k]["offset"]], np.float32)
            off_err = max(off_err, abs(float(off[0]) - off64) / max(1e-3, abs(off64)))
            nt = np.array([row["ntrue"]], np.uint32)
            fmin, df8 = float(row["fmin"]), float(np.float32(row["df"]) * np.float32(fstride))
            nf8 = (int(row["nf"]) + fstride - 1) // fstride
            osr, op1, op2, opmax = oracle.bls(resid, t[:, None], nf8, NB, KMA, KMI, int(row["kkmi"]), fmin, df8,
                                              offset=off, ntrue=nt, nthreads=threads)
            sr, p1, p2 = (a[::fstride] for a in bat.bls_result(k))
            fin = np.isfinite(osr[0])
            err = max(err, float(np.max(np.abs(sr[fin] - osr[0][fin]) / np.maximum(osr[0][fin], 1e-30))))
            evals += nf8
            diff = ((p1 != op1[0]) | (p2 != op2[0])) & fin
            same += int(fin.sum() - diff.sum())

            def tie(j):
                pw = oracle.bls_window_power(resid, t[:, None], 0, j, int(p1[j]), int(p2[j]), NB, fmin, df8,
                                             offset=off, ntrue=nt)
                return abs(pw - opmax[0, j]) <= 1e-5 * opmax[0, j]
            for j in np.flatnonzero(diff):
                if tie(j):
                    ties += 1
                else:
                    bad += 1
            # the curve's best period: argmax over the sampled frequencies, then its bins
            jg, jo = int(np.argmax(sr)), int(np.argmax(osr[0]))
            if jg == jo and p1[jg] == op1[0, jg] and p2[jg] == op2[0, jg]:
                best_same += 1
            elif osr[0, jg] >= osr[0, jo] * (1 - 1e-5) and tie(jg):
                best_tie += 1
            else:
                best_bad += 1
        out["bls"] = {"curves": len(ks), "evals": evals, "frequency_stride": fstride,
                      "sr_max_rel_err": err, "bins_identical": same, "bins_tie_equivalent": ties,
                      "bins_mismatched": bad, "best_period_bins_identical": best_same,
                      "best_period_bins_tie_equivalent": best_tie, "best_period_bins_mismatched": best_bad,
                      "offset_max_rel_err": off_err}
    if bat.n_tls:
        ks = sorted(set(np.linspace(0, bat.n_tls - 1, min(n_curves, bat.n_tls)).astype(int).tolist()))
        err = 0.0
        evals = wsame = 0
        for k in ks:
            c = tls_curves[k]
            x, t = c["x"].astype(np.float32), c["t"].astype(np.float32)
            resid = oracle.medfilt_residual(x[:, None], R_MEDIAN)
            n = x.size
            ref = oracle.gtls(resid, t[:, None], n, NW, NL, c["nsc"], c["wmax"], c["dw"], c["deltat"],
                              nthreads=threads)
            got = bat.tls_result(k)
            err = max(err, float(np.max(np.abs(got[0] - ref[0][:, 0]) / np.maximum(np.abs(ref[0][:, 0]), 1.0))))
            evals += n
            wsame += int(np.sum(got[1] == ref[1][:, 0]))
        out["gtls"] = {"curves": len(ks), "evals": evals, "sn_max_err": err, "w_identical": wsame}
    out["oracle_seconds"] = time.perf_counter() - t0
    return out


def saturation(S, server, pool, out=None):
    """Every request of ``pool`` offered at once; throughput and latency over the whole run.
    Each result's arrays are released as it arrives (its byte count kept); ``out`` collects
    the results."""
    t0 = time.perf_counter()
    res = S.serve_trace(server, pool, np.zeros(len(pool)), keep_outputs=False)
    wall = time.perf_counter() - t0
    if out is not None:
        out.extend(res)
    return S.latency_summary(res, wall)


def served_block(dev, rank, npool=600, fracs=(0.1, 0.5, 0.9)):
    """The continuous-batching server on a Poisson pool of single-curve requests (BLS or GTLS
    50/50, detrended; n log-uniform [1000, 70000]): saturation throughput and p50/p99 latency
    at ``fracs`` of saturation, beside the plain per-request path at the same offered rates."""
    from gtrap_gb300 import serve as S, synth
    curves = synth.ragged_mix(npool, seed=5000 + 100000 * rank, n_range=(1000, 70000))
    pool = [S.Request.from_curve(c) for c in curves]
    srv = S.TransitServer(detrend_r=R_MEDIAN, hbm_budget=100e9)
    for r in pool[:40]:
        srv.submit(r)
    srv.run_until_idle()
    # results are released as they arrive (a consuming client), in every run below
    sat = saturation(S, srv, pool)
    plain = S.PlainServer(detrend_r=R_MEDIAN)
    for r in pool[:10]:
        plain.process(r)
    psat = saturation(S, plain, pool[:200])
    sweep = []
    for frac in fracs:
        rate = frac * sat["req_per_s"]
        m = min(npool, max(200, int(rate * 1.0)))
        s = S.latency_summary(S.serve_trace(srv, pool[:m], S.poisson_trace(m, rate, seed=int(frac * 1000)),
                                            keep_outputs=False))
        pm = min(200, max(60, int(rate * 0.3)))
        ps = S.latency_summary(S.serve_trace(plain, pool[:pm], S.poisson_trace(pm, rate, seed=int(frac * 1000)),
                                             keep_outputs=False))
        sweep.append({"offered_frac": frac, "offered_req_per_s": rate, "requests": m,
                      "served_req_per_s": s["req_per_s"], "p50_ms": s["p50_ms"], "p99_ms": s["p99_ms"],
                      "evals_per_s": s["evals_per_s"],
                      "plain": {"requests": pm, "served_req_per_s": ps["req_per_s"], "p50_ms": ps["p50_ms"],
                                "p99_ms": ps["p99_ms"]}})
    return {"what": "continuous-batching server (gtrap_gb300.serve.TransitServer), Poisson arrivals of "
                    "single-curve BLS/GTLS requests (50/50, detrended), n log-uniform [1000, 70000], nf 2k-32k, "
                    "HBM budget 100 GB; latency = result on the host minus arrival",
            "pool": npool, "saturation": sat, "plain_saturation": psat, "sweep": sweep,
            "hbm_high_water_bytes": srv.hbm_high_water()}


def run_ragged(args, rank, world, local_rank):
    import torch
    import torch.distributed as dist
    from gtrap_gb300 import _build, batch as B

    _build.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    nc = args.nq or NCURVES
    mix = make_mix(nc, 4000 + 100000 * rank)
    bat = build_batch(mix, local_rank, args.tls_kind)
    stream = torch.cuda.current_stream(dev)
    B.autotune(bat)
    graphs = bat.capture_stages()

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize(dev)

    stages = [name for name in ("prep", "bls", "fold", "tls") if name in graphs]
    marks = {name: [] for name in stages}

    def step(timed=False):
        # events between the stage replays time each stage on the launching stream
        for name in stages:
            if timed:
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
            graphs[name].replay()
            if timed:
                b.record(stream)
                marks[name].append((a, b))

    for _ in range(args.warmup):
        step()
    barrier()
    clocks = ClockSampler(local_rank)
    clocks.start()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    start.record(stream)
    for _ in range(args.steps):
        step(timed=True)
    end.record(stream)
    barrier()
    clk = clocks.stop()
    ms = start.elapsed_time(end) / args.steps
    stage_ms = {name: float(np.mean([a.elapsed_time(b) for a, b in marks[name]])) for name in stages}
    t = torch.tensor([ms] + [stage_ms[name] for name in stages], device=dev, dtype=torch.float64)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms = float(t[0])
    stage_ms = {name: float(v) for name, v in zip(stages, t[1:].tolist())}
    bls_ms = stage_ms.get("bls", 0.0)
    evals_rank = bat.bls_evals + bat.fold_evals + bat.tls_evals
    evals = evals_rank * world
    value = evals / (ms / 1e3)
    ref = [bat.bls_result(k) for k in range(0, bat.n_bls, max(1, bat.n_bls // 64))]
    ref_t = [bat.tls_result(k) for k in range(0, bat.n_tls, max(1, bat.n_tls // 64))]
    ref_f = [bat.fold_result(k) for k in range(0, bat.n_fold, max(1, bat.n_fold // 64))]

    e2e = None
    if not args.no_e2e:
        # the public path a caller streams batches through: each step copies its inputs from
        # pinned host memory and its spectra back.  Two device buffer sets (a second batch with
        # the same configuration and graphs) let step k+1's upload and step k-1's download run
        # on copy streams under step k's kernels; every step's copies stay inside the region.
        bat2 = build_batch(mix, local_rank, args.tls_kind)
        bat2.set_config(bat.F, bat.bls_blocks, bat.tls_blocks)
        sets = [(bat, graphs), (bat2, bat2.capture_stages())]
        outs = lambda b: (b.blsp, b.ph1, b.ph2) + tuple(b.tls_outs if b.n_tls else ()) + \
            tuple(b.fold_outs if b.n_fold else ())
        h_t = bat.t.cpu().pin_memory()
        h_x = bat.x.cpu().pin_memory()
        h_o = [[torch.empty(a.numel(), dtype=a.dtype).pin_memory() for a in outs(b)] for b, _ in sets]
        s_up, s_down = torch.cuda.Stream(dev), torch.cuda.Stream(dev)

        def e2e_run(steps, start=None):
            done_c, done_d = [None, None], [None, None]
            if start is not None:
                s_up.wait_event(start)
            for k in range(steps):
                i = k % 2
                b, gr = sets[i]
                if done_c[i] is not None:  # set i's previous kernels have consumed its inputs
                    s_up.wait_event(done_c[i])
                with torch.cuda.stream(s_up):
                    b.t.copy_(h_t, non_blocking=True)
                    b.x.copy_(h_x, non_blocking=True)
                up = torch.cuda.Event()
                up.record(s_up)
                stream.wait_event(up)
                if done_d[i] is not None:  # set i's previous spectra are on the host
                    stream.wait_event(done_d[i])
                for name in ("prep", "bls", "fold", "tls"):
                    if name in gr:
                        gr[name].replay()
                done_c[i] = torch.cuda.Event()
                done_c[i].record(stream)
                s_down.wait_event(done_c[i])
                with torch.cuda.stream(s_down):
                    for h, a in zip(h_o[i], outs(b)):
                        h.copy_(a, non_blocking=True)
                done_d[i] = torch.cuda.Event()
                done_d[i].record(s_down)
            for ev in done_d:
                if ev is not None:
                    stream.wait_event(ev)

        e2e_run(2)
        barrier()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        e2e_run(args.steps, start=s)
        e.record(stream)
        barrier()
        ems = torch.tensor([s.elapsed_time(e) / args.steps], device=dev, dtype=torch.float64)
        if world > 1:
            dist.all_reduce(ems, op=dist.ReduceOp.MAX)
        h2d = (h_t.numel() + h_x.numel()) * 4
        d2h = sum(h.numel() * h.element_size() for h in h_o[0])
        same = all(np.array_equal(h.numpy(), a.cpu().numpy()) for h, a in zip(h_o[(args.steps - 1) % 2], outs(bat)))
        e2e = {"value": evals / (float(ems[0]) / 1e3), "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": float(ems[0]),
               "api": "gtrap_gb300.batch.RaggedBatch (graph replays), pinned host buffers, uploads and "
                      "downloads on copy streams overlapping the neighbouring steps' kernels",
               "spectra_equal_to_resident_run": bool(same)}
        del sets, bat2

    plain = None
    if not args.no_plain:
        # the same requests, one plain launch sequence per curve (warm-up on a few curves)
        B.run_plain(bat, bls_curves=range(min(8, bat.n_bls)), tls_curves=range(min(8, bat.n_tls)),
                    fold_curves=range(min(8, bat.n_fold)))
        barrier()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        w0 = time.perf_counter()
        s.record(stream)
        B.run_plain(bat)
        e.record(stream)
        barrier()
        pw = time.perf_counter() - w0
        pms = torch.tensor([max(s.elapsed_time(e), 1e3 * pw)], device=dev, dtype=torch.float64)
        if world > 1:
            dist.all_reduce(pms, op=dist.ReduceOp.MAX)
        same = all(np.array_equal(x, y) for a, k in zip(ref, range(0, bat.n_bls, max(1, bat.n_bls // 64)))
                   for x, y in zip(a, bat.bls_result(k)))
        same = same and all(np.array_equal(x, y) for a, k in zip(ref_t, range(0, bat.n_tls, max(1, bat.n_tls // 64)))
                            for x, y in zip(a, bat.tls_result(k)))
        same = same and all(np.array_equal(x, y) for a, k in zip(ref_f, range(0, bat.n_fold, max(1, bat.n_fold // 64)))
                            for x, y in zip(a, bat.fold_result(k)))
        plain = {"value": evals / (float(pms[0]) / 1e3), "unit": UNIT, "ms_per_step": float(pms[0]),
                 "what": "same requests through the plain per-curve entry points (gfilter, get_offset, "
                         "geebls, tls_fold or gtls per curve), one pass",
                 "bit_identical_sampled_outputs": bool(same)}
        step()  # restore the batch's own outputs

    plain_images = None
    if not args.no_plain:
        # the reference drivers' form: one padded [n, nq] image launch sequence per 256 curves
        imgs = B.ImageBatches(bat, per_image=256)
        imgs.run()  # warm-up pass (kernel attributes, allocator)
        barrier()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        w0 = time.perf_counter()
        s.record(stream)
        imgs.run()
        e.record(stream)
        barrier()
        pw = time.perf_counter() - w0
        pms = torch.tensor([max(s.elapsed_time(e), 1e3 * pw)], device=dev, dtype=torch.float64)
        if world > 1:
            dist.all_reduce(pms, op=dist.ReduceOp.MAX)
        plain_images = {"value": evals / (float(pms[0]) / 1e3), "unit": UNIT, "ms_per_step": float(pms[0]),
                        "what": "the reference drivers' per-batch form: curves in arrival order, 256 per [n, nq] "
                                "image padded to its longest curve, one gfilter + get_offset + geebls (common "
                                "grid: lowest fmin and finest df of the image's curves; kkmi of its shortest) or "
                                "gfilter + gtls (images of one cadence) launch sequence per image; value counts "
                                "the requested evaluations only",
                        "images": len(imgs.bls_images) + len(imgs.tls_images),
                        "evaluated_pairs": imgs.bls_pairs + imgs.tls_pairs, "requested_pairs": evals_rank}
        del imgs
        step()

    if rank != 0:
        return
    peak = fp32_peak_tflops(dev)
    # the exhaustive scan's work per evaluation: nb * kma candidate windows at ~5 FP32
    # operations each (two prefix differences, the square, the denominator, the compare)
    flop_per_eval = 5.0 * NB * KMA
    achieved = flop_per_eval * bat.bls_evals / (bls_ms / 1e3) / 1e12
    traffic = issue = None
    prof = _profile("bls_queue_ragged_traffic.json")
    if prof and prof.get("dram_bytes_per_sample_frequency"):
        unit_work = float(sum(int(r["n"]) * int(r["nf"]) for r in bat.bls_table))
        traffic = prof["dram_bytes_per_sample_frequency"] * unit_work
    if prof and prof.get("warp_inst_per_eval") and clk.get("sm_mhz"):
        # executed instructions (ncu count per evaluation of the same mix) per second of the
        # live kernel time, against the issue limit of 4 warp instructions per clock per SM
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        ipeak = 4.0 * sms * clk["sm_mhz"] * 1e6
        irate = prof["warp_inst_per_eval"] * bat.bls_evals / (bls_ms / 1e3)
        issue = {"achieved": irate, "peak": ipeak, "unit": "warp instructions/s", "frac": irate / ipeak,
                 "inst_per_eval": prof["warp_inst_per_eval"], "source": prof.get("source")}
    # second roofline leg: the fold's sample updates against the shared-atomic peak
    dev_table = np.frombuffer(bat.bls_curves.cpu().numpy().tobytes(), B.BLS_CURVE)
    updates = float((dev_table["nv"].astype(np.float64) * dev_table["nf"]).sum())
    apeak = smem_atomic_peak(dev)
    fold_leg = {"bound": "smem_atomics", "achieved": updates / (bls_ms / 1e3), "peak": apeak,
                "unit": "sample updates/s", "frac": updates / (bls_ms / 1e3) / apeak,
                "peak_source": "live probe: two 32-bit shared atomics per update on random bins"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+i64", "data": "synthetic",
            "config": ragged_config(nc, bat, args.tls_kind) | {"parallelism": "replicas x%d (curves sharded)" % world},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "bls_queue_kernel (persistent BLS fold + scan)", "kernel_ms": bls_ms,
                         "kernel_share": bls_ms / ms,
                         "peak_source": "live FP32 FMA-chain probe on this GPU (MEASURED_PEAKS.json has no FP32 figure)",
                         "flop_per_eval": flop_per_eval,
                         "work": "exhaustive-scan equivalent: nb*kma windows x 5 FP32 ops per evaluation; the "
                                 "pruned scan evaluates a few per cent of them, see issue",
                         "issue": issue, "fold": fold_leg},
            "per_kind": per_kind(bat, stage_ms, ms),
            "gpu_launches": (1 + 4 * (bat.n_bls > 0) + 4 * (bat.n_fold > 0) + (bat.n_tls > 0)) * args.steps,
            "clocks": clk}
    if plain:
        line["plain"] = plain
    if plain_images:
        line["plain_images"] = plain_images
    if not args.no_parity:
        line["parity"] = ragged_parity(mix, bat)
    if not args.no_served and args.tls_kind == "gtls":
        line["served"] = served_block(dev, rank)
    if e2e:
        line["e2e"] = e2e
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = ragged_cpu_baseline(mix, tls_kind=args.tls_kind)
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- image workloads

L2_FLUSH_BYTES = 256 << 20  # more than the 129 MB L2


def _timed(fn, steps, warmup, dev, world, flush=False):
    """Mean CUDA-event time of ``steps`` calls after ``warmup`` untimed ones.  With ``flush``
    (inputs that fit in L2) a 256 MiB buffer is written before every timed call, outside its
    events, so each call starts from a cold L2."""
    import torch
    import torch.distributed as dist
    stream = torch.cuda.current_stream(dev)
    for _ in range(warmup):
        fn()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize(dev)
    clocks = ClockSampler(dev.index)
    clocks.start()
    if flush:
        buf = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for k in range(steps):
            buf.fill_(k & 0xff)
            ev[k][0].record(stream)
            fn()
            ev[k][1].record(stream)
        torch.cuda.synchronize(dev)
        ms = sum(a.elapsed_time(b) for a, b in ev)
    else:
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        for _ in range(steps):
            fn()
        e.record(stream)
        torch.cuda.synchronize(dev)
        ms = s.elapsed_time(e)
    clk = clocks.stop()
    t = torch.tensor([ms / steps], device=dev, dtype=torch.float64)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t[0]), clk


def run_image(args, rank, world, local_rank):
    """Config 1 (plain BLS) or config 3 (GTLS, reference semantics) through the image entry
    points, inputs resident (evaluations: (curve, frequency) or (curve, epoch)); ``e2e`` with
    pinned host buffers through the same calls."""
    import torch
    import torch.distributed as dist
    from gtrap_gb300 import _build, api, synth
    _build.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.current_stream(dev)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    if args.workload == "plain":
        nq = args.nq or 64
        wl = synth.plain_bls(nq=nq, seed=1000 + 100000 * rank)
        lcn, tun = wl.lc, wl.tu
        lc, tu = d(lcn), d(tun)
        outs = [api.geebls_simple(lc, tu, wl.nf, wl.nb, wl.kma, wl.kmi, wl.kkmi, wl.fmin, wl.df)]
        fn = lambda: outs.__setitem__(0, api.geebls_simple(lc, tu, wl.nf, wl.nb, wl.kma, wl.kmi, wl.kkmi,
                                                           wl.fmin, wl.df))
        evals = nq * wl.nf
        cfg = {"workload": "plain BLS (geebls_simple): %d curves x 4096 samples, nf 4096, nb 1024, "
                           "qmi 0.005, qma 0.1" % nq, "curves_per_gpu": nq,
               "l2": "inputs 1 MiB fit in L2: a 256 MiB buffer is written before every timed step, "
                     "outside its CUDA events"}
    else:
        nq = args.nq or 4096
        lcn, tun, _ = synth.tess_like(nq=nq, n=18000, seed=3000 + 100000 * rank)
        g = synth.tls_grid()
        lc, tu = d(lcn), d(tun)
        outs = [api.gtls(lc, tu, 18000, g["nw"], g["nl"], g["nsc"], g["wmax"], g["dw"], g["deltat"])]
        fn = lambda: api.gtls(lc, tu, 18000, g["nw"], g["nl"], g["nsc"], g["wmax"], g["dw"], g["deltat"],
                              out=outs[0])
        evals = nq * 18000
        cfg = {"workload": "GTLS (reference semantics): %d TESS-like curves x 18000 epochs, nw 8 "
                           "(8 h .. 0.5 h), nl 16, nsc %d; 128 templates per (curve, epoch)"
                           % (nq, g["nsc"]), "curves_per_gpu": nq, "templates_per_eval": 128,
               "l2": "inputs %d MiB per GPU exceed L2" % (2 * nq * 18000 * 4 >> 20)}
    ms, clk = _timed(fn, args.steps, args.warmup, dev, world, flush=args.workload == "plain")
    e2e = None
    if not args.no_e2e:
        h_lc, h_tu = torch.from_numpy(np.ascontiguousarray(lcn)).pin_memory(), torch.from_numpy(np.ascontiguousarray(tun)).pin_memory()
        res = outs[0] if isinstance(outs[0], tuple) else (outs[0],)
        h_o = [torch.empty(a.shape, dtype=a.dtype).pin_memory() for a in res]

        def e2e_step():
            lc.copy_(h_lc, non_blocking=True)
            tu.copy_(h_tu, non_blocking=True)
            fn()
            r = outs[0] if isinstance(outs[0], tuple) else (outs[0],)
            for h, a in zip(h_o, r):
                h.copy_(a, non_blocking=True)

        e2e_step()
        torch.cuda.synchronize(dev)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        for _ in range(args.steps):
            e2e_step()
        e.record(stream)
        torch.cuda.synchronize(dev)
        ems = torch.tensor([s.elapsed_time(e) / args.steps], device=dev, dtype=torch.float64)
        if world > 1:
            dist.all_reduce(ems, op=dist.ReduceOp.MAX)
        e2e = {"value": evals * world / (float(ems[0]) / 1e3), "unit": UNIT,
               "h2d_bytes_per_step": (h_lc.numel() + h_tu.numel()) * 4,
               "d2h_bytes_per_step": sum(h.numel() * h.element_size() for h in h_o),
               "ms_per_step": float(ems[0]), "api": "gtrap_gb300.api (%s) with pinned host buffers"
               % ("geebls_simple" if args.workload == "plain" else "gtls")}
    if rank != 0:
        return
    peak = fp32_peak_tflops(dev)
    if args.workload == "plain":
        flop_per_eval = 7.0 * wl.nb * (wl.kma - max(wl.kmi, 1))
        roof = {"bound": "fp32", "kernel": "bls_fold_scan_kernel", "flop_per_eval": flop_per_eval,
                "note": "exhaustive-scan FP32 work per (curve, frequency); pruning skips most windows"}
    else:
        flop_per_eval = 40.0 * 128
        roof = {"bound": "fp32", "kernel": "gtls_kernel", "flop_per_eval": flop_per_eval,
                "note": "40 FP32 flops of the statistic per template (H, chi^2, S/N); the kernel is "
                        "issue bound (binary searches and region walks dominate its instructions), so "
                        "this fraction is low"}
    achieved = flop_per_eval * evals / (ms / 1e3) / 1e12
    roof.update({"achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak, "traffic": None,
                 "kernel_ms": ms, "peak_source": "live FP32 FMA-chain probe on this GPU"})
    line = {"metric": METRIC, "value": evals * world / (ms / 1e3), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+i64" if args.workload == "plain" else "f32",
            "data": "synthetic", "config": cfg | {"parallelism": "replicas x%d" % world}, "roofline": roof,
            "gpu_launches": (3 if args.workload == "plain" else 1) * args.steps, "clocks": clk}
    if e2e:
        line["e2e"] = e2e
    if not args.no_cpu_baseline:
        import oracle
        if args.workload == "plain":
            sr = outs[0].cpu().numpy()
            ref = oracle.bls(np.ascontiguousarray(lcn[:, :4]), tun, wl.nf, wl.nb, wl.kma, wl.kmi, wl.kkmi, wl.fmin,
                             wl.df, nthreads=os.cpu_count() or 1)[0]
            ok = ref > 0
            line["parity"] = {"sample": "4 curves x all %d frequencies (FP64 oracle)" % wl.nf,
                              "sr_max_rel_err": float(np.max(np.abs(sr[:4][ok] - ref[ok]) / ref[ok]))}
        else:
            sn = outs[0][0].cpu().numpy()[:, :2]
            osn = oracle.gtls(np.ascontiguousarray(lcn[:, :2]), np.ascontiguousarray(tun[:, :2]), 18000, g["nw"],
                              g["nl"], g["nsc"], g["wmax"], g["dw"], g["deltat"], nthreads=os.cpu_count() or 1)[0]
            line["parity"] = {"sample": "2 curves x 18000 epochs (FP64 oracle)",
                              "sn_max_err_rel_or_abs1": float(np.max(np.abs(sn - osn) / np.maximum(np.abs(osn), 1.0)))}
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        if args.workload == "plain":
            ncs = min(nq, 64)
            oracle.bls(np.ascontiguousarray(lcn[:, :ncs]), tun, wl.nf, wl.nb, wl.kma, wl.kmi, wl.kkmi, wl.fmin,
                       wl.df, nthreads=threads)
            done, sample = ncs * wl.nf, "%d curves x %d frequencies (FP64 geebls_simple restatement)" % (ncs, wl.nf)
        else:
            ncs = min(nq, 32)
            oracle.gtls(np.ascontiguousarray(lcn[:, :ncs]), np.ascontiguousarray(tun[:, :ncs]), 18000, g["nw"],
                        g["nl"], g["nsc"], g["wmax"], g["dw"], g["deltat"], nthreads=threads)
            done, sample = ncs * 18000, "%d curves x 18000 epochs (FP64 gtls restatement)" % ncs
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": done / dt, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": sample + ", %.1f s" % dt}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- folded TLS

TF_N, TF_NF, TF_NB, TF_DMAX, TF_LFRAC = 18000, 8192, 2048, 1024, 0.2
TF_FMIN = 1.0 / 12.0
TF_DF = (2.0 - TF_FMIN) / (TF_NF - 1)
TF_DURS = (np.linspace(0.5, 8.0, 8) / 24.0).astype(np.float32)


def tlsfold_config(nq):
    return {"workload": "folded trapezoid search (extension): %d TESS-like curves x %d samples, "
                        "%d periods 0.5..12 d, 8 durations 0.5..8 h, %d phase bins, ingress %.1f of "
                        "the duration, longest template %d bins; (curve, period) evaluations of up to "
                        "8 x %d templates" % (nq, TF_N, TF_NF, TF_NB, TF_LFRAC, TF_DMAX, TF_NB),
            "curves_per_gpu": nq, "l2": "inputs %d MiB per GPU exceed L2" % (2 * nq * TF_N * 4 >> 20)}


def tlsfold_valid_templates():
    """Templates per frequency the kernel evaluates (2 <= D <= dmax), per frequency index."""
    j = np.arange(TF_NF, dtype=np.float32)
    f0 = (np.float32(TF_DF) * j + np.float32(TF_FMIN)).astype(np.float32)
    D = np.rint(TF_DURS[None, :] * f0[:, None] * np.float32(TF_NB)).astype(np.int64)
    return ((D >= 2) & (D <= TF_DMAX)).sum(axis=1)


def tlsfold_cpu_sample(lcn, tun, threads, n_freqs):
    """FP64 oracle (direct sums per template, OpenMP over frequencies) on one curve and
    ``n_freqs`` frequencies spread over the whole grid.  Returns (evals/s, seconds)."""
    import oracle
    stride = max(1, TF_NF // n_freqs)
    lc = np.ascontiguousarray(lcn[:, :1])
    tu = np.ascontiguousarray(tun[:, :1])
    off = np.zeros(1, np.float32)
    t0 = time.perf_counter()
    oracle.tls_fold(lc, tu, off, n_freqs, TF_NB, TF_FMIN, TF_DF * stride, TF_DURS, lfrac=TF_LFRAC,
                    dmax=TF_DMAX)
    dt = time.perf_counter() - t0
    return n_freqs / dt, dt


def tlsfold_sampled_parity(lcn, tun, outs, curves=(0, 1), nfs=16):
    """Full-size outputs against the FP64 oracle on a sample: ``nfs`` frequencies spread
    over the grid for each sampled curve."""
    import oracle
    stride = TF_NF // nfs
    tsr = outs[0].cpu().numpy()
    st, du = outs[1].cpu().numpy(), outs[2].cpu().numpy()
    rel, same = 0.0, 0
    for q in curves:
        lc = np.ascontiguousarray(lcn[:, q:q + 1])
        tu = np.ascontiguousarray(tun[:, q:q + 1])
        otsr, ost, odu = oracle.tls_fold(lc, tu, np.zeros(1, np.float32), nfs, TF_NB, TF_FMIN, TF_DF * stride,
                                         TF_DURS, lfrac=TF_LFRAC, dmax=TF_DMAX)[:3]
        j = np.arange(nfs) * stride
        ok = otsr[0] > 0
        if ok.any():
            rel = max(rel, float(np.max(np.abs(tsr[q, j][ok] - otsr[0][ok]) / otsr[0][ok])))
        same += int(np.sum((st[q, j] == ost[0]) & (du[q, j] == odu[0])))
    return {"sample": "%d curves x %d frequencies spread over the grid (FP64 oracle, direct sums)" % (len(curves), nfs),
            "tsr_max_rel_err": rel, "best_template_equal_frac": same / (len(curves) * nfs)}


def run_tlsfold(args, rank, world, local_rank):
    """Folded trapezoid search over the BLS phase bins (an extension without a reference
    counterpart): inputs resident for ``value``; pinned host buffers for ``e2e``."""
    import torch
    import torch.distributed as dist
    from gtrap_gb300 import _build, api, synth
    _build.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.current_stream(dev)
    nq = args.nq or 4096
    lcn, tun, _ = synth.tess_like(nq=nq, n=TF_N, seed=3000 + 100000 * rank)
    lc = torch.from_numpy(lcn).to(dev)
    tu = torch.from_numpy(tun).to(dev)
    off = torch.zeros(nq, dtype=torch.float32, device=dev)
    outs = api.tls_fold(lc, tu, off, TF_NF, TF_NB, TF_FMIN, TF_DF, TF_DURS, lfrac=TF_LFRAC, dmax=TF_DMAX)
    fn = lambda: api.tls_fold(lc, tu, off, TF_NF, TF_NB, TF_FMIN, TF_DF, TF_DURS, lfrac=TF_LFRAC,
                              dmax=TF_DMAX, out=outs)
    ms, clk = _timed(fn, args.steps, args.warmup, dev, world)
    evals = nq * TF_NF
    e2e = None
    if not args.no_e2e:
        h_lc, h_tu = torch.from_numpy(lcn).pin_memory(), torch.from_numpy(tun).pin_memory()
        h_o = [torch.empty(a.shape, dtype=a.dtype).pin_memory() for a in outs]

        def e2e_step():
            lc.copy_(h_lc, non_blocking=True)
            tu.copy_(h_tu, non_blocking=True)
            fn()
            for h, a in zip(h_o, outs):
                h.copy_(a, non_blocking=True)

        e2e_step()
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize(dev)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        for _ in range(args.steps):
            e2e_step()
        e.record(stream)
        torch.cuda.synchronize(dev)
        ems = torch.tensor([s.elapsed_time(e) / args.steps], device=dev, dtype=torch.float64)
        if world > 1:
            dist.all_reduce(ems, op=dist.ReduceOp.MAX)
        e2e = {"value": evals * world / (float(ems[0]) / 1e3), "unit": UNIT,
               "h2d_bytes_per_step": (h_lc.numel() + h_tu.numel()) * 4,
               "d2h_bytes_per_step": sum(h.numel() * h.element_size() for h in h_o),
               "ms_per_step": float(ems[0]), "api": "gtrap_gb300.api.tls_fold with pinned host buffers"}
    if rank != 0:
        return
    # roofline: the template phase reads the moment entries from shared memory; per template
    # three corners of 16 + 4 bytes (GS, K with the high word of G, low word of G) = 60 B,
    # plus 20 B per start bin and frequency for the start corner
    tpl = float(tlsfold_valid_templates().sum()) * nq * TF_NB
    lds_bytes = tpl * 60.0 + float(evals) * TF_NB * 20.0
    speak = smem_load_peak(dev)
    achieved = lds_bytes / (ms / 1e3)
    nv = float(np.count_nonzero(np.isfinite(lcn) & (tun >= 0)))
    apeak = smem_atomic_peak(dev)
    fold_leg = {"bound": "smem_atomics", "achieved": nv * TF_NF / (ms / 1e3), "peak": apeak,
                "unit": "sample updates/s", "frac": nv * TF_NF / (ms / 1e3) / apeak,
                "peak_source": "live probe: two 32-bit shared atomics per update on random bins"}
    traffic = None
    prof = _profile("tlsfold_traffic.json")
    if prof and prof.get("dram_bytes_per_curve"):
        traffic = prof["dram_bytes_per_curve"] * nq
    line = {"metric": METRIC, "value": evals * world / (ms / 1e3), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+i64", "data": "synthetic",
            "config": tlsfold_config(nq) | {"parallelism": "replicas x%d (curves sharded)" % world},
            "roofline": {"bound": "smem", "achieved": achieved / 1e9, "peak": speak / 1e9, "unit": "GB/s",
                         "frac": achieved / speak, "traffic": traffic,
                         "kernel": "tlsfold_kernel (fold + moment arrays + templates)",
                         "kernel_ms": ms, "templates_per_step": tpl,
                         "algorithmic_bytes": "60 B of shared-memory loads per template + 20 B per "
                                              "start bin and frequency",
                         "peak_source": "live probe: conflict-free 64-bit shared-memory loads",
                         "fold": fold_leg},
            "gpu_launches": 2 * args.steps, "clocks": clk}
    if e2e:
        line["e2e"] = e2e
    if not args.no_cpu_baseline:
        line["parity"] = tlsfold_sampled_parity(lcn, tun, outs)
        threads = os.cpu_count() or 1
        nfs = min(TF_NF, 256 * threads)
        v, dt = tlsfold_cpu_sample(lcn, tun, threads, nfs)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": "1 curve x %d frequencies spread over the grid (FP64 oracle, "
                                          "direct sums per template), %.1f s" % (nfs, dt)}
    print(json.dumps(line), flush=True)


def run_tlsfold_reference(args, rank, world):
    """The extension has no reference implementation: the FP64 oracle port on the host."""
    if rank != 0:
        return
    from gtrap_gb300 import synth
    lcn, tun, _ = synth.tess_like(nq=2, n=TF_N, seed=3000)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        tlsfold_cpu_sample(lcn, tun, threads, threads)
    vals, total = [], 0.0
    for _ in range(args.steps):
        v, dt = tlsfold_cpu_sample(lcn, tun, threads, 64 * threads)
        vals.append(v)
        total += dt
    value = float(np.median(vals))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": tlsfold_config(args.nq or 4096),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "per step 1 curve x %d frequencies (FP64 oracle)" % (64 * threads)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- mock injection

MOCK_UNIT = "samples/s"
MOCK_METRIC = "mock transit injection: injected samples/sec"


def _hbm_peak_gbs():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (copy)"
    except Exception:
        return 6800.0, "fallback 6.8 TB/s"


def mock_case(nq, seed):
    from gtrap_gb300 import mock, synth
    lcn, tun, _ = synth.tess_like(nq=nq, n=TF_N, seed=seed)
    lcn = (lcn + np.float32(1.0)).astype(np.float32)  # normalised flux, as the drivers inject into
    rng = np.random.default_rng(seed + 7)
    rs = rng.uniform(0.5, 1.5, nq)
    rec = mock.draw_population(rng, tun, rs, rs ** 1.25, trends=True, lc=lcn)
    return lcn, tun, rec


def mock_cpu_sample(lcn, tun, rec, ncurves):
    """The oracle's injection (scipy quadrature per in-transit sample), one core."""
    import oracle.mock as om
    t0 = time.perf_counter()
    om.inject(lcn[:, :ncurves], tun[:, :ncurves], rec[:ncurves], mode=1)
    dt = time.perf_counter() - t0
    return lcn.shape[0] * ncurves / dt, dt


def run_mock(args, rank, world, local_rank):
    import torch
    import torch.distributed as dist
    from gtrap_gb300 import _build, api
    _build.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.current_stream(dev)
    nq = args.nq or 4096
    lcn, tun, rec = mock_case(nq, 6000 + 100000 * rank)
    lc = torch.from_numpy(lcn).to(dev)
    tu = torch.from_numpy(tun).to(dev)
    # in-place injection repeated on the same image: the same samples and transits every step
    fn = lambda: api.inject_transit(lc, tu, rec, mode=1)
    ms, clk = _timed(fn, args.steps, args.warmup, dev, world)
    samples = TF_N * nq
    e2e = None
    if not args.no_e2e:
        h_lc, h_tu = torch.from_numpy(lcn).pin_memory(), torch.from_numpy(tun).pin_memory()
        h_out = torch.empty_like(h_lc).pin_memory()

        def e2e_step():
            lc.copy_(h_lc, non_blocking=True)
            tu.copy_(h_tu, non_blocking=True)
            fn()
            h_out.copy_(lc, non_blocking=True)

        e2e_step()
        torch.cuda.synchronize(dev)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        for _ in range(args.steps):
            e2e_step()
        e.record(stream)
        torch.cuda.synchronize(dev)
        ems = torch.tensor([s.elapsed_time(e) / args.steps], device=dev, dtype=torch.float64)
        if world > 1:
            dist.all_reduce(ems, op=dist.ReduceOp.MAX)
        e2e = {"value": samples * world / (float(ems[0]) / 1e3), "unit": MOCK_UNIT,
               "h2d_bytes_per_step": (h_lc.numel() + h_tu.numel()) * 4, "d2h_bytes_per_step": h_out.numel() * 4,
               "ms_per_step": float(ems[0]), "api": "gtrap_gb300.api.inject_transit with pinned host buffers"}
    if rank != 0:
        return
    peak, src = _hbm_peak_gbs()
    nbytes = samples * 12.0  # read lc and tu, write lc
    achieved = nbytes / (ms / 1e3) / 1e9
    ph = ((tun - rec["t0"][None, :]) / rec["per"][None, :]) % 1.0
    dur = np.arcsin(np.minimum(1.0, (1.0 + rec["rp"]) / rec["a"])) / (2 * np.pi)
    intransit = float(np.mean((np.minimum(ph, 1.0 - ph) < dur[None, :]) & (tun > 0)))
    line = {"metric": MOCK_METRIC, "value": samples * world / (ms / 1e3), "unit": MOCK_UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "mock injection as the TESS mock driver: %d TESS-like curves x %d samples, "
                                   "one planet per curve (P ~ P^-5/3 on 3..30 d, Rp 0.2..1 R_J, b uniform), "
                                   "lc *= 2 - model, sine and double-cosine trends" % (nq, TF_N),
                       "curves_per_gpu": nq, "in_transit_fraction": intransit,
                       "l2": "inputs %d MiB per GPU exceed L2" % (2 * nq * TF_N * 4 >> 20),
                       "parallelism": "replicas x%d (curves sharded)" % world},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None, "kernel": "inject_kernel", "kernel_ms": ms,
                         "algorithmic_bytes": "12 B per sample (lc and tu read, lc written)", "peak_source": src},
            "gpu_launches": args.steps, "clocks": clk}
    if e2e:
        line["e2e"] = e2e
    if not args.no_cpu_baseline:
        import oracle.mock as om
        fresh = torch.from_numpy(lcn[:, :4].copy()).to(dev)
        got = api.inject_transit(fresh, torch.from_numpy(np.ascontiguousarray(tun[:, :4])).to(dev), rec[:4],
                                 mode=1).cpu().numpy()
        want = om.inject(lcn[:, :4], tun[:, :4], rec[:4], mode=1)
        ulp = np.spacing(np.abs(want).astype(np.float32))
        line["parity"] = {"sample": "4 curves x %d samples injected once (quadrature oracle)" % TF_N,
                          "max_err_in_float32_ulp": float(np.max(np.abs(got - want) / ulp))}
        v, dt = mock_cpu_sample(lcn, tun, rec, 16)
        line["cpu_baseline"] = {"value": v, "unit": MOCK_UNIT, "cores": 1, "kind": "port",
                                "sample": "16 curves x %d samples through the oracle (scipy quadrature per "
                                          "in-transit sample), %.1f s" % (TF_N, dt)}
    print(json.dumps(line), flush=True)


def run_mock_reference(args, rank, world):
    """batman is absent: the oracle port of the injection on one host core."""
    if rank != 0:
        return
    lcn, tun, rec = mock_case(64, 6000)
    for _ in range(args.warmup):
        mock_cpu_sample(lcn, tun, rec, 2)
    vals, total = [], 0.0
    for _ in range(args.steps):
        v, dt = mock_cpu_sample(lcn, tun, rec, 8)
        vals.append(v)
        total += dt
    value = float(np.median(vals))
    line = {"impl": "reference", "metric": MOCK_METRIC, "value": value, "unit": MOCK_UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "mock injection as the TESS mock driver (oracle port; batman is absent)"},
            "cpu_baseline": {"value": value, "unit": MOCK_UNIT, "cores": 1, "kind": "port",
                             "sample": "per step 8 curves x %d samples" % TF_N},
            "e2e": {"value": value, "unit": MOCK_UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- served workload

def run_served(args, rank, world, local_rank):
    """Offered Poisson load swept over fractions of the measured saturation; one JSON line
    with the saturation throughput and p50/p99 latency per offered load, beside the plain
    per-request server."""
    import torch
    from gtrap_gb300 import _build, batch as B, serve as S, synth

    _build.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    npool = args.nq or 1500
    curves = synth.ragged_mix(npool, seed=5000 + 100000 * rank, n_range=(1000, 70000))
    fold = args.tls_kind == "fold"
    if fold:  # TLS-kind curves through the folded search on the BLS frequency rule
        pool = [S.Request("fold", c["t"], c["x"], *fold_grid(c)) if c["kind"] == "tls" else S.Request.from_curve(c)
                for c in curves]
    else:
        pool = [S.Request.from_curve(c) for c in curves]
    fspec = B.FoldSpec(nb=TF_NB, durations=tuple(float(w) for w in TF_DURS), lfrac=TF_LFRAC, dmax=TF_DMAX)
    peaks_only = args.peaks_only
    srv = S.TransitServer(detrend_r=R_MEDIAN, hbm_budget=100e9, fold=fspec, spectrum_stats=peaks_only,
                          tls_peaks={} if peaks_only else None)
    for r in pool[:40]:
        srv.submit(r)
    srv.run_until_idle()
    # results are released as they arrive (a consuming client), in every run below
    res = []
    sat = saturation(S, srv, pool, res)
    plain = S.PlainServer(detrend_r=R_MEDIAN, fold=fspec)
    for r in pool[:10]:
        plain.process(r)
    psat = saturation(S, plain, pool[:300])
    sweep = []
    for frac in (0.1, 0.5, 0.9) if fold or peaks_only else (0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.8, 0.9, 1.0, 1.1, 1.2):
        rate = frac * sat["req_per_s"]
        m = min(npool, max(200, int(rate * 1.5)))
        offs = S.poisson_trace(m, rate, seed=int(frac * 1000))
        s = S.latency_summary(S.serve_trace(srv, pool[:m], offs, keep_outputs=False))
        prate = frac * sat["req_per_s"]
        pm = min(300, max(60, int(prate * 0.5)))
        ps = S.latency_summary(S.serve_trace(plain, pool[:pm], S.poisson_trace(pm, prate, seed=int(frac * 1000)),
                                             keep_outputs=False))
        sweep.append({"offered_frac": frac, "offered_req_per_s": rate, "requests": m,
                      "served_req_per_s": s["req_per_s"], "p50_ms": s["p50_ms"], "p99_ms": s["p99_ms"],
                      "evals_per_s": s["evals_per_s"],
                      "plain": {"requests": pm, "served_req_per_s": ps["req_per_s"],
                                "p50_ms": ps["p50_ms"], "p99_ms": ps["p99_ms"]}})
    # the same requests as one packed batch (detrend, offsets, encoding and one persistent
    # launch per kind, with the server's tile size and block counts): the batched path's rate
    # on identical content, the reference point for the server's saturation
    bat = build_batch(curves, local_rank, tls_kind=args.tls_kind)
    bat.set_config(srv.F)
    bat.launch()
    torch.cuda.synchronize()
    b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    b0.record()
    bat.launch()
    b1.record()
    torch.cuda.synchronize()
    bms = b0.elapsed_time(b1)
    bev = bat.bls_evals + bat.tls_evals + bat.fold_evals
    same_pool = {"what": "the pool's requests as one packed batch (RaggedBatch.launch, the server's tile size "
                         "and block counts, inputs resident, outputs left on the device)",
                 "ms": bms, "evals": bev, "evals_per_s": bev / (bms / 1e3),
                 "served_saturation_frac": sat["evals_per_s"] / (bev / (bms / 1e3))}
    del bat
    if rank != 0:
        return
    # bytes a request returns to the host: full series, or the statistics records
    ret = [r.nbytes for r in res]
    line = {"metric": METRIC, "value": sat["evals_per_s"], "unit": UNIT, "n_gpus": world,
            "steps": 1, "warmup": 1, "ms_per_step": 1e3 * npool / sat["req_per_s"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+i64",
            "data": "synthetic",
            "config": {"workload": "served: Poisson arrivals of single-curve BLS/%s requests (50/50, "
                                   "detrended), n log-uniform [1000, 70000], nf 2k-32k, HBM budget 100 GB"
                                   % ("folded-TLS" if fold else "GTLS"),
                       "pool": npool, "depth": srv.depth, "bls_tiles_per_step": srv.bls_tiles,
                       "tls_tiles_per_step": srv.tls_tiles, "fold_tiles_per_step": srv.fold_tiles,
                       "returns": "statistics records only (get_blsstat / GTLS peak statistics)" if peaks_only
                       else "full spectra and S/N series", "mean_bytes_returned_per_request": float(np.mean(ret))},
            "saturation": sat, "plain_saturation": psat, "batched_same_pool": same_pool, "sweep": sweep,
            "hbm_high_water_bytes": srv.hbm_high_water()}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- epilogue

EPI_METRIC = "BLS/TLS epilogue: curves/sec of the fused statistics, the best-peak refinement and detect_peaks"


def run_epilogue(args, rank, world, local_rank):
    """The steps after the searches, on the outputs of the uneven mix (``--nq`` curves, default
    2000): get_blsstat of every BLS spectrum (gtrap_blsstat_packed), the FP64 refinement of
    every BLS curve's best peak (gtrap_bls_refine_packed, K 32, S 8, M 8), the GTLS peak
    statistics of every S/N series (gtrap_peakstat) and detect_peaks over one 2^20-sample
    series.  Each timed separately with CUDA events (L2 flushed before each call)."""
    import torch
    from gtrap_gb300 import _build, api, batch as B, detect_peaks as DP

    _build.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    nc = args.nq or 2000
    mix = make_mix(nc, 4000 + 100000 * rank)
    bat = build_batch(mix, local_rank)
    B.autotune(bat)
    bat.launch()
    torch.cuda.synchronize(dev)
    rows = {}
    nf_tot = int(sum(int(r["nf"]) for r in bat.bls_table))
    ms, clk = _timed(lambda: bat.bls_stats(), args.steps, args.warmup, dev, world, flush=True)
    hbm, hsrc = _hbm_peak_gbs()
    achieved = 12.0 * nf_tot / (ms / 1e3) / 1e9
    rows["blsstat_packed"] = {"curves": bat.n_bls, "ms": ms, "curves_per_s": bat.n_bls / (ms / 1e3),
                              "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                                           "frac": achieved / hbm, "peak_source": hsrc,
                                           "bytes": "12 B per frequency (SR, start, end read once)"}}
    spec = bat.bls_spec
    refine = lambda: api.bls_refine_packed(bat.blsp, bat.ph1, bat.ph2, bat.bls_curves, bat.t, bat.resid, spec.nb,
                                           spec.kma, spec.kmi, count=bat.n_bls)
    ms, _ = _timed(refine, args.steps, args.warmup, dev, world, flush=True)
    rec = bat.bls_refine()
    gain = rec["sr"][rec["sr_grid"] > 0] / rec["sr_grid"][rec["sr_grid"] > 0]
    rows["bls_refine"] = {"curves": bat.n_bls, "ms": ms, "curves_per_s": bat.n_bls / (ms / 1e3),
                          "trials_per_curve": 65, "sr_gain_median": float(np.median(gain)) if gain.size else None,
                          "sr_gain_p90": float(np.percentile(gain, 90)) if gain.size else None}
    ms, _ = _timed(lambda: bat.tls_peakstat(), args.steps, args.warmup, dev, world, flush=True)
    rows["peakstat"] = {"curves": bat.n_tls, "ms": ms, "curves_per_s": bat.n_tls / (ms / 1e3),
                        "epochs": bat.tls_evals}
    x = np.random.default_rng(7).normal(size=1 << 20)
    xd = torch.from_numpy(x).to(dev)
    ms, _ = _timed(lambda: DP.detect_peaks(xd, mpd=10), args.steps, args.warmup, dev, world, flush=True)
    rows["detect_peaks"] = {"samples": x.size, "ms": ms, "samples_per_s": x.size / (ms / 1e3)}
    if rank != 0:
        return
    total_ms = rows["blsstat_packed"]["ms"] + rows["bls_refine"]["ms"] + rows["peakstat"]["ms"]
    value = (bat.n_bls + bat.n_tls) / (total_ms / 1e3)
    line = {"metric": EPI_METRIC, "value": value, "unit": "curves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64+f32", "data": "synthetic",
            "config": {"workload": "epilogue of the uneven mix (%d curves: %d BLS spectra, %d GTLS S/N series)"
                                   % (nc, bat.n_bls, bat.n_tls), "l2": "flushed before each timed call"},
            "kernels": rows, "gpu_launches": 6 * args.steps, "clocks": clk}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- trapezoid grid fit

FIT_UNIT = "templates/s"
FIT_METRIC = "trapezoid grid fit (gtrap/tls.py tlsfit): (W, L, t0) templates/sec"
FIT_W = np.linspace(0.5, 8.0, 8) / 24.0       # widths 0.5 .. 8 h (days)
FIT_L = np.linspace(2.0, 30.0, 8) / 1440.0    # ingress 2 .. 30 min (days)
FIT_STRIDE = 4                                # epochs: every fourth valid sample time
FIT_FLOPS = 10.0                              # FP64 flops per (template, window sample)


def fit_case(rank=0):
    """One TESS-like curve of config 3's shape (18,000 samples at 2 min, a 1-day gap, a
    trapezoid) and the epoch grid."""
    from gtrap_gb300 import synth
    lcn, tun, _ = synth.tess_like(nq=1, n=18000, seed=3000 + 100000 * rank, transit_frac=1.0)
    t = tun[:, 0].astype(np.float64)
    x = lcn[:, 0].astype(np.float64)
    return t, x, t[t >= 0][::FIT_STRIDE]


def fit_config(nT):
    return {"workload": "trapezoid grid fit of gtrap/tls.py (tlsfit: get_chi2Hmax over W x L x t0, FP64): one "
                        "TESS-like curve of 18000 samples at 2 min with a 1-day gap; W 8 values 0.5..8 h, L 8 "
                        "values 2..30 min, t0 every fourth sample time (%d); %d templates" % (nT, 64 * nT),
            "templates": 64 * nT, "l2": "inputs 0.3 MiB fit in L2: a 256 MiB buffer is written before every "
                                        "timed step, outside its CUDA events"}


def fit_window_samples(t, tl):
    """Samples in each template's window (t - t0 in [min(-W/2, -W/4-L/2), max(W/2, W/4+L/2)])."""
    ts = np.sort(t[np.isfinite(t)])
    tot = 0
    for W in FIT_W:
        for L in FIT_L:
            lo = tl + min(-W / 2, -W / 4 - L / 2)
            hi = tl + max(W / 2, W / 4 + L / 2)
            tot += int((np.searchsorted(ts, hi, "right") - np.searchsorted(ts, lo, "left")).sum())
    return tot


def fit_cpu_sample(t, x, tl, seconds):
    """The reference's algorithm (oracle port of gtrap/tls.py get_chi2Hmax, NumPy, one core)
    over templates spread through the grid until ``seconds`` pass.  Returns (templates/s, count,
    seconds)."""
    from oracle import tls_cpu
    rng = np.random.default_rng(5)
    cnt, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        W, L, T = FIT_W[rng.integers(8)], FIT_L[rng.integers(8)], tl[rng.integers(tl.size)]
        tls_cpu.get_chi2Hmax(t, x, W, L, T)
        cnt += 1
    dt = time.perf_counter() - t0
    return cnt / dt, cnt, dt


def fit_sampled_parity(t, x, tl, H, res):
    """Sampled grid points against the oracle: max relative error of H and chi^2."""
    from oracle import tls_cpu
    rng = np.random.default_rng(9)
    nT = tl.size
    eh = er = 0.0
    for k in rng.choice(H.size, 48, replace=False):
        iW, iL, iT = k // (8 * nT), (k // nT) % 8, k % nT
        oh, ores, _, _ = tls_cpu.get_chi2Hmax(t, x, FIT_W[iW], FIT_L[iL], tl[iT])
        if np.isfinite(oh):
            eh = max(eh, abs(H[k] - oh) / max(abs(oh), 1e-300))
            er = max(er, abs(res[k] - ores) / max(abs(ores), 1e-300))
    return {"sample": "48 grid points (FP64 oracle)", "h_max_err_rel": eh, "chi2_max_err_rel": er}


def fp64_peak_tflops(dev):
    """FP64 FMA issue peak of this GPU, measured live (MEASURED_PEAKS.json has no FP64 figure)."""
    import bench_probes
    return bench_probes.fp64_tflops(dev)


def run_tlsfit(args, rank, world, local_rank):
    import torch
    from gtrap_gb300 import _build, _native as N, tls
    from gtrap_gb300._dev import as_ptr
    _build.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    t, x, tl = fit_case(rank)
    ts, xs = tls._sorted_series(t, x, dev)
    Wd, Ld, Td = (tls._d64(v, dev) for v in (FIT_W, FIT_L, tl))
    k = 64 * tl.size
    H = torch.empty(k, dtype=torch.float64, device=dev)
    res, xsum, sn = torch.empty_like(H), torch.empty_like(H), torch.empty_like(H)
    npts = torch.empty(k, dtype=torch.int32, device=dev)
    idx = torch.empty(1, dtype=torch.int64, device=dev)
    h = torch.cuda.current_stream(dev).cuda_stream

    def fn():
        N.call("gtrap_tlsfit_grid", as_ptr(ts), as_ptr(xs), ts.numel(), as_ptr(Wd), 8, as_ptr(Ld), 8, as_ptr(Td),
               tl.size, 1.0, 1, as_ptr(H), as_ptr(res), as_ptr(npts), as_ptr(xsum), as_ptr(sn), h)
        N.call("gtrap_nanargmax", as_ptr(sn), k, as_ptr(idx), h)

    ms, clk = _timed(fn, args.steps, args.warmup, dev, world, flush=True)
    value = k * world / (ms / 1e3)
    e2e = None
    if not args.no_e2e:  # the drop-in call from host arrays: upload, sort, grid, argmax, model, download
        tls.tlsfit(t, x, FIT_W, FIT_L, tl)
        torch.cuda.synchronize(dev)
        w0 = time.perf_counter()
        for _ in range(args.steps):
            out = tls.tlsfit(t, x, FIT_W, FIT_L, tl)
        e_ms = 1e3 * (time.perf_counter() - w0) / args.steps
        e2e = {"value": k * world / (e_ms / 1e3), "unit": FIT_UNIT, "ms_per_step": e_ms,
               "h2d_bytes_per_step": 16 * t.size + 8 * (16 + tl.size) + 8 * t.size,
               "d2h_bytes_per_step": 8 * t.size + 8 * 3 + 8,
               "api": "gtrap_gb300.tls.tlsfit on host NumPy arrays (timed on the host clock; the call "
                      "synchronises when it returns its scalars)",
               "best": {"W": float(out[2]), "L": float(out[3]), "T0": float(out[4]), "H": float(out[1])}}
    if rank != 0:
        return
    peak = fp64_peak_tflops(dev)
    flops = FIT_FLOPS * fit_window_samples(t, tl)
    achieved = flops / (ms / 1e3) / 1e12
    line = {"metric": FIT_METRIC, "value": value, "unit": FIT_UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": fit_config(tl.size) | {"parallelism": "replicas x%d" % world},
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak,
                         "traffic": (_profile("tlsfit_traffic.json") or {}).get("dram_bytes_per_launch"),
                         "kernel": "tlsfit_kernel (one thread per template) + nanargmax_kernel",
                         "algorithmic_flops": "%g FP64 flops per (template, window sample): mean, region sums "
                                              "and residual passes" % FIT_FLOPS,
                         "peak_source": "live FP64 FMA-chain probe on this GPU (MEASURED_PEAKS.json has no FP64 "
                                        "figure)"},
            "gpu_launches": 2 * args.steps, "clocks": clk}
    line["parity"] = fit_sampled_parity(t, x, tl, H.cpu().numpy(), res.cpu().numpy())
    if e2e:
        line["e2e"] = e2e
    if not args.no_cpu_baseline:
        v, cnt, dt = fit_cpu_sample(t, x, tl, 10.0)
        line["cpu_baseline"] = {"value": v, "unit": FIT_UNIT, "cores": 1, "kind": "port",
                                "sample": "%d templates spread over the grid, one core, NumPy oracle port of "
                                          "get_chi2Hmax (as the reference), %.1f s" % (cnt, dt)}
    print(json.dumps(line), flush=True)


def run_tlsfit_reference(args, rank, world):
    """The reference's CPU path: the NumPy port of get_chi2Hmax on one core (tlsfit has no
    threading), a bounded sample of templates per step."""
    if rank != 0:
        return
    t, x, tl = fit_case()
    for _ in range(args.warmup):
        fit_cpu_sample(t, x, tl, 0.2)
    vals, total, cnt = [], 0.0, 0
    for _ in range(args.steps):
        v, c, dt = fit_cpu_sample(t, x, tl, 2.0)
        vals.append(v)
        total += dt
        cnt += c
    value = float(np.median(vals))
    line = {"impl": "reference", "metric": FIT_METRIC, "value": value, "unit": FIT_UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": fit_config(tl.size),
            "cpu_baseline": {"value": value, "unit": FIT_UNIT, "cores": 1, "kind": "port",
                             "sample": "per step about 2 s of templates spread over the grid (%d in all)" % cnt},
            "e2e": {"value": value, "unit": FIT_UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_lone(args, rank, world, local_rank):
    """Lone requests: each of six requests (BLS and GTLS requests of about 5k, 20k and 60k
    samples from the served pool's distribution) submitted to an idle server and run to
    completion, ``--steps`` times, beside the plain per-request path on the same requests.
    ``value`` is the evaluations of the requests over the sum of their median latencies."""
    import torch
    from gtrap_gb300 import _build, serve as S, synth

    _build.build()
    torch.cuda.set_device(local_rank)
    curves = synth.ragged_mix(400, seed=5000 + 100000 * rank, n_range=(1000, 70000))
    pool = [S.Request.from_curve(c) for c in curves]
    srv = S.TransitServer(detrend_r=R_MEDIAN, hbm_budget=100e9)
    plain = S.PlainServer(detrend_r=R_MEDIAN)
    for r in pool[:40]:
        srv.submit(r)
    srv.run_until_idle()
    for r in pool[:10]:
        plain.process(r)
    torch.cuda.synchronize()
    picks = []
    for kind in ("bls", "tls"):
        for target in (5000, 20000, 60000):
            picks.append(min((i for i in range(len(pool)) if pool[i].kind == kind),
                             key=lambda i: abs(pool[i].n - target)))
    rows, ev_sum, lat_sum = [], 0, 0.0
    for _ in range(args.warmup):
        for k in picks:
            srv.submit(pool[k])
            srv.run_until_idle()
            plain.process(pool[k])
    for k in picks:
        r = pool[k]
        lat, plat = [], []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            srv.submit(r, t0)
            res = srv.run_until_idle()
            lat.append(1e3 * (res[0].done - t0))
            t0 = time.perf_counter()
            pr = plain.process(r, t0)
            plat.append(1e3 * (pr.done - t0))
        ev = r.outputs
        ev_sum += ev
        lat_sum += float(np.median(lat)) / 1e3
        rows.append({"kind": r.kind, "n": r.n, "evals": ev, "server_ms_p50": float(np.median(lat)),
                     "server_ms_min": float(min(lat)), "plain_ms_p50": float(np.median(plat)),
                     "plain_ms_min": float(min(plat))})
    if rank != 0:
        return
    line = {"metric": METRIC, "value": ev_sum / lat_sum, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * lat_sum, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+i64", "data": "synthetic",
            "config": {"workload": "lone requests: one BLS or GTLS request at a time (detrended; about 5k, 20k "
                                   "and 60k samples each) through an idle TransitServer and through PlainServer",
                       "requests": len(rows)},
            "requests": rows}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if args.workload in ("served", "lone"):
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the reference has no serving loop or "
                                  "per-request path (its drivers launch one kernel per image); its CPU rate on "
                                  "the same mix is the default workload's reference arm"}), flush=True)
            return
        if args.workload == "masked":
            run_masked_reference(args, rank, world)
        elif args.workload == "tlsfold":
            run_tlsfold_reference(args, rank, world)
        elif args.workload == "mock":
            run_mock_reference(args, rank, world)
        elif args.workload == "tlsfit":
            run_tlsfit_reference(args, rank, world)
        else:
            run_ragged_reference(args, rank, world)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    try:
        {"ragged": run_ragged, "masked": run_masked, "served": run_served, "lone": run_lone, "plain": run_image,
         "tls": run_image, "tlsfold": run_tlsfold, "mock": run_mock, "tlsfit": run_tlsfit,
         "epilogue": run_epilogue}[args.workload](
            args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
