"""Benchmark of The Joker's rejection hot path on GB300.

Workload (one step): one star with 40 RV epochs over 3000 d (sigma ~ U(0.05,
0.5) km/s, Keplerian signal + noise, jitter applied with s ~ LogNormal(ln 0.5,
1) km/s per prior sample) against a device-resident prior cache of 2^28
samples (P log-uniform [2, 1024] d, e ~ Beta(0.867, 3.03), omega, M0 ~
U[0, 2 pi)); the marginal ln L of every sample plus the acceptance test
exp(lnL - max) > u against the caller's numpy PCG64 uniforms.  Seeded
synthetic inputs stand in for survey data.

metric: prior samples/s (lnL + accept).  ``value``: mixed-precision path, inputs
resident in HBM.  ``e2e``: the same through the host-facing call -- the packed
(S, 5) float64 chunk in pinned host memory, read by the ln L kernel over the
host link (40 bytes per sample, no staging copy), evaluated and accepted,
accepted indices copied back -- every step.  The plain FP64 GPU path is
reported beside it (``fp64``) on a 2^25-sample slice of the same workload,
with ``parity`` against it on that slice.  At N = 1 the line also carries one
pass of the other configurations: ``batched`` (4096 stars over one 2^24
cache), ``iterative`` (1024 stars, quadratic trend, graph rounds) and
``serving`` (a Poisson request stream, p50/p99), each beside the FP64 path.

Multi-GPU (torchrun): each rank evaluates its own 2^28-sample shard of the
cache for the same star (weak scaling); the per-star maximum is exchanged with
one all-reduce(max) before the acceptance pass.

``--impl reference`` times the reference's own CPU likelihood (the unmodified
Cython CJokerHelper compiled into oracle/_ref, else the C restatement in
oracle/) over a process pool of all host cores, on a bounded sample.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

N_EPOCHS = 40
SPAN_D = 3000.0
# precision of the mixed path timed in every mode ("mixed_fast": FP32 epoch
# sums, the first pass of the refined acceptance; "mixed": float-float sums);
# set from --precision
MIXED = "mixed_fast"
SEED_STAR = 2
SEED_CACHE = 0


# ------------------------------------------------------------------ workload
def make_star():
    from thejoker_gb300.linear import rv_unit_columns
    rng = np.random.default_rng(SEED_STAR)
    t = np.sort(2456000.0 + rng.uniform(0, SPAN_D, N_EPOCHS))
    err = rng.uniform(0.05, 0.5, N_EPOCHS)
    P = np.exp(rng.uniform(np.log(2), np.log(1024)))
    e = rng.beta(0.867, 3.03)
    om, M0 = rng.uniform(0, 2 * np.pi), rng.uniform(0, 2 * np.pi)
    K = 30.0 * (P / 365.25) ** (-1 / 3) / np.sqrt(1 - e ** 2) * rng.normal()
    rv = K * rv_unit_columns(t, t.min(), [P], [e], [om], [M0])[0] + rng.normal(0, 100.0) \
        + rng.normal(0, np.sqrt(err ** 2 + 0.5 ** 2))
    return dict(t=t, rv=rv, ivar=1 / err ** 2, t_ref=t.min(), trend_M=np.ones((N_EPOCHS, 1)),
                mu=np.zeros(2), lam=np.array([0.0, 100.0 ** 2]),
                k_prior=np.array([1.0, 30.0, 365.25, 500.0]))


def fill_cache_host(out, seed, threads=16):
    """Prior samples (P, e, omega, M0, s) into ``out`` (n x 5 float64), drawn
    in parallel blocks from independent numpy generators."""
    from concurrent.futures import ThreadPoolExecutor
    n = out.shape[0]
    nblk = max(1, min(threads * 4, n // 65536))
    bounds = np.linspace(0, n, nblk + 1).astype(np.int64)
    seqs = np.random.SeedSequence(seed).spawn(nblk)

    def work(i):
        a, b = bounds[i], bounds[i + 1]
        r = np.random.default_rng(seqs[i])
        m = b - a
        out[a:b, 0] = np.exp(r.uniform(np.log(2.0), np.log(1024.0), m))
        out[a:b, 1] = r.beta(0.867, 3.03, m)
        out[a:b, 2] = r.uniform(0, 2 * np.pi, m)
        out[a:b, 3] = r.uniform(0, 2 * np.pi, m)
        out[a:b, 4] = np.exp(r.normal(np.log(0.5), 1.0, m))

    with ThreadPoolExecutor(threads) as ex:
        list(ex.map(work, range(nblk)))
    return out


# Algorithmic work per unit, fixed for the roofline (roofline.frac): per
# (sample, epoch) F_epoch = 4 (phase: sub, mul, floor, fma) + 6 I_K (Newton
# steps, sincos counted as 2, I_K = 4 nominal) + 12 (true anomaly and RV
# column) + 2 (L(L+1)/2 + L + 1) (moment FMAs) = 62 at L = 2; per sample
# F_sample = L^3/3 + 2 L^2 + 10 (Cholesky, solve, log-det, K variance,
# accept) = 21 at L = 2.
FLOPS_PER_EPOCH = 62
FLOPS_PER_SAMPLE = 21
# FP32 operations each mixed kernel issues per (sample, epoch) with the jitter
# applied at L = 2, counted from its source (FMA = 2 flops, special-function
# ops = 1), and per sample for the setup and the tail (roofline.issued_frac):
# float-float sums (mixed) and FP32 sums (mixed_fast: about 110 for the
# out-of-reach test after the last epoch; the float-float tail and error
# bound, 420 more, run only for the warps within reach of the maximum and are
# left out of this count).
ISSUED_FLOPS = {"mixed": (196, 60), "mixed_fast": (126, 110)}
KERNEL_NAME = {"mixed": "lnl_mixed2_kernel<L=2, jitter, VAR 0, cache form> (two samples per "
                        "thread, paired FP32, float-float sums)",
               "mixed_fast": "lnl_fast2_kernel<L=2, jitter, cache form, fused acceptance> (two "
                             "samples per thread, paired FP32, FP32 sums re-centred on the "
                             "trend fit; each sample's PCG64 uniform and candidate bit)"}
# Algorithmic HBM bytes per sample of the cache-form mixed kernel (36 B prepared
# sample read, 8 B ln L + 4 B bound written, and for the fused pass 1 bit of
# candidate mask) and the DRAM bytes ncu measured per sample (read + write of
# one 2^24-sample launch / 2^24), scaled to a launch.
BYTES_PER_SAMPLE = 48.125
DRAM_BYTES_PER_SAMPLE = 46.90


def _hbm_peak():
    """(GB/s, source): the measured copy bandwidth of the GB300
    (MEASURED_PEAKS.json), else the 6800 GB/s fallback."""
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (measured)"
    except Exception:
        return 6800.0, "fallback 6800 GB/s (MEASURED_PEAKS.json absent)"


# ------------------------------------------------------------------- clocks
class ClockSampler:
    """SM clocks and throttle reasons sampled every 50 ms by one streaming
    ``nvidia-smi -lms`` process while the block runs (read only; no setting
    is changed)."""

    def __init__(self, gpu_index, interval_ms=50):
        self.gpu = gpu_index
        self.interval_ms = int(interval_ms)
        self.samples = []
        self._proc = None
        self._th = None

    def _read(self):
        for line in self._proc.stdout:
            v = [x.strip() for x in line.strip().split(",")]
            if len(v) >= 6:
                self.samples.append(v)

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={q}",
                 "--format=csv,noheader,nounits", "-lms", str(self.interval_ms)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._th = threading.Thread(target=self._read, daemon=True)
            self._th.start()
            # let the stream start before the timed block
            t_end = time.time() + 2.0
            while not self.samples and time.time() < t_end:
                time.sleep(0.02)
            self.samples.clear()
        except Exception:
            self._proc = None
        return self

    def __exit__(self, *a):
        if self._proc is not None:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except Exception:
                self._proc.kill()
            self._th.join(timeout=5)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 2 + i and s[2 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "n_samples": len(self.samples)}


# ------------------------------------------------------------ CPU baseline
def _cpu_worker(args):
    kind, star, chunk = args
    if kind == "reference":
        from oracle import ref_cython
        h = ref_cython.make_helper(star["t"], star["rv"], star["ivar"], star["t_ref"],
                                   star["trend_M"], 1, 0, star["mu"], np.sqrt(star["lam"]),
                                   True, *star["k_prior"][1:])
        return np.array(h.batch_marginal_ln_likelihood(np.ascontiguousarray(chunk)))
    from oracle import oracle
    return oracle.batch_marginal_ln_likelihood(
        star["t"], star["rv"], star["ivar"], star["t_ref"], star["trend_M"], star["mu"],
        star["lam"], chunk, True, *star["k_prior"][1:], jitter=True)


def cpu_baseline(star, n_samples, seed=1):
    """Time the CPU likelihood + accept over a process pool of all cores on a
    bounded sample; returns (samples/s, kind, cores, seconds)."""
    import multiprocessing as mp
    from oracle import build as ob, ref_cython
    ob.build_all()
    kind = "reference" if ref_cython.available() else "port"
    cores = os.cpu_count() or 1
    chunk = np.empty((n_samples, 5))
    fill_cache_host(chunk, seed)
    tasks = [(kind, star, c) for c in np.array_split(chunk, cores * 4)]
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        pool.map(_cpu_worker, tasks[:cores])          # warm the workers
        t0 = time.perf_counter()
        lls = np.concatenate(pool.map(_cpu_worker, tasks))
        uu = np.random.default_rng(seed).uniform(size=len(lls))
        np.where(np.exp(lls - lls.max()) > uu)
        dt = time.perf_counter() - t0
    return n_samples / dt, kind, cores, dt


# ---------------------------------------------------------------- GPU path
def run_ours(args, rank, world, dist):
    import torch
    from thejoker_gb300 import build as tb
    from thejoker_gb300 import device as dev

    tb.build()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    S = args.samples
    star = make_star()
    table = dev.StarTable([star], jitter="applied")

    # host chunk (pinned) for this rank's shard, and the resident cache
    host = torch.empty((S, 5), dtype=torch.float64).pin_memory()
    fill_cache_host(host.numpy(), SEED_CACHE + rank)
    cache = dev.PriorCache(S)
    stage = torch.empty((args.h2d_chunk, 5), dtype=torch.float64, device="cuda")
    for a in range(0, S, args.h2d_chunk):
        b = min(S, a + args.h2d_chunk)
        stage[: b - a].copy_(host[a:b], non_blocking=True)
        cache.load(stage[: b - a], row0=a)
    torch.cuda.synchronize()
    from thejoker_gb300.batch import BatchRejection
    from thejoker_gb300.parallel import ShardedRejection
    gen = np.random.default_rng(1000)
    pcg_state, pcg_inc = dev.pcg64_state(gen)
    del stage
    torch.cuda.empty_cache()
    # work-item size from the autotuner, measured here on this workload
    from thejoker_gb300 import autotune
    tuned, tune_ms = autotune.tune(table, cache, precision=MIXED, count=min(S, 1 << 26),
                                   reps=2)
    if world > 1:
        runner = ShardedRejection(table, cache, row0=rank * S, precision=MIXED, max_out=S)
    else:
        runner = BatchRejection(table, cache, precision=MIXED, max_out=S, seeds=[1000],
                                timing=True)
    lnl_ms = []

    def step():
        if world > 1:
            return runner.run((pcg_state, pcg_inc))
        runner.run()

    def barrier():
        if dist is not None and world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- value: inputs resident
    for _ in range(args.warmup):
        step()
    barrier()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    from thejoker_gb300 import _native as nat
    with ClockSampler(int(os.environ.get("LOCAL_RANK", 0))) as clk:
        barrier()
        launches0 = nat.lib().joker_launch_count()
        t0.record()
        for _ in range(args.steps):
            step()
        t1.record()
        barrier()
        launches = nat.lib().joker_launch_count() - launches0
    ms = t0.elapsed_time(t1) / args.steps
    early = None
    if world == 1:
        lnl_ms.append(runner.lnl_ms())
        n_acc = int(runner.counts[0].item())
        if MIXED == "mixed_fast":
            early = early_exit_measure(runner, table, cache, S, args.steps, args.warmup)
    else:
        lnl_ms.append(float("nan"))
        n_acc = None

    # ---- e2e: pinned host chunk -> device (sliced, copies overlapped with the
    # preparation and ln L of the previous slice) -> acceptance -> host indices
    from thejoker_gb300.pipeline import HostRejection
    if world == 1:
        del runner, cache
        torch.cuda.empty_cache()
        hr = HostRejection(table, S, precision=MIXED, slice_rows=args.h2d_chunk, max_out=S)

        def e2e_step():
            hr.run(host, [(pcg_state, pcg_inc)])
            return hr.d2h_bytes
    else:
        # each rank streams its shard into its cache, then the sharded pass
        # exchanges the maximum and accepts
        stage = torch.empty((args.h2d_chunk, 5), dtype=torch.float64, device="cuda")

        def e2e_step():
            for a0 in range(0, S, args.h2d_chunk):
                b0 = min(S, a0 + args.h2d_chunk)
                stage[: b0 - a0].copy_(host[a0:b0], non_blocking=True)
                cache.load(stage[: b0 - a0], row0=a0)
            idx, _ = runner.run((pcg_state, pcg_inc))
            return len(idx) * 8 + 8
    for _ in range(max(1, args.warmup // 2)):
        e2e_step()
    barrier()
    te0 = time.perf_counter()
    for _ in range(args.steps):
        d2h = e2e_step()
    barrier()
    e2e_ms = (time.perf_counter() - te0) * 1e3 / args.steps
    if world == 1:
        del hr
    else:
        del runner, cache, stage
    torch.cuda.empty_cache()
    cache = dev.PriorCache(min(S, args.fp64_samples)).load(host[:min(S, args.fp64_samples)].cuda())

    # ---- plain FP64 GPU path on a slice of the same workload (ln L + accept)
    S64 = min(S, args.fp64_samples)
    b64 = BatchRejection(table, cache, precision="fp64", max_out=S64, seeds=[1000])
    b64.run(count=S64)
    barrier()
    f0 = time.perf_counter()
    for _ in range(2):
        b64.run(count=S64)
    barrier()
    fp64_ms = (time.perf_counter() - f0) * 1e3 / 2

    # ---- parity of the mixed path on the same slice (after the timed region)
    parity = _parity_slice(table, cache, b64, S64) if world == 1 else None
    del b64, cache
    torch.cuda.empty_cache()

    # ---- max over ranks
    def gmax(x):
        if dist is None or world == 1:
            return x
        tt = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        return float(tt.item())

    ms, e2e_ms, fp64_ms = gmax(ms), gmax(e2e_ms), gmax(fp64_ms)
    kern_ms = float(np.median(lnl_ms))
    if rank != 0:
        return None
    total = S * world
    flops = S * (N_EPOCHS * FLOPS_PER_EPOCH + FLOPS_PER_SAMPLE)
    achieved = flops / (kern_ms * 1e-3) / 1e12
    ipe, ips = ISSUED_FLOPS[MIXED]
    issued = S * (N_EPOCHS * ipe + ips)
    peak = args.fp32_peak
    hbm_peak, hbm_src = _hbm_peak()
    line = {
        "metric": "prior samples/s (lnL+accept)",
        "value": total / (ms * 1e-3),
        "unit": "samples/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+f64 (mixed)",
        "data": "synthetic (seeded; prior cache and star drawn with numpy)",
        "config": {"workload": f"1 star x {N_EPOCHS} epochs over {SPAN_D:.0f} d, jitter "
                               f"applied, prior cache 2^{int(math.log2(S))} samples per GPU",
                   "prior_samples_per_gpu": S, "n_epochs": N_EPOCHS, "n_linear": 2,
                   "l2": "inputs larger than L2 (cache 76 B/sample resident, 2^28 samples)",
                   "precision": MIXED, "u_source": "numpy PCG64 stream regenerated on device",
                   "accept": "refined to the FP64 decisions; first pass fused into the ln L "
                             "kernel" if MIXED == "mixed_fast" else
                             "refined to the FP64 decisions",
                   "autotune": {"chunk": tuned, "ms_per_2^26_samples": tune_ms}},
        "e2e": {"value": total / (e2e_ms * 1e-3), "unit": "samples/s",
                "h2d_bytes_per_step": S * 40, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_ms},
        "fp64": {"value": S64 * world / (fp64_ms * 1e-3), "unit": "samples/s",
                 "samples": S64, "ms_per_step": fp64_ms},
        "accepted_per_step": n_acc,
        "gpu_launches": int(launches),
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak,
                     "work": f"algorithmic: {FLOPS_PER_EPOCH} flops per (sample, epoch) + "
                             f"{FLOPS_PER_SAMPLE} per sample (L = 2)",
                     "issued_tflops": issued / (kern_ms * 1e-3) / 1e12,
                     "issued_frac": issued / (kern_ms * 1e-3) / 1e12 / peak,
                     "issued_work": f"FP32 operations issued, counted from the kernel source: "
                                    f"{ipe} per (sample, epoch) + about {ips} per sample (the "
                                    f"float-float tail, 420 more, only for warps within reach "
                                    f"of the maximum, not counted)" if MIXED == "mixed_fast" else
                                    f"FP32 operations issued, counted from the kernel source: "
                                    f"{ipe} per (sample, epoch) + {ips} per sample",
                     "traffic": args.traffic if args.traffic else DRAM_BYTES_PER_SAMPLE * S,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one "
                                       "2^24-sample launch, scaled by samples",
                     "hbm": {"achieved_gbs": BYTES_PER_SAMPLE * S / (kern_ms * 1e-3) / 1e9,
                             "peak_gbs": hbm_peak,
                             "frac": BYTES_PER_SAMPLE * S / (kern_ms * 1e-3) / 1e9 / hbm_peak,
                             "peak_source": hbm_src},
                     "kernel": KERNEL_NAME[MIXED],
                     "kernel_ms": kern_ms,
                     "peak_source": "FP32 FMA throughput measured on a GB300: independent FMA "
                                    "chains, 74.9 TFLOP/s paired (73.1 scalar)",
                     "flops_per_launch": flops},
        "clocks": clk.summary(),
        "parity": parity,
    }
    if early is not None:
        line["early_exit"] = early
    if not args.no_cpu:
        v, kind, cores, secs = cpu_baseline(star, args.cpu_samples)
        line["cpu_baseline"] = {"value": v, "unit": "samples/s", "cores": cores, "kind": kind,
                                "sample": f"{args.cpu_samples} prior samples of the same star "
                                          f"({secs:.1f} s wall); the reference ignores jitter"}
    if world == 1 and not args.headline_only:
        # the 4096-star configuration and the serving stream, one pass each
        del host
        torch.cuda.empty_cache()
        line["batched"] = batched_measure(4096, 1 << 24, warmup=1, steps=1, subset_stars=64,
                                          subset_samples=1 << 22)
        torch.cuda.empty_cache()
        torch.cuda.empty_cache()
        line["iterative"] = iterative_measure(1024, 1 << 22, 256, steps=1, warmup=1,
                                              subset_stars=64, eager=False)
        torch.cuda.empty_cache()
        line["serving"] = serving_measure(1 << 28, rates=[500.0], window=4.0, n_all=2000,
                                          slots=1024, round_budget=1 << 26, fp64_requests=64)
    return line


def early_exit_measure(runner, table, cache, S, steps, warmup):
    """The same step with the fused pass's early exit (not the headline): warps
    whose samples the partial epoch sums put more than 746 nats below the
    running lower bound stop evaluating epochs.  The kept rows and their ln L
    must equal the full step's (``identical``)."""
    import torch
    from thejoker_gb300.batch import BatchRejection
    c0, i0, l0 = runner.results()
    ex = BatchRejection(table, cache, precision=MIXED, max_out=S, seeds=[1000], timing=True,
                        early_exit=True)
    for _ in range(max(1, warmup)):
        ex.run()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(int(os.environ.get("LOCAL_RANK", 0))) as clk:
        t0.record()
        for _ in range(steps):
            ex.run()
        t1.record()
        torch.cuda.synchronize()
    ms = t0.elapsed_time(t1) / steps
    c1, i1, l1 = ex.results()
    stopped = float(torch.isinf(ex.err[0, :S]).float().mean().item())
    same = bool(np.array_equal(c0, c1) and np.array_equal(i0[0], i1[0]) and
                np.array_equal(l0[0], l1[0]))
    del ex
    torch.cuda.empty_cache()
    return {"value": S / (ms * 1e-3), "unit": "samples/s", "ms_per_step": ms,
            "samples_stopped_early": stopped, "identical": same,
            "note": "opt-in (early_exit=True), not the headline: samples rejected for every "
                    "uniform by an upper bound from their first 8..96 epochs are not evaluated "
                    "further; kept rows and their ln L are the full step's",
            "clocks": clk.summary()}


def _parity_slice(table, cache, b64, S):
    """The mixed path against the plain FP64 path on the first S rows of the
    workload: |d ln L| before and after the band refinement (samples within
    JOKER_MIXED_LNL_BAND of the maximum), the raw error against its bound
    everywhere, and the accepted indices of both paths (same uniforms)."""
    import torch
    from thejoker_gb300 import device as dev
    from thejoker_gb300 import _native as nat
    from thejoker_gb300.batch import BatchRejection
    l64 = torch.empty((1, S), dtype=torch.float64, device="cuda")
    dev.lnl(table, cache, l64, precision="fp64", count=S)
    lm = torch.empty((1, S), dtype=torch.float64, device="cuda")
    err = torch.empty((1, S), dtype=torch.float32, device="cuda")
    bk = dev.MaxKeys(2)
    dev.lnl(table, cache, lm, precision=MIXED, count=S, err=err, bound_keys=bk)
    raw, eraw = lm.clone(), err.clone()
    seg = [dict(lnl_off=0, n=S, out_off=0, max_out=0, max_slot=0, star=0, row0=0)]
    exact, n1 = dev.refine_max(table, cache, lm.view(-1), err.view(-1), bk, seg)
    n2 = dev.refine_band(table, cache, lm.view(-1), err.view(-1), exact, seg)
    a64, ar, ab = (x.view(-1).cpu().numpy() for x in (l64, raw, lm))
    band_nats = nat.JOKER_MIXED_LNL_BAND
    mx = a64.max()
    band = a64 >= mx - band_nats
    bm = BatchRejection(table, cache, precision=MIXED, max_out=S, seeds=[1000])
    bm.run(count=S)
    c64, i64, l64k = b64.results()
    cm, im, lmk = bm.results()
    same = bool(c64[0] == cm[0] and np.array_equal(i64[0], im[0]))
    # the raw values against their own bounds, as the ln L kernel wrote both
    # (the refinements tighten or zero the bounds of the samples they touch)
    ev = eraw.view(-1).cpu().numpy()
    kept_bound = ev > 0
    over = np.abs(ar - a64)[kept_bound] / ev[kept_bound]
    return {"rows": int(S), "band_nats": band_nats, "tol": nat.JOKER_MIXED_LNL_TOL,
            "samples_in_band": int(band.sum()),
            "max_abs_dlnl_in_band": float(np.abs(ab - a64)[band].max()),
            "max_abs_dlnl_in_band_raw": float(np.abs(ar - a64)[band].max()),
            "max_abs_dlnl_all_raw": float(np.nanmax(np.abs(ar - a64))),
            "max_dlnl_over_bound": float(np.nanmax(over)) if over.size else 0.0,
            "fp64_refined": int((n1 + n2).item()),
            "max_abs_dmax": float(abs(exact.values()[0] - mx)),
            "accepted": int(c64[0]), "accept_identical": same,
            "max_abs_dlnl_kept": float(np.max(np.abs(lmk[0] - l64k[0]))) if same and
            len(lmk[0]) else 0.0}


def batched_measure(n_stars, S, warmup=1, steps=1, subset_stars=64, subset_samples=1 << 22,
                    group=None, rank=0, world=1):
    """The 4096-star configuration: every star against one shared 2^24-sample
    prior cache, ln L + acceptance (mixed, refined to FP64 decisions), timed
    over ``steps`` passes after ``warmup``; the mixed and the plain FP64 paths
    timed on a subset of stars x samples beside it, with their accepted counts
    compared."""
    import torch
    from thejoker_gb300 import _native as nat
    from thejoker_gb300 import autotune
    from thejoker_gb300 import device as dev
    from thejoker_gb300.batch import BatchRejection
    from thejoker_gb300.synthetic import fill_prior_cache, survey_stars
    stars = survey_stars(n_stars * world, seed=3)[rank * n_stars:(rank + 1) * n_stars]
    host = torch.empty((S, 5), dtype=torch.float64).pin_memory()
    fill_prior_cache(host.numpy(), SEED_CACHE)
    cache = dev.PriorCache(S).load(host.cuda())
    table = dev.StarTable(stars)
    sub_t = dev.StarTable(stars[:256])
    sub_t.n_epochs = table.n_epochs            # tune for the survey's epoch counts
    tuned, tune_ms = autotune.tune(sub_t, cache, precision=MIXED, count=min(S, 1 << 22),
                                   reps=1)
    del sub_t
    br = BatchRejection(table, cache, precision=MIXED, max_out=256,
                        seeds=np.arange(n_stars) + rank * n_stars, group=group)
    for _ in range(warmup):
        br.run()
    torch.cuda.synchronize()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", 0))) as clk:
        launches0 = nat.lib().joker_launch_count()
        t0 = time.perf_counter()
        for _ in range(steps):
            br.run()
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) * 1e3 / steps
        launches = nat.lib().joker_launch_count() - launches0
    counts, _, _ = br.results()
    n_refined = br.n_refined_last
    group_used = br.group
    del br
    torch.cuda.empty_cache()
    # mixed vs FP64 on the same subset
    sub = subset_stars
    Ssub = min(S, subset_samples)
    table_sub = dev.StarTable(stars[:sub])
    res = {}
    for key, prec in (("mixed", MIXED), ("fp64", "fp64")):
        b = BatchRejection(table_sub, cache, precision=prec, max_out=256, seeds=np.arange(sub))
        b.run(count=Ssub)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b.run(count=Ssub)
        torch.cuda.synchronize()
        res[key] = (time.perf_counter() - t0, b.results())
        del b
    c_m, i_m, _ = res["mixed"][1]
    c_64, i_64, _ = res["fp64"][1]
    same_counts = bool(np.array_equal(c_m, c_64))
    same_idx = same_counts and all(np.array_equal(a, b) for a, b in zip(i_m, i_64))
    n_ep = np.array([len(s["t"]) for s in stars])
    return {
        "value": n_stars * world * S / (ms * 1e-3), "unit": "samples/s",
        "ms_per_step": ms, "steps": steps, "warmup": warmup,
        "workload": f"{n_stars} stars x 2^{int(math.log2(S))} shared prior samples, epochs "
                    f"log-uniform [3,256] (mean {n_ep.mean():.1f}), 30% companions; acceptance "
                    "refined to FP64 decisions",
        "stars_per_gpu": n_stars, "prior_samples": S, "group": group_used,
        "autotune": {"chunk": tuned, "ms_256_stars_2^22_samples": tune_ms},
        "fp64_refined_per_step": n_refined,
        "subset": {"stars": sub, "samples": Ssub,
                   "mixed_samples_per_s": sub * Ssub / res["mixed"][0],
                   "fp64_samples_per_s": sub * Ssub / res["fp64"][0],
                   "speedup_mixed_vs_fp64": res["fp64"][0] / res["mixed"][0],
                   "accept_counts_identical": same_counts,
                   "accepted_indices_identical": same_idx},
        "accepted_total": int(counts.sum()),
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }


def run_batched(args, rank, world):
    """The 4096-star configuration as its own bench line (batched_measure)."""
    import torch
    from thejoker_gb300 import build as tb
    tb.build()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    m = batched_measure(args.stars, args.samples, warmup=args.warmup, steps=args.steps,
                        subset_stars=args.subset_stars,
                        subset_samples=min(args.samples, args.fp64_samples), group=args.group,
                        rank=rank, world=world)
    return {
        "metric": "prior samples/s (lnL+accept)",
        "value": m["value"], "unit": "samples/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": m["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64 (mixed)", "data": "synthetic (seeded survey, numpy prior cache)",
        "config": {"workload": m["workload"], "stars_per_gpu": m["stars_per_gpu"],
                   "prior_samples": m["prior_samples"], "group": m["group"],
                   "autotune": m["autotune"]},
        "subset": m["subset"], "accepted_total": m["accepted_total"],
        "fp64_refined_per_step": m["fp64_refined_per_step"],
        "gpu_launches": m["gpu_launches"], "clocks": m["clocks"],
    }


def iterative_measure(n_stars, S, n_req, steps=1, warmup=1, subset_stars=64, rank=0, world=1,
                      eager=True):
    """Iterative rejection of ``n_stars`` stars with a quadratic trend
    (poly_trend=3: K, v0, v1, v2 with N(0, [100 km/s, 1 km/s/d, 0.01 km/s/d^2])
    priors), 8-64 epochs each, ``n_req`` samples requested, over an S-sample
    prior library; every round on the device, rounds after the first replayed
    from a CUDA graph.  The plain FP64 path runs the same schedule on a star
    subset."""
    import torch
    from thejoker_gb300 import device as dev
    from thejoker_gb300.iterative import IterativeBatch
    from thejoker_gb300.synthetic import fill_prior_cache, survey_stars
    stars = survey_stars(n_stars * world, seed=4, n_min=8, n_max=64,
                         poly_trend=3)[rank * n_stars:(rank + 1) * n_stars]
    host = np.empty((S, 5))
    fill_prior_cache(host, SEED_CACHE + 1)
    cache = dev.PriorCache.from_samples(host)
    table = dev.StarTable(stars)
    seeds = lambda k: np.arange(n_stars) + 7919 * k + rank * n_stars
    it = IterativeBatch(table, cache, n_req, precision=MIXED, seeds=seeds(0))
    it.run()
    for w in range(warmup):
        it.reset(seeds(w + 1)).run()
    torch.cuda.synchronize()
    evals, rounds = [], []
    with ClockSampler(int(os.environ.get("LOCAL_RANK", 0))) as clk:
        t0 = time.perf_counter()
        for k in range(steps):
            it.reset(seeds(100 + k)).run()
            st, _, _ = it.results()
            evals.append(int(st[:, 2].sum()))
            rounds.append(int(st[:, 5].max()))
        ms = (time.perf_counter() - t0) * 1e3 / steps
    it.close()
    # the FP64 path on a subset, same schedule
    sub = min(subset_stars, n_stars)
    table_sub = dev.StarTable(stars[:sub])
    res = {}
    for key, prec in (("mixed", MIXED), ("fp64", "fp64")):
        b = IterativeBatch(table_sub, cache, n_req, precision=prec, seeds=np.arange(sub))
        b.run()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b.reset(np.arange(sub)).run()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        stt, idx, _ = b.results()
        res[key] = (dt, stt, idx)
        b.close()
    same = bool(np.array_equal(res["mixed"][1], res["fp64"][1]) and
                all(np.array_equal(a, b) for a, b in zip(res["mixed"][2], res["fp64"][2])))
    eager_ms = None
    if eager:
        e = IterativeBatch(table, cache, n_req, precision=MIXED, seeds=seeds(100))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e.run(use_graph=False)
        eager_ms = (time.perf_counter() - t0) * 1e3
        e.close()
    n_ep = np.array([len(s["t"]) for s in stars])
    ev = float(np.mean(evals))
    return {
        "value": ev * world / (ms * 1e-3), "unit": "samples/s", "ms_per_step": ms,
        "steps": steps, "warmup": warmup,
        "workload": f"{n_stars} stars, poly_trend=3, epochs log-uniform [8,64] "
                    f"(mean {n_ep.mean():.1f}), n_requested={n_req}, prior library "
                    f"2^{int(math.log2(S))}, rounds replayed from a CUDA graph",
        "stars_per_gpu": n_stars, "library": S, "n_requested": n_req,
        "stars_per_s": n_stars * world / (ms * 1e-3),
        "samples_evaluated_per_step": ev, "rounds_per_step": float(np.mean(rounds)),
        "eager_rounds_ms": eager_ms,
        "subset": {"stars": sub, "mixed_s": res["mixed"][0], "fp64_s": res["fp64"][0],
                   "speedup_mixed_vs_fp64": res["fp64"][0] / res["mixed"][0],
                   "results_identical": same},
        "clocks": clk.summary(),
    }


def run_iterative(args, rank, world):
    """The iterative configuration as its own bench line (iterative_measure)."""
    import torch
    from thejoker_gb300 import build as tb
    tb.build()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    r = iterative_measure(args.stars, args.samples, args.n_requested, steps=args.steps,
                          warmup=args.warmup, subset_stars=args.subset_stars, rank=rank,
                          world=world)
    return {
        "metric": "prior samples/s (lnL+accept), iterative",
        "value": r["value"], "unit": "samples/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": r["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64 (mixed)", "data": "synthetic (seeded survey, numpy prior library)",
        "config": {"workload": r["workload"], "stars_per_gpu": r["stars_per_gpu"],
                   "library": r["library"], "n_requested": r["n_requested"]},
        "stars_per_s": r["stars_per_s"],
        "samples_evaluated_per_step": r["samples_evaluated_per_step"],
        "rounds_per_step": r["rounds_per_step"], "eager_rounds_ms": r["eager_rounds_ms"],
        "subset": r["subset"], "clocks": r["clocks"],
    }


def _serving_requests(n, seed, budget_log2=(20, 27), n_req_choices=(1, 128, 512)):
    from thejoker_gb300.synthetic import survey_stars
    rng = np.random.default_rng(seed)
    stars = survey_stars(n, seed=seed + 1, n_min=3, n_max=200, poly_trend=1)
    budgets = (2.0 ** rng.uniform(*budget_log2, n)).astype(np.int64)
    n_reqs = rng.choice(np.asarray(n_req_choices), n)
    return stars, budgets, n_reqs


def _serve_stream(eng, reqs, arrivals):
    """Feed requests at their arrival times (seconds from now) and step the
    engine until all are done; latency counts from the scheduled arrival."""
    t_start = time.perf_counter()
    arr = t_start + np.asarray(arrivals)
    i, n = 0, len(reqs)
    n_done0 = len(eng.done)
    while i < n or eng.active or eng.queue:
        now = time.perf_counter()
        while i < n and arr[i] <= now:
            eng.submit(reqs[i], t=arr[i])
            i += 1
        if not eng.active and not eng.queue:
            if i < n:
                while time.perf_counter() < arr[i]:
                    pass
            continue
        eng.step()
    span = time.perf_counter() - t_start
    done = eng.done[n_done0:]
    lat = np.array([r.t_done - r.t_arrival for r in done])
    evals = sum(r.result[2] for r in done)
    return lat, span, evals


def _lindley(arrivals, service):
    """Latencies of a FIFO single server (one star at a time)."""
    t_free, out = 0.0, np.empty(len(arrivals))
    for k, (a, s) in enumerate(zip(arrivals, service)):
        start = max(a, t_free)
        t_free = start + s
        out[k] = t_free - a
    return out


def serving_measure(S, rates, window=4.0, n_all=20000, slots=1024, round_budget=1 << 26,
                    fp64_requests=128, rank=0):
    """Serving: a Poisson stream of star requests (epochs log-uniform [3,200],
    prior budget log-uniform 2^20-2^27 samples of a device-resident 2^28
    cache, n_requested in {1, 128, 512}), admitted by free device memory into
    the continuously batched iterative rounds; p50/p99 latency and throughput
    per arrival rate, and the plain FP64 per-star path (one star at a time)
    measured on a prefix of the stream, its latency at each rate from its
    measured service times (FIFO queue)."""
    import torch
    from thejoker_gb300 import device as dev
    from thejoker_gb300.serve import Request, ServingEngine
    # the resident cache is drawn on the device (P log-uniform [2, 1024] d,
    # e ~ Beta(0.867, 3.03), uniform angles, s = 0)
    cache = dev.PriorCache(S)
    t0 = time.perf_counter()
    cache.sample_prior(dict(P_min=2.0, P_max=1024.0, e_alpha=0.867, e_beta=3.03, s_kind=0,
                            s_value=0.0), S, seed=SEED_CACHE + 2)
    torch.cuda.synchronize()
    cache_s = time.perf_counter() - t0
    stars, budgets, n_reqs = _serving_requests(n_all, 11 + rank)

    def make(k):
        return Request(stars[k], budget=int(budgets[k]), n_requested=int(n_reqs[k]),
                       seed=100000 + k)

    eng = ServingEngine(cache, n_slots=slots, max_epochs=200, n_linear=2,
                        max_requested=512, precision=MIXED, round_budget=round_budget,
                        pool_fraction=0.6)
    # warm-up: the first rounds load the kernels and capture the round graph
    for k in range(min(n_all, 64)):
        eng.submit(make(k))
    eng.drain()
    rng = np.random.default_rng(77)
    sweep = []
    with ClockSampler(int(os.environ.get("LOCAL_RANK", 0))) as clk:
        for rate in rates:
            n = int(min(n_all, max(200, rate * window)))
            arrivals = np.cumsum(rng.exponential(1.0 / rate, n))
            reqs = [make(k) for k in range(n)]
            lat, span, evals = _serve_stream(eng, reqs, arrivals)
            sweep.append({"rate_per_s": rate, "requests": n,
                          "p50_ms": float(np.percentile(lat, 50) * 1e3),
                          "p99_ms": float(np.percentile(lat, 99) * 1e3),
                          "throughput_req_per_s": n / span,
                          "samples_per_s": evals / span, "span_s": span})
    rounds = eng.rounds
    eng.close()
    # plain FP64 per-star path: one star at a time, same requests
    n64 = min(fp64_requests, n_all)
    one = ServingEngine(cache, n_slots=1, max_epochs=200, n_linear=2, max_requested=512,
                        precision="fp64", pool_samples=1 << 27)
    one.submit(make(0))
    one.drain()
    service = []
    for k in range(n64):
        r = make(k)
        t0 = time.perf_counter()
        one.submit(r, t=t0)
        one.drain()
        service.append(time.perf_counter() - t0)
    one.close()
    service = np.array(service)
    fp64 = {"requests_timed": n64, "mean_service_ms": float(service.mean() * 1e3),
            "capacity_req_per_s": float(1.0 / service.mean()), "per_rate": []}
    for rate in rates:
        n = int(min(n_all, max(200, rate * window)))
        arrivals = np.cumsum(np.random.default_rng(5).exponential(1.0 / rate, n))
        lat = _lindley(arrivals, np.resize(service, n))
        fp64["per_rate"].append({"rate_per_s": rate, "p50_ms": float(np.percentile(lat, 50) * 1e3),
                                 "p99_ms": float(np.percentile(lat, 99) * 1e3)})
    del cache
    torch.cuda.empty_cache()
    return {"workload": "Poisson stream of star requests, epochs log-uniform [3,200], "
                        "budget log-uniform 2^20-2^27 of a resident "
                        f"2^{int(math.log2(S))} cache, n_requested in {{1,128,512}}",
            "slots": slots, "round_budget": round_budget, "window_s": window,
            "sweep": sweep, "rounds": rounds, "cache_sample_s": cache_s,
            "fp64_per_star": fp64, "clocks": clk.summary()}


def run_serving(args, rank, world):
    """The serving stream as its own bench line (serving_measure), swept over
    arrival rates."""
    import torch
    from thejoker_gb300 import build as tb
    tb.build()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    rates = [float(r) for r in args.rates.split(",")]
    m = serving_measure(args.samples, rates, window=args.window, n_all=args.requests,
                        slots=args.slots, round_budget=args.round_budget,
                        fp64_requests=args.fp64_requests, rank=rank)
    top = m["sweep"][-1]
    return {
        "metric": "p50/p99 per-star latency and request throughput, serving",
        "value": top["throughput_req_per_s"], "unit": "requests/s",
        "n_gpus": world, "steps": len(rates), "warmup": 1,
        "ms_per_step": top["span_s"] * 1e3 / max(top["requests"], 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64 (mixed)", "data": "synthetic (seeded survey stream, numpy prior cache)",
        "config": {"workload": m["workload"], "slots": args.slots,
                   "round_budget": args.round_budget, "requests_max": args.requests,
                   "window_s": args.window},
        "sweep": m["sweep"], "rounds": m["rounds"], "cache_sample_s": m["cache_sample_s"],
        "fp64_per_star": m["fp64_per_star"], "clocks": m["clocks"],
    }


def run_small(args, rank, world):
    """The reference's own small case: one star, 16 epochs at 2456000 +
    U(0, 1000) d, sigma ~ U(0.1, 1) km/s, a Keplerian drawn from the prior plus
    noise; a 2^20-sample prior cache (s = 0); the plain FP64 GPU path, the
    mixed path and the reference's CPU likelihood over all 2^20 samples; ln L
    differences and accept-mask agreement."""
    import torch
    from thejoker_gb300 import build as tb
    from thejoker_gb300 import device as dev
    from thejoker_gb300.batch import BatchRejection
    from thejoker_gb300.linear import rv_unit_columns
    from thejoker_gb300.synthetic import fill_prior_cache
    tb.build()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    rng = np.random.default_rng(0)
    N, S = 16, args.samples
    t = np.sort(2456000.0 + rng.uniform(0, 1000.0, N))
    err = rng.uniform(0.1, 1.0, N)
    P = np.exp(rng.uniform(np.log(2), np.log(1024)))
    e = rng.beta(0.867, 3.03)
    om, M0 = rng.uniform(0, 2 * np.pi, 2)
    K = 30.0 * (P / 365.25) ** (-1 / 3) / np.sqrt(1 - e ** 2) * rng.normal()
    rv = K * rv_unit_columns(t, t.min(), [P], [e], [om], [M0])[0] + rng.normal(0, 100.0) \
        + rng.normal(0, err)
    star = dict(t=t, rv=rv, ivar=1 / err ** 2, t_ref=t.min(), trend_M=np.ones((N, 1)),
                mu=np.zeros(2), lam=np.array([0.0, 100.0 ** 2]),
                k_prior=np.array([1.0, 30.0, 365.25, 500.0]))
    chunk = fill_prior_cache(np.empty((S, 5)), 0)
    cache = dev.PriorCache.from_samples(chunk)
    table = dev.StarTable([star])
    from thejoker_gb300 import _native as nat
    res = {}
    for key, prec in (("fp64", "fp64"), ("mixed", MIXED)):
        br = BatchRejection(table, cache, precision=prec, max_out=S, seeds=[1])
        for _ in range(args.warmup):
            br.run()
        torch.cuda.synchronize()
        launches0 = nat.lib().joker_launch_count()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            br.run()
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) * 1e3 / args.steps
        launches = nat.lib().joker_launch_count() - launches0
        counts, idx, ll = br.results()
        res[key] = (ms, idx[0], br.lnl[0, :S].cpu().numpy(), ll[0])
    d = np.abs(res["mixed"][2] - res["fp64"][2])
    kept_d = np.abs(res["mixed"][3] - res["fp64"][2][res["mixed"][1]]) \
        if np.array_equal(res["fp64"][1], res["mixed"][1]) else np.array([np.inf])
    near = res["fp64"][2] > res["fp64"][2].max() - 40
    line = {
        "metric": "prior samples/s (lnL+accept)", "value": S / (res["mixed"][0] * 1e-3),
        "unit": "samples/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": res["mixed"][0], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64 (mixed)",
        "data": "synthetic (seeded star and prior cache)",
        "config": {"workload": f"1 star x {N} epochs over 1000 d, prior cache 2^"
                               f"{int(math.log2(S))} (s = 0)"},
        "fp64": {"value": S / (res["fp64"][0] * 1e-3), "ms_per_step": res["fp64"][0]},
        "gpu_launches": int(launches),
        "max_abs_dlnl": float(d.max()), "max_abs_dlnl_within_40_of_max": float(d[near].max()),
        "max_abs_dlnl_kept": float(kept_d.max()),
        "accepted": int(len(res["fp64"][1])),
        "accept_identical": bool(np.array_equal(res["fp64"][1], res["mixed"][1])),
    }
    if not args.no_cpu:
        v, kind, cores, secs = cpu_baseline(star, S, seed=0)
        line["cpu_baseline"] = {"value": v, "unit": "samples/s", "cores": cores, "kind": kind,
                                "sample": f"all {S} prior samples ({secs:.2f} s wall)"}
    return line


def _gpu_ms(fn, reps=3, warmup=1):
    """Mean CUDA-event time of fn() on the current stream, after warm-up."""
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def run_posterior(args, rank, world):
    """The paths either side of the likelihood, each timed on the GPU beside a
    CPU statement of the same work on the host cores:
    - prior draws on the device (joker_prior_sample; JokerPrior.sample,
      prior.py:297-407), against numpy draws of the same distributions;
    - the linear-parameter posterior of accepted samples with one draw each
      (joker_linear_posterior plus host draws in the reference's rng order;
      batch_get_posterior_samples, fast_likelihood.pyx:471-545), against the
      reference's own Cython batch_get_posterior_samples;
    - the unmarginalized ln L (joker_unmarginalized_lnl;
      samples.py:611-632), against NumPy over the oracle's RV model;
    - the RV model on its own (joker_rv_from_elements; c_rv_from_elements),
      against the oracle's C statement."""
    import torch
    from thejoker_gb300 import _native as nat
    from thejoker_gb300 import build as tb
    from thejoker_gb300 import device as dev
    from thejoker_gb300.linear import multivariate_normal_draws
    from oracle import build as ob, oracle, ref_cython
    tb.build()
    ob.build_all()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    star = make_star()
    cores = os.cpu_count() or 1
    out = {}
    # ---- prior draws
    n_pr = min(args.samples, 1 << 28)
    cache = dev.PriorCache(n_pr)
    spec = dict(P_min=2.0, P_max=1024.0, e_alpha=0.867, e_beta=3.03,
                s_kind=nat.JOKER_S_LOGNORMAL, s_mu=float(np.log(0.5)), s_sigma=1.0)
    ms = _gpu_ms(lambda: cache.sample_prior(spec, n_pr, seed=11))
    n_cpu = 1 << 22
    t0 = time.perf_counter()
    fill_cache_host(np.empty((n_cpu, 5)), 5, threads=cores)
    dt = time.perf_counter() - t0
    out["prior_draws"] = {
        "gpu": n_pr / (ms * 1e-3), "cpu": n_cpu / dt, "unit": "samples/s",
        "gpu_samples": n_pr, "cpu_samples": n_cpu, "cpu_cores": cores, "cpu_kind": "port",
        "hbm_gbs": 76 * n_pr / (ms * 1e-3) / 1e9,
        "note": "76 B written per sample (FP64 columns + prepared mixed form); numpy draws "
                "of the same distributions on the CPU (the reference samples through pymc)"}
    del cache
    torch.cuda.empty_cache()
    # ---- linear posterior of accepted rows, one draw each
    n_po = 1 << 20
    chunk = fill_cache_host(np.empty((n_po, 5)), 6)
    table = dev.StarTable([star], jitter="reference")
    pc = dev.PriorCache.from_samples(chunk)
    rows = torch.arange(n_po, dtype=torch.int64, device="cuda")
    ms_dev = _gpu_ms(lambda: dev.linear_posterior(table, pc, 0, rows))
    t0 = time.perf_counter()
    a, A, ll = dev.linear_posterior(table, pc, 0, rows)
    draws = multivariate_normal_draws(np.random.default_rng(3), a.cpu().numpy(),
                                      A.cpu().numpy(), 1)
    dt_e2e = time.perf_counter() - t0
    n_ref = 1 << 14
    h = ref_cython.make_helper(star["t"], star["rv"], star["ivar"], star["t_ref"],
                               star["trend_M"], 1, 0, star["mu"], np.sqrt(star["lam"]), True,
                               *star["k_prior"][1:]) if ref_cython.available() else None
    if h is not None:
        t0 = time.perf_counter()
        h.batch_get_posterior_samples(np.ascontiguousarray(chunk[:n_ref]), 1,
                                      np.random.default_rng(3))
        dt_ref = time.perf_counter() - t0
        cpu = {"cpu": n_ref / dt_ref, "cpu_rows": n_ref, "cpu_cores": 1, "cpu_kind": "reference"}
    else:
        cpu = {"cpu": None, "cpu_kind": "unavailable"}
    out["linear_posterior"] = dict(
        {"gpu_device": n_po / (ms_dev * 1e-3), "gpu_with_host_draws": n_po / dt_e2e,
         "unit": "rows/s", "gpu_rows": n_po, "draws_shape": list(draws.shape)}, **cpu)
    del pc, a, A, ll
    torch.cuda.empty_cache()
    # ---- unmarginalized ln L
    n_un = 1 << 20
    rng = np.random.default_rng(7)
    pars = np.column_stack([chunk[:n_un], rng.normal(0, 30, n_un), rng.normal(0, 100, n_un)])
    table_j = dev.StarTable([star], jitter="applied")
    d_pars = torch.from_numpy(np.ascontiguousarray(pars)).cuda()
    ms_un = _gpu_ms(lambda: dev.unmarginalized_lnl(table_j, 0, d_pars, 1))
    n_c = 1 << 14
    t0 = time.perf_counter()
    m = oracle.rv_unit(star["t"], star["t_ref"], pars[:n_c, :5])
    model = pars[:n_c, 5:6] * m + pars[:n_c, 6:7]
    var = 1.0 / star["ivar"][None, :] + pars[:n_c, 4:5] ** 2
    _ = -0.5 * np.sum(np.log(2 * np.pi * var) + (star["rv"][None, :] - model) ** 2 / var, axis=1)
    dt_un = time.perf_counter() - t0
    out["unmarginalized_lnl"] = {"gpu": n_un / (ms_un * 1e-3), "cpu": n_c / dt_un,
                                 "unit": "rows/s", "gpu_rows": n_un, "cpu_rows": n_c,
                                 "cpu_cores": 1, "cpu_kind": "port"}
    # ---- RV model alone
    el = np.column_stack([chunk[:, 0], rng.normal(0, 30, n_po), chunk[:, 1], chunk[:, 2],
                          chunk[:, 3]])
    d_el = torch.from_numpy(np.ascontiguousarray(el)).cuda()
    d_t = torch.from_numpy(star["t"]).cuda()
    ms_rv = _gpu_ms(lambda: dev.rv_from_elements(d_t, d_el, star["t_ref"]))
    t0 = time.perf_counter()
    oracle.rv_unit(star["t"], star["t_ref"], chunk[:n_c])
    dt_rv = time.perf_counter() - t0
    ne = len(star["t"])
    out["rv_from_elements"] = {"gpu": n_po * ne / (ms_rv * 1e-3), "cpu": n_c * ne / dt_rv,
                               "unit": "orbit-epochs/s", "gpu_orbits": n_po, "epochs": ne,
                               "cpu_cores": 1, "cpu_kind": "port"}
    return {
        "metric": "rows/s of the paths around the likelihood (linear posterior with draws)",
        "value": out["linear_posterior"]["gpu_with_host_draws"], "unit": "rows/s",
        "n_gpus": world, "steps": 3, "warmup": 1, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded star and prior samples)",
        "config": {"workload": f"1 star x {N_EPOCHS} epochs over {SPAN_D:.0f} d; prior draws "
                               f"2^{int(math.log2(n_pr))}, posterior / unmarginalized / RV "
                               f"rows 2^20"},
        **out,
    }


def run_reference(args, rank):
    if rank != 0:
        return None
    star = make_star()
    vals = []
    for _ in range(args.warmup):
        cpu_baseline(star, args.cpu_samples // 4)
    for k in range(args.steps):
        v, kind, cores, secs = cpu_baseline(star, args.cpu_samples, seed=10 + k)
        vals.append((v, secs))
    v = float(np.mean([x[0] for x in vals]))
    ms = float(np.mean([x[1] for x in vals])) * 1e3
    return {
        "metric": "prior samples/s (lnL+accept)", "value": v, "unit": "samples/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)", "impl": "reference",
        "config": {"workload": f"1 star x {N_EPOCHS} epochs over {SPAN_D:.0f} d, jitter in "
                               "the samples (ignored by the reference)",
                   "prior_samples_per_step": args.cpu_samples},
        "cpu_baseline": {"value": v, "unit": "samples/s", "cores": cores, "kind": kind,
                         "sample": f"{args.cpu_samples} prior samples per step"},
        "e2e": {"value": v, "unit": "samples/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--samples", type=int, default=None)
    p.add_argument("--fp64-samples", type=int, default=1 << 25)
    p.add_argument("--cpu-samples", type=int, default=1 << 20)
    p.add_argument("--h2d-chunk", type=int, default=1 << 24)
    p.add_argument("--fp32-peak", type=float, default=74.9)
    p.add_argument("--traffic", type=float, default=None)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--headline-only", action="store_true",
                   help="default mode: skip the batched and serving sub-objects")
    p.add_argument("--precision", default="mixed_fast", choices=["mixed_fast", "mixed"],
                   help="the mixed path: FP32 epoch sums (mixed_fast) or float-float sums")
    p.add_argument("--config", default="single",
                   choices=["single", "small", "batched", "iterative", "serving",
                            "posterior"])
    p.add_argument("--stars", type=int, default=None)
    p.add_argument("--n-requested", type=int, default=256)
    p.add_argument("--requests", type=int, default=20000)
    p.add_argument("--rates", default="100,500,1000,2000,5000")
    p.add_argument("--window", type=float, default=4.0)
    p.add_argument("--slots", type=int, default=1024)
    p.add_argument("--round-budget", type=int, default=1 << 26)
    p.add_argument("--fp64-requests", type=int, default=128)
    p.add_argument("--group", type=int, default=None)
    p.add_argument("--subset-stars", type=int, default=64)
    args = p.parse_args()
    global MIXED
    MIXED = args.precision
    if args.samples is None:
        args.samples = {"single": 1 << 28, "small": 1 << 20, "batched": 1 << 24,
                        "iterative": 1 << 22, "serving": 1 << 28,
                        "posterior": 1 << 27}[args.config]
    if args.stars is None:
        args.stars = {"batched": 4096, "iterative": 1024}.get(args.config, 1)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if args.impl == "reference":
        line = run_reference(args, rank)
    else:
        if world > 1:
            import torch
            import torch.distributed as tdist
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
            tdist.init_process_group("nccl")
            dist = tdist
        if args.config == "batched":
            line = run_batched(args, rank, world)
        elif args.config == "small":
            line = run_small(args, rank, world)
        elif args.config == "iterative":
            line = run_iterative(args, rank, world)
        elif args.config == "serving":
            line = run_serving(args, rank, world)
        elif args.config == "posterior":
            line = run_posterior(args, rank, world)
        else:
            line = run_ours(args, rank, world, dist)
        if dist is not None:
            dist.destroy_process_group()
    if line is not None:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
