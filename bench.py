"""K-SVD benchmark (one JSON line on stdout).

Workload: the headline configuration n=256, K=1024, N=1,000,000, T=16 (seeded synthetic data of
that shape and distribution: the reference's fMRI inputs are not published).  One "step" is one
full K-SVD iteration (D'X, Batch-OMP, per-atom lists, the atom sweep, error/RMSE, Gram,
clearDict) through ``ksvd_iterate`` with every input resident in HBM.  X is 1 GB, far larger
than the 129 MB L2, so no L2 flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--precision fp32|mixed] [--config cfg2]

--impl reference times the reference algorithm's CPU restatement (the oracle: the reference
itself has no CPU path and cannot be built here) on the host cores, on a bounded sample of the
same workload, scaled to the full workload.
"""
from __future__ import annotations

import argparse
import gc
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# kernels launched by one ksvd_iterate call: before the first iteration (pad copy, normcols,
# Gram; mixed adds the D split for the Gram and the X split) and per iteration (D'X, OMP, six
# list/precompute kernels, sweep, error, RMSE, Gram, coherence, clearDict; mixed adds two
# dictionary splits)
# library kernels per ksvd_iterate call: copy_pad_cols, normcols, Gram (mixed: + BF16 splits of D
# and X); per iteration: D'X, OMP, Gram, 4 list kernels, init_state, prepare, P = D'Y, sweep,
# error + rmse, Gram, coherence + clear_seq, advance_counter (mixed: + 3 BF16 splits of D and
# the FP16 copy of G and its column coherences for Batch-OMP); the windowed preparation (X above
# 96 MiB, T <= 16, n % 4 == 0, n <= 256) adds the reduction of the windows' partials
KERNELS_PER_CALL = {"fp32": 3, "mixed": 5}
KERNELS_PER_ITER = {"fp32": 17, "mixed": 22}


def windowed_prep(n, T, N):
    """Whether the list preparation runs in windows of X (the library's rule)."""
    return T <= 16 and n % 4 == 0 and n <= 256 and N * n * 4 > (96 << 20)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            m = json.load(f)
        return dict(hbm=m["hbm_gbs"], bf16=m["bf16_tflops"], bf16_sus=m["bf16_tflops_sustained"],
                    src="measured")
    return dict(hbm=6800.0, bf16=1900.0, bf16_sus=1700.0, src="fallback")


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        # nvidia-smi takes a moment to start: wait for its first row, so the samples cover the
        # timed region that follows
        t0 = time.time()
        while time.time() - t0 < 5.0 and self.proc.poll() is None:
            try:
                if os.path.getsize(self.f.name) > 0:
                    break
            except OSError:
                break
            time.sleep(0.05)

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = max(mx, float(r[2]))
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def stage_bytes(cfg, N, stage):
    """Algorithmic HBM bytes of one launch of each stage (FP32 data, 4-byte indices)."""
    n, K, T = cfg.n, cfg.K, cfg.T
    Kp = 128 if K <= 128 else 256 if K <= 256 else 512 if K <= 512 else 1024
    if stage == "omp":      # stream alpha0 (Kp rows), write T (index, coefficient) + nnz
        return N * (Kp * 4 + T * 8 + 4)
    if stage == "sweep":    # gather x_s for every (signal, atom) entry, read the signal's code
        #                     twice (a'D product and C refresh), write the new coefficient
        return N * T * (n * 4) + 2 * N * T * T * 8 + N * T * 4
    if stage == "lists":    # idx/nnz twice (count, fill), list write, X gathered per entry
        if windowed_prep(n, T, N):
            # windowed preparation: each ~32 MB window of X (and its codes) is read from HBM
            # once and gathered from L2; the windows' partials are written and read once
            w = max(1, (32 << 20) // (4 * n) // 256) * 256
            nwin = -(-N // w)
            return (2 * N * T * 4 + N * T * 4 + N * T * 4 + N * n * 4 + N * T * 8
                    + 2 * nwin * Kp * (n + Kp + 1) * 4)
        return 2 * N * T * 4 + N * T * 4 + N * T * (n * 4 + T * 8)
    if stage == "error":    # X once, the code once, the error vector
        return N * n * 4 + N * T * 8 + N * 4
    if stage == "dtx":      # X once, alpha0 written
        return N * n * 4 + N * Kp * 4
    return 0


def stage_flops(cfg, N, stage):
    n, K, T = cfg.n, cfg.K, cfg.T
    if stage == "dtx":
        return 2.0 * n * K * N
    if stage == "gram":
        return 2.0 * n * K * K
    if stage == "omp":      # alpha updates: sum over steps t of 2*K*t  (= K*T(T+1) per signal)
        return float(N) * K * T * (T + 1)
    return 0.0


# DRAM bytes per signal of one launch from an ncu capture (dram__bytes_read.sum +
# dram__bytes_write.sum) of the same kernel on 100,000 signals of the same (n, K, T) -- traffic
# grows in proportion to the signals, so the bench scales it to its N -- with the capture's L2
# throughput and issue activity (lts__throughput, smsp__issue_active, percent of peak).  Each
# entry is keyed by the fingerprint of the kernel source it was measured on (KERNEL_SOURCES): when
# the source changes, no entry matches and the line reports traffic as null instead of a stale
# figure.
KERNEL_SOURCES = {"omp": ("omp.cu",)}
# (n, K, T, precision, fingerprint) -> (bytes per signal, L2 %, issue %): omp_kernel<32, 32, H16, 1>
# at 100,000 signals, dram__bytes_read.sum + dram__bytes_write.sum per signal
MEASURED_OMP = {
    (256, 1024, 16, "mixed", "278aec7dbdb97848"): ((416187904 + 7526656) / 100_000, 46.98, 71.26),
    (256, 1024, 16, "fp32", "278aec7dbdb97848"): ((413833216 + 7440128) / 100_000, 77.82, 53.98),
}
# omp_batched_kernel<64> on the cfg3 mix scaled to 293,494 signals (same source fingerprint):
# DRAM bytes per signal -- far above the algorithmic bytes, the support columns of 64 Gram
# matrices miss L2 (86 % hit rate)
MEASURED_BATCHED = {"278aec7dbdb97848": (42805705216 + 95426816) / 293494}


def source_fingerprint(stage):
    """sha256 (16 hex digits) of the kernel sources of a stage."""
    import hashlib

    h = hashlib.sha256()
    for f in KERNEL_SOURCES.get(stage, ()):
        with open(os.path.join(ROOT, "ksvd_gb300", "csrc", f), "rb") as fh:
            h.update(f.encode() + b"\0" + fh.read())
    return h.hexdigest()[:16]


# FP32 CUDA-core peak (nominal): 152 SMs x 128 FMA lanes x 2 FLOP x 2.07 GHz.
FP32_SIMT_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12


def cpu_time_at(N, Ns, ts, Nl, tl):
    """Seconds of one CPU iteration at N signals from timings at two sample sizes: the affine
    model t = a + b n through (Ns, ts) and (Nl, tl) -- a holds the per-iteration work that does
    not grow with the signals (the K-dependent parts of the sweep and clearDict); linear in N
    from the larger sample when only one size was timed or the fit is not increasing."""
    if tl is None or Nl <= Ns:
        return ts * N / Ns
    b = (tl - ts) / (Nl - Ns)
    a = ts - b * Ns
    if b <= 0 or a < 0:
        return tl * N / Nl
    return a + b * N


def max_over_ranks(x, dist, device):
    """The slowest rank's time (every rank gets it); identity without a process group."""
    if dist is None:
        return float(x)
    import torch

    t = torch.tensor([float(x)], device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank, steps, ms, world):
    """Whole-job throughput: every rank processes `units_per_rank` per step (weak scaling),
    timed by the slowest rank."""
    return world * units_per_rank * steps / (ms / 1e3)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def run_reference(args, cfg):
    """The reference algorithm on the host cores (the oracle port), bounded sample."""
    import numpy as np

    import oracle
    from ksvd_gb300 import datagen

    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    if args.config == "cfg3":
        probs = datagen.make_batched(device="cpu", scale=0.02)
        cpu = cpu_baseline_batched(probs, max(200, args.cpu_sample // 64))
        line = {"impl": "reference", "metric": "ksvd_batched_iters_per_s", "value": cpu["value"],
                "unit": "iter/s", "n_gpus": ws, "steps": 1, "warmup": 0,
                "ms_per_step": 1e3 / cpu["value"], "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "fp32", "data": "synthetic (seeded, cfg3 shapes)",
                "config": {"workload": "cfg3: 64 problems, one K-SVD iteration of every problem"},
                "cpu_baseline": cpu,
                "e2e": {"value": cpu["value"], "unit": "iter/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return 0
    oracle.build()
    threads = oracle.num_threads()
    Ns = min(cfg.N, args.cpu_sample)
    Nl = min(cfg.N, 4 * Ns)                 # a second, larger sample: is the cost linear in N?
    p = datagen.make_problem(cfg, N=Nl)
    XL, DL = p["X"], p["D"]
    X, D = np.asfortranarray(XL[:, :Ns]), DL.copy(order="F")
    rng = np.random.default_rng(0)
    times = []
    for step in range(args.warmup + args.steps):
        perm = rng.permutation(cfg.K).astype(np.int32)[None, :]
        t0 = time.perf_counter()
        D, idx, coef, nnz, rmse = oracle.ksvd(X, D, cfg.T, 1, perm)
        dt = time.perf_counter() - t0
        if step >= args.warmup:
            times.append(dt)
    t = statistics.median(times)
    lin = None
    tl = None
    if Nl > Ns:
        perm = rng.permutation(cfg.K).astype(np.int32)[None, :]
        t0 = time.perf_counter()
        oracle.ksvd(XL, DL.copy(order="F"), cfg.T, 1, perm)
        tl = time.perf_counter() - t0
    value = 1.0 / cpu_time_at(cfg.N, Ns, t, Nl, tl)   # iterations/s at the full N
    if tl is not None:
        lin = {"signals": [Ns, Nl], "seconds": [t, tl], "s_per_signal": [t / Ns, tl / Nl],
               "ratio_large_over_small": (tl / Nl) / (t / Ns),
               "value_linear_from_small": 1.0 / (t * cfg.N / Ns),
               "value_linear_from_large": 1.0 / (tl * cfg.N / Nl)}
    line = {
        "impl": "reference", "metric": "ksvd_iters_per_s", "value": value, "unit": "iter/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 / value, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32", "data": "synthetic (seeded, %s shape)" % cfg.name,
        "config": {"workload": "%s: n=%d K=%d N=%d T=%d, one K-SVD iteration per step"
                   % (cfg.name, cfg.n, cfg.K, cfg.N, cfg.T), "n": cfg.n, "K": cfg.K,
                   "N": cfg.N, "T": cfg.T},
        "cpu_baseline": {"value": value, "unit": "iter/s", "cores": threads, "kind": "port",
                         "sample": "%d of %d signals per step (%.2f s each, median of %d steps) "
                         "and one iteration on %d signals (%s); the full-N time from the affine "
                         "fit t = a + b N through the two sizes"
                         % (Ns, cfg.N, t, args.steps, Nl,
                            "%.2f s" % tl if tl is not None else "n/a"),
                         "linearity": lin},
        "sample_s_per_step": t,
        "e2e": {"value": value, "unit": "iter/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def cpu_baseline(cfg, sample, reps=1, check_iters=3, check_signals=20000):
    """The oracle on the host cores: one K-SVD iteration on a sample of the workload, timed and
    scaled by N.  Also returns the FP64 oracle's per-iteration RMSE over `check_iters`
    iterations of the first `check_signals` signals of that sample with fixed atom orders, for
    the GPU path to be compared with on the same signals (the check, not a timing)."""
    import numpy as np

    import oracle
    from ksvd_gb300 import datagen

    oracle.build()
    Ns = min(cfg.N, sample)
    Nl = min(cfg.N, 4 * Ns)                 # a second, larger sample: is the cost linear in N?
    p = datagen.make_problem(cfg, N=Nl)
    perm = np.random.default_rng(0).permutation(cfg.K).astype(np.int32)[None, :]
    Xs = np.asfortranarray(p["X"][:, :Ns])
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        oracle.ksvd(Xs, p["D"], cfg.T, 1, perm)
        ts.append(time.perf_counter() - t0)
    t = statistics.median(ts)
    tl = None
    if Nl > Ns:
        t0 = time.perf_counter()
        oracle.ksvd(p["X"], p["D"], cfg.T, 1, perm)
        tl = time.perf_counter() - t0
    base = {"value": 1.0 / cpu_time_at(cfg.N, Ns, t, Nl, tl), "unit": "iter/s",
            "cores": oracle.num_threads(), "kind": "port",
            "sample": "one K-SVD iteration on %d of %d signals (%.2f s)%s; the full-N time from "
                      "the affine fit t = a + b N through the two sizes" %
                      (Ns, cfg.N, t, "" if tl is None else
                       " and one on %d signals (%.2f s)" % (Nl, tl))}
    if tl is not None:
        base["linearity"] = {"signals": [Ns, Nl], "seconds": [t, tl],
                             "s_per_signal": [t / Ns, tl / Nl],
                             "ratio_large_over_small": (tl / Nl) / (t / Ns),
                             "value_linear_from_small": 1.0 / (t * cfg.N / Ns)}
    check = None
    if check_iters > 0:
        rng = np.random.default_rng(1)
        perms = np.stack([rng.permutation(cfg.K) for _ in range(check_iters)]).astype(np.int32)
        Xc = np.asfortranarray(p["X"][:, :min(Ns, check_signals)])
        r64 = oracle.ksvd(Xc.astype(np.float64), p["D"].astype(np.float64), cfg.T,
                          check_iters, perms)[4]
        check = dict(X=Xc, D=p["D"], perms=perms, rmse_fp64=[float(v) for v in r64])
    return base, check


def error_vs_fp64(cfg, check, precision, device):
    """Per-iteration RMSE of the GPU path on the oracle check's sample (same data, initial
    dictionary and atom orders) beside the FP64 oracle's."""
    import numpy as np
    import torch

    from ksvd_gb300 import Handle

    X = torch.from_numpy(np.ascontiguousarray(check["X"].T)).to(device)
    D = torch.from_numpy(np.ascontiguousarray(check["D"].T)).to(device)
    iters = check["perms"].shape[0]
    h = Handle(cfg.n, cfg.K, cfg.T, precision=precision)
    rg = [float(v) for v in h.iterate(D, X, iters, perms=check["perms"])[3]]
    h.close()
    r64 = check["rmse_fp64"]
    return {"sample_signals": int(X.shape[0]), "iterations": iters,
            "rmse_gpu": rg, "rmse_fp64_oracle": r64,
            "rel_diff_per_iter": [abs(a - b) / b for a, b in zip(rg, r64)]}


def cpu_baseline_batched(probs, per_problem):
    """The oracle on the host cores: one K-SVD iteration (error-constrained OMP, update, error,
    clearDict) on the first ``per_problem`` signals of every problem, scaled by each N."""
    import numpy as np

    import oracle

    oracle.build()
    total = 0.0
    used = 0
    for q in probs:
        m = min(q["N"], per_problem)
        X = np.asfortranarray(q["X"][:m].double().cpu().numpy().T)
        D = oracle.normcols(np.asfortranarray(q["D"].double().cpu().numpy().T))
        e2 = q["eps2"][:m].double().cpu().numpy()
        perm = np.random.default_rng(0).permutation(q["K"]).astype(np.int32)
        t0 = time.perf_counter()
        G, A0 = oracle.gram(D), oracle.dtx(D, X)
        idx, coef, nnz = oracle.omp(G, A0, q["T"], xnorm2=np.sum(X * X, 0), eps2=e2)
        D1, coef, stt = oracle.update(X, D, idx, coef, nnz, perm)
        _, err = oracle.error(X, D1, idx, coef, nnz, stt["bitmap"])
        oracle.cleardict(X, D1, idx, coef, nnz, stt["replaced"], err)
        total += (time.perf_counter() - t0) * q["N_full"] / m
        used += m
    return {"value": 1.0 / total, "unit": "iter/s", "cores": oracle.num_threads(), "kind": "port",
            "sample": "one iteration of every problem on its first %d signals (%d in all), "
                      "scaled by each problem's full N" % (per_problem, used)}


def run_batched(args):
    """The batched workload: 64 independent dictionaries (n in {32, 64, 128, 256}, K = 4n,
    N in 10k..200k, error-constrained supports of 1..64 atoms); one step = one K-SVD iteration
    of every problem (one persistent Batch-OMP launch + concurrent per-problem updates)."""
    import numpy as np
    import torch

    from ksvd_gb300 import Handle, datagen

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    scale = (args.signals / 6.7e6) if args.signals else 1.0
    probs = datagen.make_batched(seed=datagen.SEED_BASE + 3 + 1000 * rank, device=dev,
                                 scale=scale)
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu = cpu_baseline_batched(probs, max(200, args.cpu_sample // 64))
    Ntot = sum(q["N"] for q in probs)
    h = Handle(1, 1, 1, profile=True, precision=args.precision)
    tuning = h.autotune_batched(probs)
    outs, _ = h.batched_iterate(probs, args.warmup)
    torch.cuda.synchronize()
    h.stage_times(reset=True)
    sampler = ClockSampler(local)
    sampler.start()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    _, rmse = h.batched_iterate(probs, args.steps, out=outs)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1)
    st = h.stage_times()
    omp_ms = st["omp"][0] / max(st["omp"][1], 1)
    gemm_ms = st["dtx"][0] / max(st["dtx"][1], 1)
    # the persistent OMP launch: alpha0 streamed once, codes written
    kp = lambda K: 128 if K <= 128 else 256 if K <= 256 else 512 if K <= 512 else 1024
    omp_bytes = sum(q["N"] * (kp(q["K"]) * 4 + q["T"] * 8 + 4 + q["n"] * 4 + 4) for q in probs)
    pk = peaks()
    ach = omp_bytes / (omp_ms / 1e3) / 1e9
    roof = {"bound": "hbm", "achieved": ach, "peak": pk["hbm"], "unit": "GB/s",
            "frac": ach / pk["hbm"], "traffic": None, "kernel": "omp_batched_kernel",
            "peak_source": pk["src"]}
    fpb = source_fingerprint("omp")
    if fpb in MEASURED_BATCHED:
        Ntot_ = sum(q["N"] for q in probs)
        roof["traffic"] = MEASURED_BATCHED[fpb] * Ntot_
        roof["traffic_source"] = ("ncu capture of this kernel source on the cfg3 mix at 293,494 "
                                  "signals, scaled by the signals")
        roof["dram_gbs_measured_traffic"] = roof["traffic"] / (omp_ms / 1e3) / 1e9
    else:
        roof["traffic_source"] = "no ncu capture of kernel source %s: not reported" % fpb
    sizes = torch.cat([o[2] for o in outs]).float()
    e2e = None
    if not args.no_e2e:
        hx = [torch.empty_like(q["X"], device="cpu").pin_memory().copy_(q["X"]) for q in probs]
        hd = [torch.empty_like(q["D"], device="cpu").pin_memory().copy_(q["D"]) for q in probs]
        ho = [tuple(torch.empty_like(t, device="cpu").pin_memory() for t in o) for o in outs]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_steps = max(1, min(args.steps, 3))
        for _ in range(e2e_steps):
            for q, x, d in zip(probs, hx, hd):
                q["X"].copy_(x, non_blocking=True)
                q["D"].copy_(d, non_blocking=True)
            h.batched_iterate(probs, 1, out=outs)
            for q, d, o, ho_ in zip(probs, hd, outs, ho):
                d.copy_(q["D"], non_blocking=True)
                for a, b in zip(ho_, o):
                    a.copy_(b, non_blocking=True)
            torch.cuda.synchronize()
        te = time.perf_counter() - t0
        h2d = sum(q["X"].numel() * 4 + q["D"].numel() * 4 for q in probs)
        d2h = sum(q["D"].numel() * 4 + q["N"] * (q["T"] * 8 + 4) for q in probs)
        e2e = {"value": e2e_steps / te, "unit": "iter/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "steps": e2e_steps}
    line = {
        "metric": "ksvd_batched_iters_per_s", "value": args.steps / (ms / 1e3), "unit": "iter/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32" if args.precision == "fp32" else "bf16-mixed",
        "data": "synthetic (seeded, cfg3 shapes)",
        "config": {"workload": "cfg3: %d problems, n in {32,64,128,256}, K=4n, %d signals in all,"
                   " error-constrained OMP, one K-SVD iteration of every problem per step"
                   % (len(probs), Ntot), "problems": len(probs), "signals": Ntot,
                   "precision": args.precision,
                   "l2": "inputs larger than L2 (X = %.2f GB)"
                   % (sum(q["X"].numel() for q in probs) * 4 / 1e9), "autotuned": tuning},
        "omp_signals_per_s": {"value": Ntot / ((omp_ms + gemm_ms) / 1e3), "unit": "signals/s",
                              "stages": "D'X/Gram GEMMs (grouped FP32, or per-problem "
                                        "tensor-core products for the mixed path) + persistent "
                                        "batched OMP",
                              "omp_ms": omp_ms, "gemm_ms": gemm_ms},
        "support_sizes": {"min": int(sizes.min()), "mean": float(sizes.mean()),
                          "max": int(sizes.max())},
        "stage_ms_per_step_summed_over_problems": {
            k: round(v[0] / args.steps, 3) for k, v in st.items() if v[1] > 0},
        "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
        "rmse_last_mean": float(np.mean(rmse[:, -1])),
    }
    print(json.dumps(line), flush=True)
    h.close()
    return 0


def run_adjoint(args):
    """Fixed-support coding forward + adjoint backward (n=128, K=512, N=100,000, T=12): one step
    = ksvd_code_fixed then ksvd_code_backward on every signal; signals/s."""
    import torch

    from ksvd_gb300 import Handle, datagen

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    cfg = datagen.CONFIGS["cfg4"]
    p = datagen.make_problem(cfg, N=args.signals, device="cuda")
    X, D = p["X"], p["D"]
    N = X.shape[0]
    h = Handle(cfg.n, cfg.K, cfg.T)
    idx, _, nnz = h.omp(D, X)
    g = torch.Generator(device="cuda")
    g.manual_seed(7)
    dcoef = torch.randn((N, cfg.T), generator=g, device="cuda")
    dD = torch.zeros_like(D)
    dX = torch.empty_like(X)
    coef = torch.empty((N, cfg.T), dtype=torch.float32, device="cuda")
    chol = torch.empty((N, cfg.T * (cfg.T + 1) // 2), dtype=torch.float32, device="cuda")

    def step():
        h._check(h._lib.ksvd_code_fixed(h._h, _p(D), _p(X), N, _p(idx), _p(nnz), _p(coef),
                                        _p(chol)))
        dD.zero_()
        h._check(h._lib.ksvd_code_backward(h._h, _p(D), _p(X), N, _p(idx), _p(nnz), _p(coef),
                                           _p(chol), _p(dcoef), _p(dD), _p(dX)))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    # per signal: x read twice, t support columns gathered three times (L2), chol, code and
    # gradients written
    t = cfg.T
    byts = N * (2 * cfg.n * 4 + t * (t + 1) // 2 * 8 + t * 12 + cfg.n * 4 + 8)
    pk = peaks()
    line = {"metric": "adjoint_signals_per_s", "value": N / (ms / 1e3), "unit": "signals/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "dtype": "fp32", "data": "synthetic (seeded, cfg4 shape)",
            "config": {"workload": "cfg4: n=128 K=512 N=%d T=12, forward + backward" % N},
            "roofline": {"bound": "hbm", "achieved": byts / (ms / 1e3) / 1e9, "peak": pk["hbm"],
                         "unit": "GB/s", "frac": byts / (ms / 1e3) / 1e9 / pk["hbm"]}}
    print(json.dumps(line), flush=True)
    h.close()
    return 0


def _p(t):
    import ctypes

    return ctypes.c_void_p(t.data_ptr())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["fp32", "mixed"],
                    help="mixed (default): BF16 tensor-core GEMMs; the plain FP32 path is also "
                         "timed on the same workload for the ratio unless --no-compare")
    ap.add_argument("--no-compare", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="built-in launch shapes (profiler captures count launches from the start)")
    ap.add_argument("--config", default="cfg2")
    ap.add_argument("--cpu-sample", type=int, default=50000)
    ap.add_argument("--signals", type=int, default=None,
                    help="override N (smaller cases for profiler captures)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-graph", action="store_true",
                    help="time plain launches instead of CUDA-graph replays of the iteration")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    from ksvd_gb300 import datagen

    if args.config == "cfg3":
        return run_reference(args, None) if args.impl == "reference" else run_batched(args)
    if args.config == "cfg4" and args.impl != "reference":
        return run_adjoint(args)
    cfg = datagen.CONFIGS[args.config]
    if args.signals:
        import dataclasses

        cfg = dataclasses.replace(cfg, N=int(args.signals))
    if args.impl == "reference":
        return run_reference(args, cfg)
    if args.config == "cfg3":
        return run_batched(args)

    import numpy as np
    import torch

    ws, rank, local = dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from ksvd_gb300 import Handle

    # CPU baseline first (before any CUDA work in this process), rank 0 at N=1 only
    cpu = check = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        # the FP64 check runs as many iterations as this run times (warm-up included)
        cpu, check = cpu_baseline(cfg, args.cpu_sample, check_iters=args.warmup + args.steps)

    prob = datagen.make_problem(cfg, N=args.signals,
                                seed=datagen.SEED_BASE + cfg.index + 1000 * rank, device="cuda")
    X, D = prob["X"], prob["D"]
    N = X.shape[0]
    D0 = D.clone()
    # timed handle: iterations 2..K of each call replay a CUDA graph of one iteration;
    # a second, profiling handle measures per-stage times (events) in a separate pass
    h = Handle(cfg.n, cfg.K, cfg.T, precision=args.precision, graph=not args.no_graph)
    hp = Handle(cfg.n, cfg.K, cfg.T, precision=args.precision, profile=True)
    tuning = None if args.no_autotune else h.autotune(D, X)   # launch shapes timed on this workload
    if tuning:
        hp.tuning = tuning
    idx, coef, nnz = h._code(N, dev)
    out = (idx, coef, nnz)
    rms = list(h.iterate(D, X, args.warmup, out=out)[3])
    sampler = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sampler.start()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t_wall = time.perf_counter()
    e0.record(stream)
    rms += list(h.iterate(D, X, args.steps, out=out)[3])      # K steps = K iterations
    e1.record(stream)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall
    clocks = sampler.stop()
    ms = max_over_ranks(e0.elapsed_time(e1), dist, dev)
    value = aggregate_rate(1, args.steps, ms, ws)
    replays = h.graph_replays()
    # the plain FP32 path on the same workload from the same initial dictionary (the ratio the
    # mixed path is measured against; RMSE compared iteration by iteration)
    fp32_leg = None
    if args.precision == "mixed" and not args.no_compare:
        hf = Handle(cfg.n, cfg.K, cfg.T, precision="fp32", graph=not args.no_graph)
        if not args.no_autotune:
            hf.tuning = hf.autotune(D0, X)
        Df = D0.clone()
        rf = list(hf.iterate(Df, X, args.warmup, out=out)[3])
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        rf += list(hf.iterate(Df, X, args.steps, out=out)[3])
        f1.record(stream)
        torch.cuda.synchronize()
        fms = max_over_ranks(f0.elapsed_time(f1), dist, dev)
        fval = aggregate_rate(1, args.steps, fms, ws)
        fp32_leg = {"value": fval, "unit": "iter/s", "ms_per_step": fms / args.steps,
                    "mixed_over_fp32": value / fval,
                    "rmse_last_fp32": rf[-1], "rmse_last_mixed": rms[-1],
                    "rmse_max_rel_diff": max(abs(a - b) / b for a, b in zip(rms, rf)),
                    "rmse_per_iter_mixed": rms, "rmse_per_iter_fp32": rf}
        hf.close()
    if cpu is not None:
        # like for like beside the headline: the FP32 GPU path against the FP32 CPU port
        cpu["mixed_gpu_over_cpu"] = value / cpu["value"]
        if fp32_leg is not None:
            cpu["fp32_gpu_over_cpu"] = fp32_leg["value"] / cpu["value"]
    fp64_check = None
    if check is not None:
        fp64_check = error_vs_fp64(cfg, check, args.precision, dev)
    hp.iterate(D, X, 1, out=out)                  # warm the profiling handle's workspace
    hp.stage_times(reset=True)
    hp.iterate(D, X, min(args.steps, 5), out=out)
    st = hp.stage_times()

    # dominant stage and its roofline (per-launch device time from events on the kernels' stream)
    pk = peaks()
    per = {k: (v[0] / max(v[1], 1), v[1]) for k, v in st.items() if v[1] > 0}
    dom = max(per, key=lambda k: per[k][0] * per[k][1])
    launch_ms = per[dom][0]
    if dom in ("dtx", "gram") and args.precision == "mixed":
        ach = stage_flops(cfg, N, dom) / (launch_ms / 1e3) / 1e12
        roof = {"bound": "tensor", "achieved": ach, "peak": pk["bf16"], "unit": "TFLOP/s",
                "frac": ach / pk["bf16"], "traffic": None}
    else:
        ach = stage_bytes(cfg, N, dom) / (launch_ms / 1e3) / 1e9
        roof = {"bound": "hbm", "achieved": ach, "peak": pk["hbm"], "unit": "GB/s",
                "frac": ach / pk["hbm"], "traffic": None}
    fp = source_fingerprint(dom) if dom in KERNEL_SOURCES else None
    meas = MEASURED_OMP.get((cfg.n, cfg.K, cfg.T, args.precision, fp)) if dom == "omp" else None
    if meas is not None and roof["bound"] == "hbm":
        roof["traffic"] = meas[0] * N
        roof["traffic_source"] = "ncu capture at N=100000 of this kernel source, scaled by N"
    elif dom in KERNEL_SOURCES:
        roof["traffic_source"] = ("no ncu capture of kernel source %s at this shape: not "
                                  "reported" % fp)
    fl = stage_flops(cfg, N, dom)
    if dom == "omp" and fl > 0:
        # the OMP step's alpha updates also have a compute roof (FP32 CUDA cores)
        tf = fl / (launch_ms / 1e3) / 1e12
        roof["compute"] = {"achieved": tf, "peak": FP32_SIMT_TFLOPS, "unit": "TFLOP/s",
                           "frac": tf / FP32_SIMT_TFLOPS, "peak_source": "nominal FP32 SIMT"}
        gbytes = 2 if args.precision == "mixed" else 4
        roof["l2"] = {"support_column_bytes": float(N) * cfg.K * gbytes * cfg.T * (cfg.T - 1) / 2}
        if meas is not None:
            roof["l2"].update(throughput_pct_of_peak=meas[1], issue_active_pct=meas[2],
                              source="ncu lts__throughput / smsp__issue_active at N=100000")
    roof["kernel"] = dom
    roof["peak_source"] = pk["src"]
    stage_summary = {k: {"ms_per_launch": round(v[0], 4), "share": round(v[0] * v[1] / sum(
        a * b for a, b in per.values()), 4)} for k, v in per.items()}
    for k, v in stage_summary.items():
        # each stage against its own roof: algorithmic HBM bytes (or tensor FLOPs) per launch
        b = stage_bytes(cfg, N, k)
        if b and not (k in ("dtx", "gram") and args.precision == "mixed"):
            gbs = b / (v["ms_per_launch"] / 1e3) / 1e9
            v["hbm_gbs"] = round(gbs, 1)
            v["hbm_frac"] = round(gbs / pk["hbm"], 4)
        elif k in ("dtx", "gram"):
            tf = stage_flops(cfg, N, k) / (v["ms_per_launch"] / 1e3) / 1e12
            v["tflops"] = round(tf, 1)
            if args.precision == "mixed":
                v["tensor_frac_3pass"] = round(3 * tf / pk["bf16"], 4)
    omp_ms = per.get("omp", (0, 0))[0] + per.get("dtx", (0, 0))[0]

    # end to end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        Xh = torch.empty((N, cfg.n), dtype=torch.float32, pin_memory=True)
        Xh.copy_(X)
        Dh = torch.empty((cfg.K, cfg.n), dtype=torch.float32, pin_memory=True)
        Dh.copy_(D)
        Xn = Xh.numpy().T          # (n, N) column-major view of the pinned buffer
        Dn = Dh.numpy().T
        oi = torch.empty((N, cfg.T), dtype=torch.int32, pin_memory=True).numpy()
        oc = torch.empty((N, cfg.T), dtype=torch.float32, pin_memory=True).numpy()
        on = torch.empty((N,), dtype=torch.int32, pin_memory=True).numpy()
        for _ in range(max(1, args.warmup)):                  # warm the staging buffers
            h.iterate_host(Dn, Xn, 1, out=(oi, oc, on))
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        # no Python garbage collection inside the timed calls (as timeit does): a collection of
        # the benchmark's own objects is not the library's time
        gc.collect()
        gc.disable()
        t0 = time.perf_counter()
        # each call copies X and D in, runs one iteration, copies D and the code out and
        # synchronises; the per-call times are kept (the host's copies vary from call to call)
        e2e_steps = max(1, min(args.steps, 10))
        per = []
        for _ in range(e2e_steps):
            t1 = time.perf_counter()
            h.iterate_host(Dn, Xn, 1, out=(oi, oc, on))
            per.append((time.perf_counter() - t1) * 1e3)
        torch.cuda.synchronize()
        te = time.perf_counter() - t0
        gc.enable()
        te = max_over_ranks(te, dist, dev)
        e2e = {"value": aggregate_rate(1, e2e_steps, te * 1e3, ws), "unit": "iter/s",
               "h2d_bytes_per_step": int(X.numel() * 4 + D.numel() * 4),
               "d2h_bytes_per_step": int(D.numel() * 4 + N * cfg.T * 8 + N * 4 + 8),
               "steps": e2e_steps, "ms_per_call": [round(v, 2) for v in per],
               "median_rate": 1e3 / statistics.median(per)}
    if rank == 0:
        line = {
            "metric": "ksvd_iters_per_s", "value": value, "unit": "iter/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32" if args.precision == "fp32" else "bf16-mixed",
            "data": "synthetic (seeded, %s shape; reference data unpublished)" % cfg.name,
            "config": {"workload": "%s: n=%d K=%d N=%d T=%d, one K-SVD iteration per step"
                       % (cfg.name, cfg.n, cfg.K, N, cfg.T), "n": cfg.n, "K": cfg.K, "N": N,
                       "T": cfg.T, "precision": args.precision,
                       "parallelism": "replicas%d" % ws if ws > 1 else "single",
                       "cuda_graph": {"enabled": not args.no_graph,
                                      "replayed_iterations": replays},
                       "autotuned": tuning,
                       "l2": "inputs larger than L2 (X = %.2f GB)" % (X.numel() * 4 / 1e9)},
            "omp_signals_per_s": {"value": ws * N / (omp_ms / 1e3) if omp_ms else None,
                                  "unit": "signals/s", "stages": "D'X + Batch-OMP"},
            "stages": stage_summary,
            "roofline": roof,
            "fp32_path": fp32_leg,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": KERNELS_PER_CALL[args.precision] +
            args.steps * (KERNELS_PER_ITER[args.precision] + windowed_prep(cfg.n, cfg.T, N)),
            "clocks": clocks,
            "rmse_last": rms[-1] if rms else None,
            "error_vs_fp64_oracle": fp64_check,
            "wall_s_timed": t_wall,
        }
        print(json.dumps(line), flush=True)
    h.close()
    hp.close()
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
