"""Benchmark: PMC samples/s of one full iteration on the mixture microbench.

Workload (per GPU): D=32, K=64 Student-t (nu=3) proposal with condition-1e6
covariances, target a different normalised 16-component Gaussian mixture,
N = 2^20 samples; one step = draw -> log q -> log posterior -> weights /
evidence / perplexity -> Rao-Blackwellised EM update (+ Cholesky, burial).
Synthetic, seeded data of the named shapes.

`value`  : mixed-precision engine, device-resident run, samples/s over all ranks.
`e2e`    : same metric through the pmclib-named drop-in C ABI with host
           (pinned) buffers, host<->device copies inside the timed region.
fp64     : the plain FP64 path on the same workload (the drop-in baseline).
--impl reference : the CPU restatement (oracle) on all host cores, on a bounded
           sample of the same workload.
Multi-GPU: replicas only (independent runs, one per rank, no collective on the
data path); `value` = total samples / max-over-ranks time.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "PMC samples/s (one full iteration: draw, log q, log posterior, weights+evidence, RB-EM update)"
UNIT = "samples/s"
WORKLOAD = "mixture microbench: D=32, K=64 Student-t nu=3 (cond 1e6), 16-comp Gaussian-mixture target, N=2^20"


# DRAM traffic of one launch of the tensor-core proposal log-density at the
# mixture workload (N = 2^20): dram__bytes_read.sum + dram__bytes_write.sum of
# one ncu capture at N = 262144 (34.18 + 75.62 MB), scaled by 4 (traffic grows
# with N).
UMMA_TRAFFIC_BYTES = 4 * (34.18e6 + 75.62e6)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nsamples", type=int, default=1 << 20)
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--cpu-sample", type=int, default=16384)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 leg (profiling runs)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the drop-in e2e leg (profiling runs)")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-runs measurement")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving measurement")
    ap.add_argument("--no-likelihoods", action="store_true", help="skip the SN and template measurements")
    ap.add_argument("--tensor-cores", type=int, default=None, choices=[0, 1],
                    help="single-precision log-densities on tcgen05 (1) or CUDA cores (0); default: library setting")
    ap.add_argument("--profile-case", default=None, choices=["mixture", "sn", "template", "ragged"],
                    help="run one workload for --iterations iterations with every kernel launched directly and "
                         "print its per-stage times (the command that profiler captures start from); no JSON line")
    ap.add_argument("--iterations", type=int, default=2, help="iterations of --profile-case")
    return ap.parse_args()


def max_over_ranks(ms_local, world, device):
    """The largest per-rank time over all ranks, on every rank (replicas: each
    rank times its own independent run; the whole job takes the slowest)."""
    import torch
    t = torch.tensor([ms_local], dtype=torch.float64, device=device)
    if world > 1:
        import torch.distributed as dist
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, ms_max, world):
    """Units of all ranks per second of the slowest rank."""
    return units_per_rank * world / (ms_max / 1000.0)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ----------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 8:
                continue
            try:
                sm.append(float(p[0]))
                smax.append(float(p[1]))
            except ValueError:
                continue
            for nm, v in zip(names, p[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "source": "nvidia-smi, 200 ms"}


class NvmlSampler:
    """Reads the SM clock, its maximum and the clock-event reasons every 5 ms
    through NVIDIA's NVML library (ctypes; read-only queries), so a timed
    region of a few tens of milliseconds still gets samples."""
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_slowdown"}

    def __init__(self, index):
        import ctypes as C
        self.C = C
        lib = C.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        cnt = C.c_uint(0)
        lib.nvmlDeviceGetCount_v2(C.byref(cnt))
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
        ids = [v for v in vis.split(",") if v.strip()]
        if cnt.value == 1:
            idx = 0
        elif ids and all(v.strip().isdigit() for v in ids) and index < len(ids):
            idx = int(ids[index])
        else:
            idx = index
        self.h = C.c_void_p()
        if lib.nvmlDeviceGetHandleByIndex_v2(idx, C.byref(self.h)) != 0:
            raise OSError("no NVML handle")
        self.reasons_fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            lib.nvmlDeviceGetCurrentClocksThrottleReasons
        self.lib = lib
        self.samples = []
        self.stop_ev = threading.Event()

    def _run(self):
        C = self.C
        clk, mx, rs = C.c_uint(0), C.c_uint(0), C.c_ulonglong(0)
        while not self.stop_ev.is_set():
            if (self.lib.nvmlDeviceGetClockInfo(self.h, 1, C.byref(clk)) == 0 and
                    self.lib.nvmlDeviceGetMaxClockInfo(self.h, 1, C.byref(mx)) == 0 and
                    self.reasons_fn(self.h, C.byref(rs)) == 0):
                self.samples.append((clk.value, mx.value, rs.value))
            time.sleep(0.005)

    def start(self):
        self.t = threading.Thread(target=self._run, daemon=True)
        self.t.start()

    def stop(self):
        self.stop_ev.set()
        self.t.join(timeout=2)
        sm = [a for a, _, _ in self.samples]
        reasons = set()
        for _, _, r in self.samples:
            for bit, nm in self.REASONS.items():
                if r & bit:
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(b for _, b, _ in self.samples) if sm else None,
                "reasons": sorted(reasons), "samples": len(sm), "source": "NVML, 5 ms"}


def clock_sampler(index):
    try:
        return NvmlSampler(index)
    except (OSError, AttributeError):
        return ClockSampler(index)


# ----------------------------------------------------------------- workload
def build_workload(P, W, N, seed_offset=0):
    wl = W.mixture_workload(D=32, K=64, Kt=16, nu=3, seed=64)
    w, mu, cov, df = wl["prop"]
    wt, mut, covt, _ = wl["target"]
    prop = P.MixMvdens.from_arrays(w, mu, cov=cov, df=df).cholesky()
    target = P.MixMvdens.from_arrays(wt, mut, cov=covt, df=-1).cholesky()
    post = P.Posterior(32).add_mix(target)
    return prop, target, post


def flush_l2(buf):
    """Write a buffer larger than L2 (the engine's own arrays are larger too)."""
    if buf is not None:
        buf.add_(1.0)


def time_run(P, run, steps, warmup, l2buf, sync, prop, stage_steps=3):
    """Every step is one full iteration from the same starting proposal (reset
    outside the timed events), so each step does identical work. The timed
    steps run as in production (single-precision iterations replay one CUDA
    graph) and are timed whole; stage_steps more iterations with every kernel
    launched directly give the per-stage breakdown.
    Returns (stats, ms per step, per-stage ms per step, launches, wall)."""
    for _ in range(warmup):
        run.set_proposal(prop)
        run.iterate(1.0)
    run.set_timing(True, stages=False)
    launches = 0
    stats = None
    sync()
    t0 = time.perf_counter()
    for _ in range(steps):
        run.set_proposal(prop)
        flush_l2(l2buf)
        sync()
        stats = run.iterate(1.0)
        launches += run.last_launches()
    sync()
    wall = time.perf_counter() - t0
    tot, n = run.iteration_ms()
    run.set_timing(True, stages=True)
    for _ in range(stage_steps):
        run.set_proposal(prop)
        flush_l2(l2buf)
        sync()
        run.iterate(1.0)
    ms, ns = run.stage_ms()
    run.set_timing(False)
    return stats, tot / n, ([v / ns for v in ms] if ns else None), launches, wall


def same_draw_accuracy(P, prop, post, N, seed=2024):
    """Both paths on the same draw: one iteration of a fresh mixed and a fresh
    FP64 run with one seed (the samples agree to single precision), compared
    by ln Z and by the weighted posterior mean and covariance in units of the
    FP64 posterior standard deviations."""
    out = {}
    for prec, tag in ((P.MIXED, "mixed"), (P.FP64, "fp64")):
        r = P.Run(prop, post, N, precision=prec, seed=seed)
        st = r.iterate(1.0)
        s = r.sample()
        mean, cov = s.weighted_moments()
        out[tag] = (st["ln_evidence"], mean, cov)
        del s
        r.free()
    (z32, m32, c32), (z64, m64, c64) = out["mixed"], out["fp64"]
    sig = np.sqrt(np.diag(c64))
    return {"draw": f"first iteration of fresh runs, seed {seed}, both paths", "ln_evidence_mixed": z32,
            "ln_evidence_fp64": z64, "abs_dlnZ": abs(z32 - z64),
            "posterior_mean_max_sigma": float(np.max(np.abs(m32 - m64) / sig)),
            "posterior_cov_max_sigma2": float(np.max(np.abs(c32 - c64) / np.outer(sig, sig)))}


def oracle_iteration_rate(O, prop, lpf, bmin, bmax, n, min_s=3.0, max_reps=4):
    """samples/s of whole FP64 oracle iterations (draw, log q, log posterior,
    weights, EM) on the host cores, from the same proposal each time."""
    t0 = time.perf_counter()
    reps = 0
    while True:
        O.iterate_posterior(prop, lpf, n, 11, reps, 1.0, bmin, bmax)
        reps += 1
        el = time.perf_counter() - t0
        if el > min_s or reps >= max_reps:
            return n * reps / el, reps


def likelihood_bench(P, W, l2buf, sync, steps=5, warmup=3, O=None):
    """The other likelihoods at their configuration sizes: SN Ia (D=6, K=10, 740
    supernovae, Fisher start; N = 10^4 as configured and N = 2^18) and the dense
    template (D=12, K=16, M=2048, N = 2^18, Fisher start); mixed precision vs
    FP64, same seeds. With the oracle module O: the FP64 oracle's iterations on
    the host cores beside them (SN at N = 10^4, the template on a 2^14 sample)."""
    out = {}
    wl = W.sn_workload(K=10, init="fisher")
    w, mu, cov, df = wl["prop"]
    sn_prop = P.MixMvdens.from_arrays(w, mu, cov=cov, df=df).cholesky()
    sn_post = P.Posterior(6, wl["bmin"], wl["bmax"]).add_snia(wl["sn"])
    sn_box = P.Parabox(wl["bmin"], wl["bmax"])
    tw = W.template_workload(D=12, M=2048, K=16)
    w, mu, cov, df = W.fisher_proposal(np.random.default_rng(92), 16, tw["theta0"], W.template_fisher(tw),
                                       tw["bmin"], tw["bmax"])
    tpl_prop = P.MixMvdens.from_arrays(w, mu, cov=cov, df=df).cholesky()
    tpl_post = P.Posterior(12, tw["bmin"], tw["bmax"]).add_template(tw["A"], tw["C"], tw["dobs"])
    tpl_box = P.Parabox(tw["bmin"], tw["bmax"])
    cases = [("sn_N1e4", sn_prop, sn_post, sn_box, 10000), ("sn_N2e18", sn_prop, sn_post, sn_box, 1 << 18),
             ("template_N2e18", tpl_prop, tpl_post, tpl_box, 1 << 18)]
    for name, prop, post, box, N in cases:
        rec = {"N": N}
        for prec, tag in ((P.MIXED, "mixed"), (P.FP64, "fp64")):
            run = P.Run(prop, post, N, precision=prec, seed=11, box=box)
            st, step, ms, _, _ = time_run(P, run, steps, warmup, l2buf, sync, prop)
            rec[tag] = {"samples_per_s": N / (step / 1e3), "ms_per_step": step, "ln_evidence": st["ln_evidence"],
                        "stage_ms": ms}
            run.free()
        rec["speedup_mixed_vs_fp64"] = rec["mixed"]["samples_per_s"] / rec["fp64"]["samples_per_s"]
        out[name] = rec
    if O is not None:
        ow, omu, oL = sn_prop.arrays()
        lpr = -np.sum(np.log(wl["bmax"] - wl["bmin"]))

        def sn_lpf(X, flg):
            l, ok = O.sn_loglike(wl["sn"], X, flg)
            return l + lpr, ok

        v, reps = oracle_iteration_rate(O, O.Mix(ow, omu, df=sn_prop.df, L=oL), sn_lpf, wl["bmin"], wl["bmax"], 10000)
        out["sn_N1e4"]["cpu_oracle"] = {"samples_per_s": v, "cores": O.num_threads(),
                                        "sample": f"{reps} x 10^4 samples (whole iterations)"}
        At, dt = O.tpl_prepare(tw["A"], tw["C"], tw["dobs"])
        tpr = -np.sum(np.log(tw["bmax"] - tw["bmin"]))

        def tpl_lpf(X, flg):
            return O.tpl_loglike(At, dt, X, flg) + tpr, np.ones(len(X), np.int16)

        ow, omu, oL = tpl_prop.arrays()
        v, reps = oracle_iteration_rate(O, O.Mix(ow, omu, df=tpl_prop.df, L=oL), tpl_lpf, tw["bmin"], tw["bmax"],
                                        1 << 14)
        out["template_N2e18"]["cpu_oracle"] = {"samples_per_s": v, "cores": O.num_threads(),
                                               "sample": f"{reps} x 2^14 samples (whole iterations)"}
    return out


TEMPER_LEVELS, TEMPER_TMIN = 10, 0.01


def tempering_level(rng):
    """A tempering level of the log schedule (exec/cosmo_pmc.c:464-495): the beta
    of a random iteration of a 10-level schedule starting at t_min = 0.01."""
    from cosmopmc_gb300 import pmcg as P
    return P.get_tempering_beta(P.TEMPERING_LOG, int(rng.integers(0, TEMPER_LEVELS)), TEMPER_TMIN, TEMPER_LEVELS)


def ragged_specs(R, seed=256):
    """Batched workload: R runs, half SN-type (740 supernovae, the six SN parameters
    plus Gaussian nuisance parameters in a flat box, D ~ U{6..20}, Fisher-matrix
    start), half
    Gaussian-mixture targets with D ~ U{2..20}; K ~ U{1..20}, N ~ logU(1e3, 1e5);
    each run at a tempering level of the log schedule."""
    rng = np.random.default_rng(seed)
    specs = []
    for r in range(R):
        N = int(round(np.exp(rng.uniform(np.log(1e3), np.log(1e5)))))
        K = int(rng.integers(1, 21))
        beta = tempering_level(rng)
        if r % 2 == 0:
            specs.append(("sn", int(rng.integers(6, 21)), max(K, 2), N, 740 + r, beta))
        else:
            specs.append(("mix", int(rng.integers(2, 21)), K, N, 1000 + r, beta))
    return specs


NUIS_HALF, NUIS_SD = 1.0, 0.25   # nuisance parameters: box [-1, 1], Gaussian term N(0, 0.25^2)


def build_spec(P, W, spec, cache, beta0=1.0):
    """Proposal, posterior and box of one run, started for the tempered target p^beta0
    (beta0: the tempering level the run starts at). Fisher starts use the Fisher
    matrix beta0 F, with every standard deviation capped at a quarter of the box
    width; Gaussian-mixture starts have their covariances divided by beta0."""
    kind, D, K, N, seed = spec[:5]
    if kind == "sn":
        if "sn_data" not in cache:
            wl = W.sn_workload()
            cache["sn_data"] = wl["sn"]
            cache["sn_fisher"] = W.sn_fisher(wl["sn"], W.SN_TRUTH)
        if ("sn_post", D) not in cache:
            bmin = np.concatenate([W.SN_BOX_MIN, -NUIS_HALF * np.ones(D - 6)])
            bmax = np.concatenate([W.SN_BOX_MAX, NUIS_HALF * np.ones(D - 6)])
            F = np.zeros((D, D))
            F[:6, :6] = cache["sn_fisher"]
            F[6:, 6:] = np.eye(D - 6) / NUIS_SD ** 2
            theta0 = np.concatenate([W.SN_TRUTH, np.zeros(D - 6)])
            post = P.Posterior(D, bmin, bmax).add_snia(cache["sn_data"])
            if D > 6:   # Gaussian nuisance parameters: a Gaussian term on the subset 6..D-1
                post.add_prior(np.zeros(D - 6), NUIS_SD ** 2 * np.eye(D - 6), df=-1,
                               indprior=np.r_[np.zeros(6, int), np.ones(D - 6, int)])
            cache[("sn_post", D)] = (post, P.Parabox(bmin, bmax), F, theta0, bmin, bmax)
        post, box, F, theta0, bmin, bmax = cache[("sn_post", D)]
        rng = np.random.default_rng(seed)
        w, mu, cov, df = W.fisher_proposal(rng, K, theta0, beta0 * F, bmin, bmax, box_frac=0.25)
        return P.MixMvdens.from_arrays(w, mu, cov=cov, df=df).cholesky(), post, box
    if kind == "tpl":
        if "tpl_post" not in cache:
            wl = W.template_workload(D=12, M=2048, K=16)
            cache["tpl_post"] = (P.Posterior(12, wl["bmin"], wl["bmax"]).add_template(wl["A"], wl["C"], wl["dobs"]),
                                 P.Parabox(wl["bmin"], wl["bmax"]))
            cache["tpl_fisher"] = (W.template_fisher(wl), wl["theta0"])
        post, box = cache["tpl_post"]
        F, theta0 = cache["tpl_fisher"]
        rng = np.random.default_rng(seed)
        w, mu, cov, df = W.fisher_proposal(rng, K, theta0, beta0 * F, -np.ones(12), np.ones(12), box_frac=0.25)
        return P.MixMvdens.from_arrays(w, mu, cov=cov, df=df).cholesky(), post, box
    wl = W.mixture_workload(D=D, K=K, Kt=max(1, K // 3), nu=-1, seed=seed, prop_hi=2.0)
    w, mu, cov, df = wl["prop"]
    wt, mut, covt, _ = wl["target"]
    # the tempered target p^beta0 of a Gaussian component has covariance cov / beta0:
    # the start is widened to match (a start fitted to beta = 1 under a flat target
    # leaves the weights to the proposal's tails)
    prop = P.MixMvdens.from_arrays(w, mu, cov=cov / beta0, df=df).cholesky()
    target = P.MixMvdens.from_arrays(wt, mut, cov=covt, df=-1).cholesky()
    post = P.Posterior(D).add_mix(target)
    cache.setdefault("keep", []).append(target)
    return prop, post, None


def _iterate_each(P, runs, betas, reps, sizes):
    """(seconds per pass of one iteration of every run, one run at a time;
    samples per pass of the iterations that succeeded)."""
    import torch
    for r, b in zip(runs, betas):  # warm-up
        try:
            r.iterate(b)
        except P.PmcgError:
            pass
    torch.cuda.synchronize()
    ok = 0
    t0 = time.perf_counter()
    for _ in range(reps):
        for r, b, n in zip(runs, betas, sizes):
            try:
                r.iterate(b)
                ok += n
            except P.PmcgError:
                pass
    torch.cuda.synchronize()
    return (time.perf_counter() - t0) / reps, ok / reps


def batch_bench(P, W, R=256, iters=5):
    """256 ragged runs: one persistent launch per iteration vs the same runs one at
    a time (mixed precision) and vs the plain FP64 path one at a time."""
    specs = ragged_specs(R)
    cache = {}
    built = [build_spec(P, W, s, cache, beta0=s[5]) for s in specs]
    betas = np.array([s[5] for s in specs])

    def make_runs(prec):
        runs = []
        for s, (pp, po, bx) in zip(specs, built):
            r = P.Run(pp, po, s[3], precision=prec, seed=s[4], box=bx)
            if bx is not None:
                r.set_dead_comp(P.DEAD_REVIVE, 0.1)   # revival needs the prior box
            runs.append(r)
        return runs

    runs_b = make_runs(P.MIXED)
    total = sum(s[3] for s in specs)
    batch = P.Batch(runs_b)
    t0 = time.perf_counter()
    batch.autotune()
    tune_s = time.perf_counter() - t0
    sizes = [s[3] for s in specs]
    batch.iterate(betas)  # warm-up
    ms, rates = [], []
    failed, failed_runs = {}, set()
    for _ in range(iters):
        st = batch.iterate(betas)
        ms.append(batch.last_ms())
        # samples of the runs whose iteration succeeded (a run whose update buried
        # every component stops, as the reference's update does, and its later
        # iterations draw from a dead proposal: counted as failures, no samples)
        rates.append(sum(n for n, x in zip(sizes, st) if x["status"] == 0) / (ms[-1] / 1e3))
        for i, (s, x) in enumerate(zip(specs, st)):
            if x["status"] != 0:
                key = f"{s[0]}:{x['status']}"
                failed[key] = failed.get(key, 0) + 1
                failed_runs.add(i)
    med = float(np.median(ms))
    cfg = batch.config()
    # one more iteration with its stages launched one by one (per-stage times)
    batch.set_stage_timing(True)
    batch.iterate(betas)
    stage_ms = batch.stage_ms()
    batch.free()
    del runs_b
    runs_s = make_runs(P.MIXED)
    seq_s, seq_ok = _iterate_each(P, runs_s, betas, 2, sizes)
    for r in runs_s:
        r.free()
    runs_64 = make_runs(P.FP64)
    fp64_s, fp64_ok = _iterate_each(P, runs_64, betas, 1, sizes)
    for r in runs_64:
        r.free()
    value = float(np.median(rates))
    return {"workload": f"{R} runs, half SN (D~U{{6..20}}: 6 SN parameters + Gaussian nuisance in a flat box, "
                        f"start from the tempered Fisher matrix, dead components revived), half GMM "
                        f"(D~U{{2..20}}), K~U{{1..20}}, N~logU(1e3,1e5), beta from the log tempering schedule "
                        f"(t_min {TEMPER_TMIN}, {TEMPER_LEVELS} levels)",
            "samples_per_iter": total, "value": value, "unit": UNIT, "ms_per_iter": med,
            "one_run_at_a_time_samples_per_s": seq_ok / seq_s, "speedup_vs_one_at_a_time": (seq_s * 1e3) / med,
            "fp64_one_run_at_a_time_samples_per_s": fp64_ok / fp64_s,
            "speedup_mixed_vs_fp64": value / (fp64_ok / fp64_s),
            "config": cfg, "autotune_s": tune_s, "failed_run_iterations": failed, "failed_runs": len(failed_runs),
            "stage_ms": stage_ms,
            "failed_note": "kind:status of timed run iterations that failed (-9005: the update buried every "
                           "component; -9011: no sample with a weight, the later iterations of such a run); "
                           "value counts the samples of the runs whose iteration succeeded",
            "timing": "CUDA events around each graph launch (library stream), median of iterations; the one-at-a-time "
                      "legs by host clock around a synchronised pass over all runs"}


def serve_bench(P, W, rates=(10, 30, 100, 300, 1000, 2000), window_s=2.5, seed=4, fp64_jobs=96):
    """Poisson arrivals of jobs (90% from the ragged mix, 10% template-sized), 5-10
    iterations each on the log tempering schedule; and the plain FP64 path on jobs
    drawn from the same mix, run one after another."""
    rng = np.random.default_rng(seed)
    pool_specs = ragged_specs(64, seed=99)
    cache = {}
    # jobs run the log schedule from t_min: Fisher starts use t_min F
    pool = [(s, build_spec(P, W, s, cache, beta0=TEMPER_TMIN)) for s in pool_specs]
    tpl_spec = ("tpl", 12, 16, 262144, 91, 1.0)
    tpl = (tpl_spec, build_spec(P, W, tpl_spec, cache, beta0=TEMPER_TMIN))

    def pick(r):
        return tpl if r.uniform() < 0.1 else pool[int(r.integers(0, len(pool)))]

    out = []
    for rate in rates:
        srv = P.Server(dead_comp=P.DEAD_REVIVE, fshift=0.1)
        n_jobs = max(8, int(rate * window_s))
        arrivals = np.cumsum(rng.exponential(1.0 / rate, n_jobs))
        ids = []
        t_start = time.perf_counter()
        for i in range(n_jobs):
            dt = arrivals[i] - (time.perf_counter() - t_start)
            if dt > 0:
                time.sleep(dt)
            spec, (pp, po, bx) = pick(rng)
            niter = int(rng.integers(5, 11))
            ids.append((srv.submit(pp, po, spec[3], niter, int(rng.integers(1, 1 << 30)), box=bx,
                                   tempering=P.TEMPERING_LOG, t_min=TEMPER_TMIN), spec[3], niter, spec[0]))
        res = [(srv.wait(j, timeout=600), n, it, kind) for j, n, it, kind in ids]
        wall = time.perf_counter() - t_start
        info = srv.info()
        srv.free()
        lat = np.array([r["finish_s"] - r["submit_s"] for r, _, _, _ in res if r["status"] == 0])
        samples = sum(n * it for r, n, it, _ in res if r["status"] == 0)
        failed = {}
        for r, _, _, kind in res:
            if r["status"] != 0:
                key = f"{kind}:{r['status']}"
                failed[key] = failed.get(key, 0) + 1
        out.append({"rate_jobs_per_s": rate, "jobs": n_jobs, "ok": int(len(lat)), "failed_status": failed,
                    "p50_ms": float(np.percentile(lat, 50) * 1e3) if len(lat) else None,
                    "p99_ms": float(np.percentile(lat, 99) * 1e3) if len(lat) else None,
                    "samples_per_s": samples / wall, "peak_resident": info["peak_resident"],
                    "epochs": info["epochs"]})
    # plain FP64 path: jobs of the same mix, each run to completion before the next
    import torch
    r64 = np.random.default_rng(seed + 1)
    jobs = []
    for _ in range(fp64_jobs):
        spec, (pp, po, bx) = pick(r64)
        jobs.append((spec, pp, po, bx, int(r64.integers(5, 11)), int(r64.integers(1, 1 << 30))))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    samples64, failed64 = 0, 0
    for spec, pp, po, bx, niter, sd in jobs:
        run = P.Run(pp, po, spec[3], precision=P.FP64, seed=sd, box=bx)
        if bx is not None:
            run.set_dead_comp(P.DEAD_REVIVE, 0.1)
        try:
            for it in range(niter):
                run.iterate(P.get_tempering_beta(P.TEMPERING_LOG, it, TEMPER_TMIN, niter))
            samples64 += spec[3] * niter
        except P.PmcgError:
            failed64 += 1
        run.free()
    torch.cuda.synchronize()
    fp64_rate = samples64 / (time.perf_counter() - t0)
    peak = max(r["samples_per_s"] for r in out)
    return {"workload": "Poisson arrivals; 90% jobs from the ragged mix, 10% template-sized (D=12, N=2^18, "
                        "M=2048); Fisher starts from the t_min-tempered Fisher matrix; 5-10 iterations per job on "
                        f"the log tempering schedule (t_min {TEMPER_TMIN}); dead components revived (jobs with a "
                        "prior box); mixed precision",
            "latency": "job submit to result (server clock)", "rates": out,
            "fp64": {"samples_per_s": fp64_rate, "jobs": fp64_jobs, "failed": failed64,
                     "how": "plain FP64 runs of jobs drawn from the same mix (job creation included), one job "
                            "at a time, host clock"},
            "speedup_mixed_vs_fp64": peak / fp64_rate}


def cpu_baseline(O, W, nsample, seed=5):
    wl = W.mixture_workload(D=32, K=64, Kt=16, nu=3, seed=64)
    w, mu, cov, df = wl["prop"]
    wt, mut, covt, _ = wl["target"]
    prop = O.Mix(w, mu, cov, df=df)
    target = O.Mix(wt, mut, covt, df=-1)
    O.iterate_mix(prop.copy(), target, 0.0, 1024, seed, 0, check=False)  # warm the pages
    t0 = time.perf_counter()
    reps = 0
    while True:
        O.iterate_mix(prop.copy(), target, 0.0, nsample, seed, reps, check=False)
        reps += 1
        el = time.perf_counter() - t0
        if el > 8.0 or reps >= 4:
            break
    return nsample * reps / el, O.num_threads(), reps


def workload_config(N, world):
    """The config of both arms (identical keys and values)."""
    return {"workload": WORKLOAD, "global_batch": N * world, "nsamples_per_gpu": N, "D": 32, "K": 64, "nu": 3,
            "target_components": 16, "parallelism": "replicas" if world > 1 else "single",
            "l2": "flushed between steps (256 MB write); per-iteration arrays also exceed L2"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from cosmopmc_gb300 import workloads as W
    O.build()
    wl = W.mixture_workload(D=32, K=64, Kt=16, nu=3, seed=64)
    w, mu, cov, df = wl["prop"]
    wt, mut, covt, _ = wl["target"]
    prop = O.Mix(w, mu, cov, df=df)
    target = O.Mix(wt, mut, covt, df=-1)
    n = args.nsamples   # the whole workload per step, as the GPU arm
    for i in range(args.warmup):
        O.iterate_mix(prop.copy(), target, 0.0, n, 5, i, check=False)
    times = []
    for i in range(args.steps):
        p = prop.copy()  # same starting proposal every step, as in the GPU arm
        t0 = time.perf_counter()
        O.iterate_mix(p, target, 0.0, n, 5, args.warmup + i, check=False)
        times.append(time.perf_counter() - t0)
    ms = 1000.0 * sum(times) / len(times)
    v = n / (ms / 1000.0)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded, shapes of the mixture microbench)",
        "config": workload_config(n, world),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": O.num_threads(), "kind": "port",
                         "sample": f"the whole workload ({n} samples) per step; oracle/pmc_oracle.c, OpenMP over "
                                   f"all host threads"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def profile_case(args):
    """One workload of the benchmark, mixed precision, every kernel launched
    directly with per-stage CUDA events, after one untimed iteration from the same
    proposal: "mixture" (D=32, K=64 Student-t nu=3,
    condition 1e6, 16-component target), "sn" (740 supernovae, D=6, K=10 Fisher
    start), "template" (D=12, M=2048, P=91, K=16, Fisher start)."""
    from cosmopmc_gb300 import pmcg as P
    from cosmopmc_gb300 import workloads as W
    P.load()
    if args.tensor_cores is not None:
        P.set_tensor_cores(args.tensor_cores)
    if args.profile_case == "ragged":
        return profile_ragged(P, W)
    N = args.nsamples
    box = None
    if args.profile_case == "mixture":
        prop, target, post = build_workload(P, W, N)
    elif args.profile_case == "sn":
        wl = W.sn_workload(K=10, init="fisher")
        w, mu, cov, df = wl["prop"]
        prop = P.MixMvdens.from_arrays(w, mu, cov=cov, df=df).cholesky()
        post = P.Posterior(6, wl["bmin"], wl["bmax"]).add_snia(wl["sn"])
        box = P.Parabox(wl["bmin"], wl["bmax"])
    else:
        tw = W.template_workload(D=12, M=2048, K=16)
        w, mu, cov, df = W.fisher_proposal(np.random.default_rng(92), 16, tw["theta0"], W.template_fisher(tw),
                                           tw["bmin"], tw["bmax"])
        prop = P.MixMvdens.from_arrays(w, mu, cov=cov, df=df).cholesky()
        post = P.Posterior(12, tw["bmin"], tw["bmax"]).add_template(tw["A"], tw["C"], tw["dobs"])
        box = P.Parabox(tw["bmin"], tw["bmax"])
    run = P.Run(prop, post, N, precision=P.MIXED, seed=11, box=box)
    run.iterate(1.0)               # untimed: loads every kernel (lazy module loading)
    run.set_proposal(prop)
    run.set_timing(True, stages=True)
    st = None
    for _ in range(args.iterations):
        st = run.iterate(1.0)
    ms, n = run.stage_ms()
    run.free()
    names = ["draw", "logq", "logpost", "weights", "em"]
    print(f"{args.profile_case} N={N}: ln Z = {st['ln_evidence']:.6f}; ms per iteration "
          + ", ".join(f"{k} {v / n:.4f}" for k, v in zip(names, ms)), flush=True)
    return 0


def profile_ragged(P, W, R=256):
    """The batched workload's runs one at a time (mixed precision), every kernel
    launched directly with per-stage CUDA events: the stage times summed over the
    runs, by run kind, for one iteration after an untimed one."""
    specs = ragged_specs(R)
    cache = {}
    names = ["draw", "logq", "logpost", "weights", "em"]
    tot = {}
    for s in specs:
        pp, po, bx = build_spec(P, W, s, cache, beta0=s[5])
        run = P.Run(pp, po, s[3], precision=P.MIXED, seed=s[4], box=bx)
        if bx is not None:
            run.set_dead_comp(P.DEAD_REVIVE, 0.1)
        try:
            run.iterate(s[5])
            run.set_timing(True, stages=True)
            run.iterate(s[5])
            ms, n = run.stage_ms()
        except P.PmcgError:
            run.free()
            continue
        run.free()
        t = tot.setdefault(s[0], [0.0] * 5 + [0])
        for i in range(5):
            t[i] += ms[i] / n
        t[5] += s[3]
    for kind, t in tot.items():
        print(f"ragged {kind}: {t[5]} samples; ms summed over runs " +
              ", ".join(f"{k} {v:.3f}" for k, v in zip(names, t[:5])), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_case:
        return profile_case(args)
    rank, world, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from cosmopmc_gb300 import pmcg as P
    from cosmopmc_gb300 import workloads as W

    P.load()
    if args.tensor_cores is not None:
        P.set_tensor_cores(args.tensor_cores)
    N = args.nsamples
    prop, target, post = build_workload(P, W, N)
    l2buf = torch.zeros(64 << 20, dtype=torch.float32, device="cuda")  # 256 MB > L2
    sync = torch.cuda.synchronize

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        sync()

    # ---------------- mixed-precision engine (the headline)
    run = P.Run(prop, post, N, precision=P.MIXED, seed=1000 + rank)
    barrier()
    clk = clock_sampler(local)
    clk.start()
    stats, step_ms, stage_ms, launches, wall = time_run(P, run, args.steps, args.warmup, l2buf, sync, prop)
    clocks = clk.stop()
    barrier()
    nt = 1  # stage_ms is per step
    step_ms_max = max_over_ranks(step_ms, world, "cuda")
    value = whole_job_rate(N, step_ms_max, world)

    # ---------------- plain FP64 path on the same workload
    fp64 = None
    if not args.no_fp64:
        run64 = P.Run(prop, post, N, precision=P.FP64, seed=1000 + rank)
        s64, fp64_ms, _, _, _ = time_run(P, run64, args.fp64_steps, 1, l2buf, sync, prop, stage_steps=0)
        fp64_ms = max_over_ranks(fp64_ms, world, "cuda")
        fp64_value = whole_job_rate(N, fp64_ms, world)
        run64.free()
        fp64 = {"value": fp64_value, "unit": UNIT, "ms_per_step": fp64_ms, "steps": args.fp64_steps,
                "speedup_mixed_vs_fp64": value / fp64_value,
                "accuracy": same_draw_accuracy(P, prop, post, N)}
    if args.no_e2e:
        return finish(args, rank, world, value, step_ms_max, N, stats, fp64, None, launches, stage_ms, nt, clocks,
                      W)

    # ---------------- e2e: drop-in C ABI with host buffers (mixed precision)
    P.set_dropin_precision(P.MIXED)
    ps = P.PmcSimu(N, 32)
    rng = P.Rng(7 + rank)
    w0, mu0, L0 = prop.arrays()
    m = P.MixMvdens.from_arrays(w0, mu0, L=L0, df=prop.df)

    def dropin_step():
        P.simulate_mix_mvdens(ps, m, rng, None)
        P.importance_weights(ps, m, post, 1.0)
        P.normalize_importance_weight(ps)
        P.update_prop_rb(m, ps)
        P.perplexity_and_ess(ps)
        return P.evidence(ps)

    for _ in range(args.warmup):
        m.set(w0, mu0, L=L0, df=prop.df)
        dropin_step()
    barrier()
    e2e_tot = 0.0
    for _ in range(args.steps):
        m.set(w0, mu0, L=L0, df=prop.df)   # same starting proposal every step (host side, untimed)
        flush_l2(l2buf)
        sync()
        t0 = time.perf_counter()
        dropin_step()
        e2e_tot += time.perf_counter() - t0
    e2e_ms = 1000.0 * e2e_tot / args.steps
    e2e_ms_max = max_over_ranks(e2e_ms, world, "cuda")
    e2e_value = whole_job_rate(N, e2e_ms_max, world)
    K, D = 64, 32
    h2d = K * (1 + D + D * D) * 8 + 2 * K * (1 + D + D * D) * 8   # proposal uploads (draw + update)
    d2h = N * D * 8 + N * 4 + N * 2 + N * 8 + N * 2 + N * 8 + K * (1 + D + D * D) * 8
    e2e = {"value": e2e_value, "unit": UNIT, "ms_per_step": e2e_ms_max, "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h,
           "path": "simulate_mix_mvdens + generic_get_importance_weight + normalize + update_prop_rb + "
                   "perplexity_and_ess + evidence, pinned pmc_simu host arrays",
           "link": link_rates(N * D * 8)}
    e2e["link"]["d2h_floor_ms"] = d2h / (e2e["link"]["d2h_gbs"] * 1e6)
    return finish(args, rank, world, value, step_ms_max, N, stats, fp64, e2e, launches, stage_ms, nt, clocks, W)


def link_rates(nbytes, reps=5):
    """The host link on its own: one device -> pinned-host copy (and back) of the
    FP64 sample's size, cudaMemcpyAsync through torch, CUDA events, best of reps."""
    import torch
    dev = torch.empty(nbytes // 8, dtype=torch.float64, device="cuda")
    host = torch.empty(nbytes // 8, dtype=torch.float64, pin_memory=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = {"bytes": nbytes}
    for tag, dst, src in (("d2h_gbs", host, dev), ("h2d_gbs", dev, host)):
        best = None
        for _ in range(reps):
            torch.cuda.synchronize()
            e0.record()
            dst.copy_(src, non_blocking=True)
            e1.record()
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        out[tag] = nbytes / (best * 1e6)
    del dev, host
    return out


def finish(args, rank, world, value, step_ms_max, N, stats, fp64, e2e, launches, stage_ms, nt, clocks, W):
    K, D = 64, 32
    # ---------------- roofline of the dominant kernel
    from cosmopmc_gb300 import pmcg as P
    tc = P.set_tensor_cores(True)
    P.set_tensor_cores(tc)
    stage_names = ["draw", "logq", "logpost", "weights", "em"]
    per_stage = {nm: v / nt for nm, v in zip(stage_names, stage_ms)}
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    sm_mhz = clocks.get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
    # algorithmic flops of the proposal log-density per launch: the batched
    # Mahalanobis contraction X [N x D] times K factors [D x D], 2 N K D^2
    flops = 2.0 * N * K * D * D
    t_ms = per_stage["logq"]
    achieved = flops / (t_ms / 1000.0) / 1e12
    if tc:
        bf16 = peaks.get("bf16_tflops")
        peak = bf16 if bf16 else 1900.0
        roof = {"bound": "tensor", "kernel": "umma_logq_kernel (tcgen05 kind::tf32, three-term split)",
                "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                # DRAM bytes per launch at this workload from an ncu capture (lt and Q writes dominate)
                "traffic": UMMA_TRAFFIC_BYTES, "stage_ms": per_stage,
                "peak_note": ("measured cuBLAS bf16 dense burst rate (MEASURED_PEAKS.json bf16_tflops)"
                              if bf16 else "fallback bf16 1.9 PFLOP/s"),
                "flops_note": "2 N K D^2 per launch (the full D x D product per sample and component); the "
                              "kernel multiplies only the lower triangle, three times (TF32 split), in "
                              "kind::tf32, whose dense rate is half the bf16 one: against that rate "
                              f"frac = {2 * achieved / peak:.3f}",
                "tf32_frac": 2 * achieved / peak}
    else:
        fp32_peak = 152 * 128 * 2 * (sm_mhz * 1e6) / 1e12
        roof = {"bound": "fp32", "kernel": "mixlogpdf_f32_kernel", "achieved": achieved, "peak": fp32_peak,
                "unit": "TFLOP/s", "frac": achieved / fp32_peak, "traffic": None, "stage_ms": per_stage,
                "peak_note": "FP32 CUDA-core peak derived from 152 SMs x 128 lanes x 2 x median SM clock under load"}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms_max, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded)",
        "config": workload_config(N, world),
        "timing": "CUDA events on the library stream around each iteration as run in production (one replayed CUDA "
                  "graph per iteration); roofline.stage_ms from 3 more iterations with every kernel launched "
                  "directly",
        "fp64": fp64,
        "iteration_stats": {k: stats[k] for k in ("ln_evidence", "perplexity", "ess", "enc")},
        "e2e": e2e,
        "gpu_launches": launches,
        "roofline": roof,
        "clocks": clocks,
    }
    O = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        O.build()
        v, cores, reps = cpu_baseline(O, W, args.cpu_sample)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": f"{reps} x {args.cpu_sample} samples of this workload "
                                          f"(oracle/pmc_oracle.c, OpenMP)"}
    if not args.no_likelihoods:
        import torch
        l2 = torch.zeros(64 << 20, dtype=torch.float32, device="cuda")
        line["likelihoods"] = likelihood_bench(P, W, l2, torch.cuda.synchronize, O=O)
        del l2
    if not args.no_batch:
        line["batch"] = batch_bench(P, W)
    if not args.no_serve:
        line["serving"] = serve_bench(P, W)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
