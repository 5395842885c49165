"""Run one of the benchmark workloads for a few iterations on the GPU and print
the per-stage times: the command that profiler captures of the kernels start
from (a profiler run of a small case times one kernel at a time).

    python -m cosmopmc_gb300.profile_cases mixture --nsamples 262144 --iterations 2
    python -m cosmopmc_gb300.profile_cases sn --nsamples 10000 --iterations 4
    python -m cosmopmc_gb300.profile_cases template --nsamples 262144 --iterations 2

Workloads (seeded synthetic data): "mixture" = D=32, K=64 Student-t (nu=3,
covariance condition 1e6) proposal against a 16-component Gaussian-mixture
target; "sn" = 740 supernovae, D=6 wCDM + SALT2 nuisance, K=10 proposal from
the Fisher matrix; "template" = D=12, M=2048 data points, P=91 quadratic
monomials, K=16 proposal. Single precision (tensor cores on), every kernel
launched directly (per-stage CUDA events).
"""
import argparse

from . import pmcg as P
from . import workloads as W


def build(case, N):
    if case == "mixture":
        wl = W.mixture_workload(D=32, K=64, Kt=16, nu=3, seed=64)
        w, mu, cov, df = wl["prop"]
        wt, mut, covt, _ = wl["target"]
        prop = P.MixMvdens.from_arrays(w, mu, cov=cov, df=df).cholesky()
        target = P.MixMvdens.from_arrays(wt, mut, cov=covt, df=-1).cholesky()
        return prop, P.Posterior(32).add_mix(target), None, [target]
    if case == "sn":
        wl = W.sn_workload(K=10, init="fisher")
        w, mu, cov, df = wl["prop"]
        prop = P.MixMvdens.from_arrays(w, mu, cov=cov, df=df).cholesky()
        post = P.Posterior(6, wl["bmin"], wl["bmax"]).add_snia(wl["sn"])
        return prop, post, P.Parabox(wl["bmin"], wl["bmax"]), []
    if case == "template":
        tw = W.template_workload(D=12, M=2048, K=16)
        w, mu, cov, df = tw["prop"]
        prop = P.MixMvdens.from_arrays(w, mu, cov=cov, df=df).cholesky()
        post = P.Posterior(12, tw["bmin"], tw["bmax"]).add_template(tw["A"], tw["C"], tw["dobs"])
        return prop, post, P.Parabox(tw["bmin"], tw["bmax"]), []
    raise ValueError(case)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("case", choices=["mixture", "sn", "template"])
    ap.add_argument("--nsamples", type=int, default=1 << 18)
    ap.add_argument("--iterations", type=int, default=2)
    ap.add_argument("--seed", type=int, default=11)
    a = ap.parse_args(argv)
    P.load()
    prop, post, box, keep = build(a.case, a.nsamples)
    run = P.Run(prop, post, a.nsamples, precision=P.MIXED, seed=a.seed, box=box)
    run.set_timing(True, stages=True)
    st = None
    for _ in range(a.iterations):
        st = run.iterate(1.0)
    ms, n = run.stage_ms()
    run.free()
    names = ["draw", "logq", "logpost", "weights", "em"]
    print(f"{a.case} N={a.nsamples}: ln Z = {st['ln_evidence']:.6f}; ms per iteration "
          + ", ".join(f"{k} {v / n:.4f}" for k, v in zip(names, ms)))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
