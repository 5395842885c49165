"""Single-precision iterations replay one captured CUDA graph (per-iteration
beta and call counter read from device memory): the results equal those of
the same iterations with every kernel launched directly, bit for bit."""
import numpy as np
import pytest

from cosmopmc_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def run_pair(pmcg, prop, post, N, box=None, iters=3, betas=(0.7, 1.0, 1.0)):
    graph = pmcg.Run(prop, post, N, precision=pmcg.MIXED, seed=19, box=box)
    direct = pmcg.Run(prop, post, N, precision=pmcg.MIXED, seed=19, box=box)
    direct.set_timing(True, stages=True)   # per-stage timing launches every kernel directly
    out = []
    for it in range(iters):
        sg = graph.iterate(betas[it])
        sd = direct.iterate(betas[it])
        out.append((sg, sd, graph.sample(), direct.sample(), graph.proposal().arrays(), direct.proposal().arrays()))
    graph.free()
    direct.free()
    return out


def assert_same(out):
    for sg, sd, pg, pd, mg, md in out:
        for k in ("ln_evidence", "perplexity", "ess", "enc", "logSum"):
            assert sg[k] == sd[k], (k, sg[k], sd[k])
        np.testing.assert_array_equal(pg.X, pd.X)
        np.testing.assert_array_equal(pg.indices, pd.indices)
        np.testing.assert_array_equal(pg.weights, pd.weights)
        for a, b in zip(mg, md):
            np.testing.assert_array_equal(a, b)


def test_graph_iterations_equal_direct_mixture(pmcg):
    wl = W.mixture_workload(D=32, K=64, Kt=16, seed=64)
    w, mu, cov, df = wl["prop"]
    wt, mut, covt, _ = wl["target"]
    prop = pmcg.MixMvdens.from_arrays(w, mu, cov=cov, df=df).cholesky()
    target = pmcg.MixMvdens.from_arrays(wt, mut, cov=covt, df=-1).cholesky()
    post = pmcg.Posterior(32).add_mix(target)
    assert_same(run_pair(pmcg, prop, post, 40000))


def test_graph_iterations_equal_direct_sn_with_box(pmcg):
    wl = W.sn_workload(K=10, init="fisher")
    w, mu, cov, df = wl["prop"]
    prop = pmcg.MixMvdens.from_arrays(w, mu, cov=cov, df=df).cholesky()
    post = pmcg.Posterior(6, wl["bmin"], wl["bmax"]).add_snia(wl["sn"])
    assert_same(run_pair(pmcg, prop, post, 10000, box=pmcg.Parabox(wl["bmin"], wl["bmax"])))


def test_graph_recaptured_when_tensor_cores_switch(pmcg):
    """The captured graph holds the log-density kernel chosen at capture: a
    switch between iterations re-captures, matching direct launches."""
    wl = W.mixture_workload(D=16, K=12, Kt=4, seed=3)
    w, mu, cov, df = wl["prop"]
    wt, mut, covt, _ = wl["target"]
    prop = pmcg.MixMvdens.from_arrays(w, mu, cov=cov, df=df).cholesky()
    target = pmcg.MixMvdens.from_arrays(wt, mut, cov=covt, df=-1).cholesky()
    post = pmcg.Posterior(16).add_mix(target)
    prev = pmcg.set_tensor_cores(True)
    try:
        graph = pmcg.Run(prop, post, 30000, precision=pmcg.MIXED, seed=5)
        direct = pmcg.Run(prop, post, 30000, precision=pmcg.MIXED, seed=5)
        direct.set_timing(True, stages=True)
        for on in (True, False, True):
            pmcg.set_tensor_cores(on)
            sg, sd = graph.iterate(1.0), direct.iterate(1.0)
            assert sg["ln_evidence"] == sd["ln_evidence"]
            np.testing.assert_array_equal(graph.sample().weights, direct.sample().weights)
        graph.free()
        direct.free()
    finally:
        pmcg.set_tensor_cores(prev)
