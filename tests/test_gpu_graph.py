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


def test_async_iterations_equal_synchronous(pmcg):
    """pmcg_run_iterate_async / _wait: iterations of two runs started together and
    waited for in turn equal the same runs iterated synchronously, in single
    precision (a replayed graph in flight) and in FP64 (direct launches)."""
    P = pmcg
    wl = W.mixture_workload(D=8, K=4, Kt=2, nu=-1, seed=5, prop_hi=2.0)
    w, mu, cov, df = wl["prop"]
    wt, mut, covt, _ = wl["target"]
    prop = P.MixMvdens.from_arrays(w, mu, cov=cov, df=df).cholesky()
    target = P.MixMvdens.from_arrays(wt, mut, cov=covt, df=-1).cholesky()
    post = P.Posterior(8).add_mix(target)
    for prec in (P.MIXED, P.FP64):
        a, b = (P.Run(prop, post, 30000, precision=prec, seed=s) for s in (1, 2))
        a2, b2 = (P.Run(prop, post, 30000, precision=prec, seed=s) for s in (1, 2))
        for it in range(3):
            a.iterate_async(1.0)
            b.iterate_async(0.5)
            sa, sb = a.iterate_wait(), b.iterate_wait()
            assert sa == a2.iterate(1.0) and sb == b2.iterate(0.5), (prec, it)
        for x, y in ((a, a2), (b, b2)):
            for u, v in zip(x.proposal().arrays(), y.proposal().arrays()):
                assert np.array_equal(u, v)
        with pytest.raises(P.PmcgError):
            a.iterate_wait()            # nothing in flight
        a.iterate_async(1.0)
        for call in (lambda: a.iterate(1.0), lambda: a.iterate_async(1.0), a.proposal):
            with pytest.raises(P.PmcgError) as e:
                call()                  # one iteration in flight: other calls are refused
            assert e.value.code == -9008
        a.iterate_wait()
        a2.iterate(1.0)
        for u, v in zip(a.proposal().arrays(), a2.proposal().arrays()):
            assert np.array_equal(u, v)
        for r in (a, b, a2, b2):
            r.free()


def test_tensor_core_setting_per_run(pmcg):
    """pmcg_run_set_tensor_cores: two runs in one process with different
    settings; each equals a run that follows the process default set to its
    own setting (and None returns a run to the default)."""
    P = pmcg
    wl = W.mixture_workload(D=16, K=8, Kt=3, nu=4, seed=8, prop_hi=2.0)
    w, mu, cov, df = wl["prop"]
    wt, mut, covt, _ = wl["target"]
    prop = P.MixMvdens.from_arrays(w, mu, cov=cov, df=df).cholesky()
    target = P.MixMvdens.from_arrays(wt, mut, cov=covt, df=-1).cholesky()
    post = P.Posterior(16).add_mix(target)
    prev = P.set_tensor_cores(False)
    try:
        on, off = (P.Run(prop, post, 20000, precision=P.MIXED, seed=3) for _ in range(2))
        assert on.set_tensor_cores(True) is None
        off.set_tensor_cores(False)
        P.set_tensor_cores(True)              # the default no longer decides for these two
        s_on = [on.iterate(1.0) for _ in range(2)]
        s_off = [off.iterate(1.0) for _ in range(2)]
        ref = {}
        for flag in (True, False):
            P.set_tensor_cores(flag)
            r = P.Run(prop, post, 20000, precision=P.MIXED, seed=3)
            ref[flag] = ([r.iterate(1.0) for _ in range(2)], r.proposal().arrays())
            r.free()
        assert s_on == ref[True][0] and s_off == ref[False][0]
        assert s_on != s_off                  # the two kernels round differently
        for x, y in zip(on.proposal().arrays(), ref[True][1]):
            assert np.array_equal(x, y)
        assert off.set_tensor_cores(None) == 0
        for r in (on, off):
            r.free()
    finally:
        P.set_tensor_cores(prev)
