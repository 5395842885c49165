"""Batched runs (one persistent cooperative launch per iteration) against the
same runs iterated alone: statistics and proposals must be bit-identical,
and a failing run must not disturb the others."""
import numpy as np
import pytest

from cosmopmc_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _cuda_core_log_density(pmcg):
    """Batched runs evaluate log q on the CUDA cores; runs alone match them bit
    for bit with the same kernel."""
    prev = pmcg.set_tensor_cores(False)
    yield
    pmcg.set_tensor_cores(prev)


def make_run(P, kind, D, K, N, seed):
    if kind == "mix":
        wl = W.mixture_workload(D=D, K=K, Kt=max(1, K // 3), nu=4 if seed % 2 else -1, seed=seed, prop_hi=2.0)
        w, mu, cov, df = wl["prop"]
        wt, mut, covt, _ = wl["target"]
        prop = P.MixMvdens.from_arrays(w, mu, cov=cov, df=df).cholesky()
        target = P.MixMvdens.from_arrays(wt, mut, cov=covt, df=-1).cholesky()
        post = P.Posterior(D).add_mix(target)
        return prop, post, None
    if kind == "sn":
        wl = W.sn_workload(K=K, seed=seed, init="fisher")
        w, mu, cov, df = wl["prop"]
        prop = P.MixMvdens.from_arrays(w, mu, cov=cov, df=df).cholesky()
        post = P.Posterior(6, wl["bmin"], wl["bmax"]).add_snia(wl["sn"])
        return prop, post, P.Parabox(wl["bmin"], wl["bmax"])
    if kind == "tpl":
        wl = W.template_workload(D=D, M=64, K=K, seed=seed)
        w, mu, cov, df = wl["prop"]
        prop = P.MixMvdens.from_arrays(w, mu, cov=cov, df=df).cholesky()
        post = P.Posterior(D, wl["bmin"], wl["bmax"]).add_template(wl["A"], wl["C"], wl["dobs"])
        return prop, post, P.Parabox(wl["bmin"], wl["bmax"])
    if kind == "snprior":  # SN parameters + Gaussian nuisance parameters (a subset prior)
        wl = W.sn_workload(K=K, seed=seed, init="fisher")
        w, mu, cov, df = wl["prop"]
        nx = D - 6
        mu = np.concatenate([mu, np.zeros((K, nx))], axis=1)
        cov2 = np.zeros((K, D, D))
        cov2[:, :6, :6] = cov
        cov2[:, 6:, 6:] = 0.1 * np.eye(nx)
        prop = P.MixMvdens.from_arrays(w, mu, cov=cov2, df=df).cholesky()
        bmin = np.r_[wl["bmin"], -np.ones(nx)]
        bmax = np.r_[wl["bmax"], np.ones(nx)]
        post = P.Posterior(D, bmin, bmax).add_snia(wl["sn"])
        post.add_prior(np.zeros(nx), 0.0625 * np.eye(nx), indprior=np.r_[np.zeros(6, int), np.ones(nx, int)])
        return prop, post, P.Parabox(bmin, bmax)
    if kind == "buried":  # 15 draws of one component: the update buries it (fewer than 20 draws)
        return make_run(P, "mix", D, K, N, seed)
    if kind == "dead":  # every draw falls outside the box
        prop = P.MixMvdens.from_arrays([1.0], [[10.0, 10.0]], cov=[np.eye(2) * 0.01], df=-1).cholesky()
        target = P.MixMvdens.from_arrays([1.0], [[0.0, 0.0]], cov=[np.eye(2)], df=-1).cholesky()
        post = P.Posterior(2, [-1, -1], [1, 1]).add_mix(target)
        return prop, post, P.Parabox([-1, -1], [1, 1])
    raise ValueError(kind)


SPECS = [("mix", 2, 1, 1000, 1), ("mix", 5, 3, 3001, 2), ("mix", 13, 7, 20000, 3), ("mix", 20, 12, 9000, 5),
         ("sn", 6, 5, 4000, 740), ("snprior", 9, 4, 3000, 741), ("tpl", 3, 4, 2500, 91), ("buried", 2, 1, 15, 11),
         ("dead", 2, 1, 777, 9)]


def test_batch_is_bit_identical_to_runs_alone(pmcg):
    P = pmcg
    keep, batch_runs, alone_runs = [], [], []
    for kind, D, K, N, seed in SPECS:
        prop, post, box = make_run(P, kind, D, K, N, seed)
        keep.append((prop, post, box))
        batch_runs.append(P.Run(prop, post, N, precision=P.MIXED, seed=seed, box=box))
        alone_runs.append(P.Run(prop, post, N, precision=P.MIXED, seed=seed, box=box))
    batch = P.Batch(batch_runs)
    cfg = batch.config()
    assert cfg["grid"] > 0
    betas = [1.0, 0.5, 1.0, 0.8, 1.0, 0.7, 1.0, 1.0, 1.0]
    for it in range(3):
        bst = batch.iterate(betas)
        for r, (spec, run) in enumerate(zip(SPECS, alone_runs)):
            if spec[0] == "dead":
                assert bst[r]["status"] == -9011
            if spec[0] == "buried":  # PMCG_ENEGWEIGHT, then nothing left to draw from
                assert bst[r]["status"] == (-9005 if it == 0 else -9011), (it, bst[r])
            if bst[r]["status"] != 0:  # the run alone fails with the same code
                with pytest.raises(P.PmcgError) as ei:
                    run.iterate(betas[r])
                assert ei.value.code == bst[r]["status"], (it, spec, ei.value)
                continue
            ast = run.iterate(betas[r])
            ast["status"] = 0
            assert bst[r] == ast, (it, spec, bst[r], ast)
            wb, mb, Lb = batch_runs[r].proposal().arrays()
            wa, ma, La = run.proposal().arrays()
            assert np.array_equal(wb, wa) and np.array_equal(mb, ma) and np.array_equal(Lb, La), (it, spec)
        # the buried run: the same buried proposal in the batch and alone
        rb = SPECS.index(next(sp for sp in SPECS if sp[0] == "buried"))
        wb, mb, Lb = batch_runs[rb].proposal().arrays()
        wa, ma, La = alone_runs[rb].proposal().arrays()
        assert np.array_equal(wb, wa) and np.all(wb == 0.0) and np.array_equal(mb, ma), it
    # the failing run kept its proposal
    w, mu, L = batch_runs[-1].proposal().arrays()
    assert np.array_equal(mu, [[10.0, 10.0]])
    batch.free()


def test_batch_autotune_keeps_results(pmcg):
    P = pmcg
    keep, runs_a, runs_b = [], [], []
    for kind, D, K, N, seed in SPECS[:5]:
        prop, post, box = make_run(P, kind, D, K, N, seed)
        keep.append((prop, post, box))
        runs_a.append(P.Run(prop, post, N, precision=P.MIXED, seed=seed, box=box))
        runs_b.append(P.Run(prop, post, N, precision=P.MIXED, seed=seed, box=box))
    a = P.Batch(runs_a)
    b = P.Batch(runs_b)
    b.autotune()
    cfg = b.config()
    assert cfg["samples_per_thread"] in (1, 2) and cfg["blocks_per_sm"] >= 1
    for it in range(2):
        assert a.iterate() == b.iterate()
    assert b.last_ms() > 0.0


def test_batch_stage_timing_keeps_results(pmcg):
    """The profiling mode launches the stages one by one: same statistics and
    proposals as the single launch, and a per-stage time for every stage."""
    P = pmcg
    keep, runs_a, runs_b = [], [], []
    for kind, D, K, N, seed in SPECS[:6]:
        prop, post, box = make_run(P, kind, D, K, N, seed)
        keep.append((prop, post, box))
        runs_a.append(P.Run(prop, post, N, precision=P.MIXED, seed=seed, box=box))
        runs_b.append(P.Run(prop, post, N, precision=P.MIXED, seed=seed, box=box))
    a = P.Batch(runs_a)
    b = P.Batch(runs_b)
    assert b.stage_ms() is None
    b.set_stage_timing(True)
    for it in range(2):
        assert a.iterate() == b.iterate(), it
        sm = b.stage_ms()
        assert sm is not None and set(sm) == set(P.Batch.BATCH_STAGES)
        assert all(v >= 0.0 for v in sm.values()) and sum(sm.values()) <= b.last_ms() + 1e-3
    for ra, rb in zip(runs_a, runs_b):
        wa, ma, La = ra.proposal().arrays()
        wb, mb, Lb = rb.proposal().arrays()
        assert np.array_equal(wa, wb) and np.array_equal(ma, mb) and np.array_equal(La, Lb)
    b.set_stage_timing(False)
    a.iterate()
    b.iterate()
    assert b.stage_ms() is None
    a.free()
    b.free()


def test_batch_rebind_equals_fresh_batches(pmcg):
    """A batch rebound to another set of runs (some continuing, some new) gives
    what fresh batches of the same runs give, bit for bit, over the rebinding
    and the graph captured again after it."""
    P = pmcg
    specs = SPECS[:6]
    keep, xs, ys = [], [], []
    for kind, D, K, N, seed in specs:
        prop, post, box = make_run(P, kind, D, K, N, seed)
        keep.append((prop, post, box))
        xs.append(P.Run(prop, post, N, precision=P.MIXED, seed=seed, box=box))
        ys.append(P.Run(prop, post, N, precision=P.MIXED, seed=seed, box=box))
    b = P.Batch(xs[:3])
    f1 = P.Batch(ys[:3])
    assert b.iterate() == f1.iterate()
    b.rebind(xs[1:6])   # runs 1 and 2 continue, 3..5 join
    f2 = P.Batch(ys[1:6])
    for it in range(3):   # direct launch, then the graph captured and replayed
        assert b.iterate() == f2.iterate(), it
    for rx, ry in zip(xs[1:6], ys[1:6]):
        wa, ma, La = rx.proposal().arrays()
        wb, mb, Lb = ry.proposal().arrays()
        assert np.array_equal(wa, wb) and np.array_equal(ma, mb) and np.array_equal(La, Lb)
    b.rebind(xs[:1])    # fewer runs than before: the arrays are kept
    f3 = P.Batch(ys[:1])
    assert b.iterate() == f3.iterate()
    for x in (b, f1, f2, f3):
        x.free()


def test_run_alone_after_a_batch_uses_the_updated_proposal(pmcg):
    """A batch updates its runs' proposals without their tensor-core operand
    image; a run iterated alone afterwards with the tensor cores rebuilds it:
    its iteration equals that of a twin whose proposal was set again from the
    host (which rebuilds everything from the FP64 proposal)."""
    P = pmcg
    kind, D, K, N, seed = SPECS[3]          # a 20-dimensional mixture
    prop, post, box = make_run(P, kind, D, K, N, seed)
    a, b = (P.Run(prop, post, N, precision=P.MIXED, seed=seed, box=box) for _ in range(2))
    ba, bb = P.Batch([a]), P.Batch([b])
    for _ in range(2):
        assert ba.iterate() == bb.iterate()
    ba.free()
    bb.free()
    b.set_proposal(b.proposal())
    P.set_tensor_cores(True)
    sa, sb = a.iterate(1.0), b.iterate(1.0)
    assert sa == sb
    for u, v in zip(a.proposal().arrays(), b.proposal().arrays()):
        assert np.array_equal(u, v)
    a.free()
    b.free()


def test_batch_at_its_largest_shapes(pmcg):
    """Runs at the batch's limits (D = 32 with K = 64 Student-t components, and
    K = 256 components) batched with a small run: bit-identical to the same runs
    alone with the CUDA-core kernels."""
    P = pmcg
    specs = [("mix", 32, 64, 6000, 41), ("mix", 4, 256, 9000, 42), ("mix", 3, 2, 1500, 43)]
    keep, xs, ys = [], [], []
    for kind, D, K, N, seed in specs:
        prop, post, box = make_run(P, kind, D, K, N, seed)
        keep.append((prop, post, box))
        xs.append(P.Run(prop, post, N, precision=P.MIXED, seed=seed, box=box))
        ys.append(P.Run(prop, post, N, precision=P.MIXED, seed=seed, box=box))
    b = P.Batch(xs)
    for it in range(2):
        bst = b.iterate()
        for r, run in enumerate(ys):
            ast = run.iterate(1.0)
            ast["status"] = 0
            assert bst[r] == ast, (it, specs[r], bst[r], ast)
            for u, v in zip(xs[r].proposal().arrays(), run.proposal().arrays()):
                assert np.array_equal(u, v), (it, specs[r])
    b.free()
