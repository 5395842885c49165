"""Dead-component revival (sdead_comp revive: update_and_deal_with_dead,
exec/cosmo_pmc.c:252-275, revive_comp :205-236) on device-resident runs,
batches and served jobs, against the oracle's restatement and against the same
runs alone.

Problem: D=2, prior box [-5, 5]^2, target N(0, I); the proposal has a third
component at (4, 4) with weight 0.02 that the first update buries (its weight
falls below 1/N); revival copies the heaviest component there with a shifted
mean. The revival's draws come from the run's stream, so the oracle reproduces
them exactly: proposals agree to 1e-9 (weights) and 1e-8 standard deviations."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BMIN, BMAX = np.array([-5.0, -5.0]), np.array([5.0, 5.0])


def _problem(pmcg):
    target = pmcg.MixMvdens.from_arrays([1.0], [[0.0, 0.0]], cov=[np.eye(2)], df=-1).cholesky()
    post = pmcg.Posterior(2, BMIN, BMAX).add_mix(target)
    w = np.array([0.49, 0.49, 0.02])
    mu = np.array([[-0.5, 0.0], [0.5, 0.2], [4.0, 4.0]])
    cov = np.array([np.eye(2) * 1.5, np.eye(2) * 1.2, np.eye(2) * 0.01])
    prop = pmcg.MixMvdens.from_arrays(w, mu, cov=cov, df=-1).cholesky()
    return target, post, prop


def test_run_revive_matches_oracle(pmcg, oracle):
    target, post, prop = _problem(pmcg)
    N, seed = 4000, 77
    run = pmcg.Run(prop, post, N, precision=pmcg.FP64, seed=seed, box=pmcg.Parabox(BMIN, BMAX))
    run.set_dead_comp(pmcg.DEAD_REVIVE, 0.1)
    w, mu, L = prop.arrays()
    om = oracle.Mix(w, mu, L=L)
    tw, tmu, tL = target.arrays()
    ot = oracle.Mix(tw, tmu, L=tL)
    logpr = -np.sum(np.log(BMAX - BMIN))

    def lpf(X, flg):
        return oracle.mix_logpdf(ot, X) + logpr, np.ones(len(X), np.int16)

    nrevive, revived = 1, 0
    for it in range(3):
        st = run.iterate(1.0)
        new, so = oracle.iterate_posterior(om, lpf, N, seed, it, 1.0, BMIN, BMAX)
        assert so["status"] == 0
        nrevive *= 2
        revived += so["ndead"]
        if so["ndead"]:
            new = oracle.revive(new, BMIN, BMAX, 0.1, nrevive, seed, it)
        assert st["ndead"] == so["ndead"], (it, st, so)
        gw, gmu, gL = run.proposal().arrays()
        np.testing.assert_allclose(gw, new.w, rtol=1e-9, atol=1e-15)
        assert np.all(gw > 0)   # every component alive after the revival
        gcov = np.einsum("kij,klj->kil", gL, gL)
        for k in range(3):
            sd = np.sqrt(np.diag(new.cov[k]))
            assert np.max(np.abs(gmu[k] - new.mu[k]) / sd) < 1e-8, (it, k)
            assert np.max(np.abs(gcov[k] - new.cov[k]) / np.outer(sd, sd)) < 1e-8, (it, k)
        om = oracle.Mix(gw, gmu, L=gL)
    assert revived >= 1
    run.free()


def test_revive_needs_a_box(pmcg):
    target, post, prop = _problem(pmcg)
    run = pmcg.Run(prop, post, 1000, precision=pmcg.FP64, seed=1)
    with pytest.raises(pmcg.PmcgError) as e:
        run.set_dead_comp(pmcg.DEAD_REVIVE, 0.1)
    assert e.value.code == -9008
    run.free()


def test_batch_and_server_revive_like_runs_alone(pmcg):
    """Mixed precision with the CUDA-core log-density (the batch's kernel): a batch
    and a served job revive exactly as the run alone does."""
    prev = pmcg.set_tensor_cores(False)
    try:
        target, post, prop = _problem(pmcg)
        box = pmcg.Parabox(BMIN, BMAX)
        N, seed = 6000, 5
        alone = pmcg.Run(prop, post, N, precision=pmcg.MIXED, seed=seed, box=box)
        alone.set_dead_comp(pmcg.DEAD_REVIVE, 0.1)
        inb = pmcg.Run(prop, post, N, precision=pmcg.MIXED, seed=seed, box=box)
        inb.set_dead_comp(pmcg.DEAD_REVIVE, 0.1)
        batch = pmcg.Batch([inb])
        for it in range(3):
            sa = alone.iterate(1.0)
            sb = batch.iterate([1.0])[0]
            assert sa == sb, (it, sa, sb)
            wa, ma, La = alone.proposal().arrays()
            wb, mb, Lb = inb.proposal().arrays()
            assert np.array_equal(wa, wb) and np.array_equal(ma, mb) and np.array_equal(La, Lb)
        batch.free()
        srv = pmcg.Server(dead_comp=pmcg.DEAD_REVIVE, fshift=0.1)
        jid = srv.submit(prop, post, N, 3, seed, box=box)
        res, fin = srv.wait(jid, timeout=120, want_proposal=True)
        assert res["status"] == 0, res
        wf, mf, Lf = fin.arrays()
        assert np.array_equal(wf, wa) and np.array_equal(mf, ma) and np.array_equal(Lf, La)
        srv.free()
    finally:
        pmcg.set_tensor_cores(prev)
