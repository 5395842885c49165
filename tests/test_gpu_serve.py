"""Serving loop with continuous batching: a job's result is the same alone and in
a mix of jobs that arrive while it runs; failures stay with their job;
admission respects the device-memory budget; waits are bounded."""
import threading
import time

import numpy as np
import pytest

from test_gpu_batch import make_run

pytestmark = pytest.mark.gpu

MIX = [("mix", 3, 2, 4000, 11), ("mix", 17, 9, 30000, 12), ("sn", 6, 4, 8000, 740), ("mix", 9, 5, 15000, 13),
       ("tpl", 3, 3, 6000, 91), ("mix", 12, 14, 25000, 14), ("mix", 20, 6, 12000, 15), ("dead", 2, 1, 500, 9),
       ("mix", 5, 1, 2000, 16), ("mix", 31, 4, 9000, 17)]
PROBE = ("mix", 8, 6, 20000, 123)


def _job(P, spec, keep):
    prop, post, box = make_run(P, *spec)
    keep.append((prop, post, box))
    return prop, post, box


def test_job_result_same_alone_and_in_the_mix(pmcg):
    P = pmcg
    keep = []
    prop, post, box = _job(P, PROBE, keep)
    s1 = P.Server()
    j = s1.submit(prop, post, PROBE[3], 6, PROBE[4], box=box, tempering=P.TEMPERING_LOG, t_min=0.05)
    alone, prop_alone = s1.wait(j, timeout=120, want_proposal=True)
    s1.free()
    assert alone["finished"] and alone["status"] == 0 and alone["iterations"] == 6

    s2 = P.Server(autotune=False)
    ids = {}
    jobs = [_job(P, spec, keep) for spec in MIX]

    def feeder():
        rng = np.random.default_rng(0)
        for i, (spec, (pp, po, bx)) in enumerate(zip(MIX, jobs)):
            ids[i] = s2.submit(pp, po, spec[3], 3 + i % 5, spec[4], box=bx)
            time.sleep(float(rng.uniform(0.0, 0.01)))
            if i == 4:  # the probe arrives while earlier jobs are on the GPU
                ids["probe"] = s2.submit(prop, post, PROBE[3], 6, PROBE[4], box=box, tempering=P.TEMPERING_LOG,
                                         t_min=0.05)

    t = threading.Thread(target=feeder)
    t.start()
    t.join()
    mixed, prop_mixed = s2.wait(ids["probe"], timeout=120, want_proposal=True)
    results = {i: s2.wait(ids[i], timeout=120) for i in range(len(MIX))}
    info = s2.info()
    s2.free()
    assert info["peak_resident"] > 1, info
    for key in ("status", "iterations", "ln_evidence", "perplexity", "ess", "enc"):
        assert mixed[key] == alone[key], (key, mixed[key], alone[key])
    for a, b in zip(prop_alone.arrays(), prop_mixed.arrays()):
        assert np.array_equal(a, b)
    for i, spec in enumerate(MIX):
        if spec[0] == "dead":
            assert results[i]["status"] == -9011
        else:
            assert results[i]["status"] == 0 and results[i]["iterations"] == 3 + i % 5, (spec, results[i])


def test_admission_respects_the_memory_budget(pmcg):
    P = pmcg
    keep = []
    specs = [("mix", 10, 5, 40000, 20 + i) for i in range(6)]
    jobs = [_job(P, s, keep) for s in specs]
    # budget for about two of these jobs at once
    probe = P.Server()
    jid = probe.submit(jobs[0][0], jobs[0][1], 40000, 1, 1)
    probe.wait(jid, timeout=60)
    one = probe.info()["peak_bytes"]
    probe.free()
    s = P.Server(hbm_budget_bytes=int(2.5 * one))
    ids = [s.submit(pp, po, sp[3], 4, sp[4]) for sp, (pp, po, bx) in zip(specs, jobs)]
    res = [s.wait(i, timeout=120) for i in ids]
    info = s.info()
    s.free()
    assert all(r["status"] == 0 for r in res)
    assert info["peak_resident"] <= 2 and info["peak_bytes"] <= info["budget_bytes"], info


def test_wait_is_bounded(pmcg):
    P = pmcg
    keep = []
    prop, post, box = _job(P, ("mix", 16, 8, 400000, 31), keep)
    s = P.Server()
    jid = s.submit(prop, post, 400000, 40, 31)
    with pytest.raises(P.PmcgError) as e:
        s.wait(jid, timeout=0.001)
    assert e.value.code == -9009
    s.free()  # stops after the current epoch


def test_large_job_alone_beside_the_batch(pmcg):
    """A job of at least alone_min_samples samples iterates with its own graph on
    its own stream, beside the batch of the smaller jobs: its result is the same
    as when served alone, and the small jobs' results are the same as when the
    large job is batched with them (SIZE_MAX: every job batched)."""
    P = pmcg
    keep = []
    big = ("mix", 10, 6, 70000, 321)
    prop, post, box = _job(P, big, keep)
    s1 = P.Server()
    j = s1.submit(prop, post, big[3], 4, big[4], box=box)
    alone, prop_alone = s1.wait(j, timeout=120, want_proposal=True)
    s1.free()
    assert alone["status"] == 0 and alone["iterations"] == 4
    small = [_job(P, spec, keep) for spec in MIX[:4]]
    res = {}
    for name, opts in (("split", {}), ("batched", {"alone_min_samples": (1 << 64) - 1})):
        s = P.Server(**opts)
        ids = [s.submit(pp, po, spec[3], 3, spec[4], box=bx) for spec, (pp, po, bx) in zip(MIX[:4], small)]
        jb = s.submit(prop, post, big[3], 4, big[4], box=box)
        res[name] = ([s.wait(i, timeout=120) for i in ids], s.wait(jb, timeout=120, want_proposal=True))
        s.free()
    (small_split, (big_split, prop_split)) = res["split"]
    (small_batched, _) = res["batched"]
    for key in ("status", "iterations", "ln_evidence", "perplexity", "ess", "enc"):
        assert big_split[key] == alone[key], (key, big_split[key], alone[key])
        for a, b in zip(small_split, small_batched):
            assert a[key] == b[key], (key, a, b)
    for a, b in zip(prop_alone.arrays(), prop_split.arrays()):
        assert np.array_equal(a, b)


def test_job_the_batch_does_not_take_runs_alone(pmcg):
    """A job with D > 32 (beyond the batch's limit) is served alone beside the
    batch of the others: it completes with the result of the same run iterated
    alone, and the batched jobs are unaffected."""
    P = pmcg
    keep = []
    wide = ("mix", 40, 3, 6000, 77)          # D = 40: the batch takes D <= 32
    prop, post, box = _job(P, wide, keep)
    run = P.Run(prop, post, wide[3], precision=P.MIXED, seed=wide[4], box=box)
    ref = [run.iterate(P.get_tempering_beta(P.TEMPERING_NONE, it, 1.0, 3)) for it in range(3)]
    ref_prop = run.proposal().arrays()
    run.free()
    small = [_job(P, spec, keep) for spec in MIX[:3]]
    s = P.Server()
    ids = [s.submit(pp, po, spec[3], 3, spec[4], box=bx) for spec, (pp, po, bx) in zip(MIX[:3], small)]
    jw = s.submit(prop, post, wide[3], 3, wide[4], box=box)
    res = [s.wait(i, timeout=120) for i in ids]
    rw, pw = s.wait(jw, timeout=120, want_proposal=True)
    s.free()
    assert all(r["status"] == 0 for r in res)
    assert rw["status"] == 0 and rw["iterations"] == 3
    assert rw["ln_evidence"] == ref[-1]["ln_evidence"] and rw["ess"] == ref[-1]["ess"]
    for a, b in zip(pw.arrays(), ref_prop):
        assert np.array_equal(a, b)


def test_job_with_two_likelihoods_runs_alone(pmcg):
    """A posterior with two likelihoods (two Gaussian-mixture targets; the batch
    takes one) is served beside the batch and gives the run alone's result."""
    P = pmcg
    keep = []
    spec = ("mix", 5, 3, 7000, 55)
    prop, post1, box = _job(P, spec, keep)
    from cosmopmc_gb300 import workloads as W
    wl = W.mixture_workload(D=5, K=2, Kt=2, nu=-1, seed=56, prop_hi=1.0)
    wt, mut, covt, _ = wl["target"]
    post = P.Posterior(5)
    for ww, mm, cc in ((wl["prop"][0], wl["prop"][1], wl["prop"][2]), (wt, mut, covt)):
        post.add_mix(P.MixMvdens.from_arrays(ww, mm, cov=cc, df=-1).cholesky())
    keep.append(post)
    run = P.Run(prop, post, spec[3], precision=P.MIXED, seed=spec[4])
    ref = [run.iterate(1.0) for _ in range(3)]
    ref_prop = run.proposal().arrays()
    run.free()
    s = P.Server()
    ids = [s.submit(pp, po, sp[3], 3, sp[4], box=bx) for sp, (pp, po, bx) in zip(MIX[:2], [_job(P, x, keep) for x in MIX[:2]])]
    j = s.submit(prop, post, spec[3], 3, spec[4])
    res = [s.wait(i, timeout=120) for i in ids]
    rj, pj = s.wait(j, timeout=120, want_proposal=True)
    s.free()
    assert all(r["status"] == 0 for r in res)
    assert rj["status"] == 0 and rj["ln_evidence"] == ref[-1]["ln_evidence"]
    for a, b in zip(pj.arrays(), ref_prop):
        assert np.array_equal(a, b)
