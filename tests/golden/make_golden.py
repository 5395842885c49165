"""Generate the golden fixtures that pin the FP64 oracle (tests/golden/golden.npz).

Every expected value here comes from an implementation independent of
oracle/pmc_oracle.c: scipy.stats densities, scipy.integrate.quad distances,
numpy linear algebra, scipy.special.logsumexp, a direct numpy restatement of
the Rao-Blackwellised EM update (Cappe et al. 2008), the published Philox4x32-10
known-answer vectors (Salmon et al. 2011), and the two tempering demo targets
of the reference (Demo/tempering/*/config_pmc, read as text when the reference
tree is present; their analytic evidence is 1, Demo/tempering/README.md:14-21).

Run:  python tests/golden/make_golden.py --reference <CosmoPMC source tree>
      (needs numpy + scipy; writes golden.npz; without --reference, or with
      the PMCG_REFERENCE environment variable unset, the demo targets are left
      out)
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np
from scipy import integrate, special, stats

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from cosmopmc_gb300 import workloads as W  # noqa: E402

C_KMS = 299792.458


def mixture(rng, K, D):
    w = rng.dirichlet(np.ones(K))
    mu = rng.normal(0, 1, (K, D))
    A = rng.normal(0, 1, (K, D, D))
    cov = np.einsum("kij,klj->kil", A, A) + np.eye(D)[None] * 0.5
    return w, mu, cov


def lum_dist_quad(om, ode, w0, h, z):
    ok = 1 - om - ode
    f = lambda t: 1.0 / np.sqrt(om * (1 + t) ** 3 + ok * (1 + t) ** 2 + ode * (1 + t) ** (3 * (1 + w0)))
    I = integrate.quad(f, 0, z, epsabs=0, epsrel=1e-13, limit=200)[0]
    if abs(ok) < 1e-10:
        dm = I
    elif ok > 0:
        dm = np.sinh(np.sqrt(ok) * I) / np.sqrt(ok)
    else:
        dm = np.sin(np.sqrt(-ok) * I) / np.sqrt(-ok)
    return (1 + z) * C_KMS / (100 * h) * dm


def sn_loglike_ref(sn, p):
    om, ode, w0, M, al, be = p
    ll_terms = []
    A = B = Cc = chi2 = sl = 0.0
    for i in range(len(sn["z"])):
        z = sn["z"][i]
        mu_th = 5 * np.log10(lum_dist_quad(om, ode, w0, sn["h"], z)) + 25
        W6 = sn["cov6"][i]
        spv = (5 / np.log(10)) * sn["v_pec"] / (C_KMS * z)
        s2 = (W6[0] + al * al * W6[1] + be * be * W6[2] + 2 * al * W6[3] - 2 * be * W6[4] - 2 * al * be * W6[5]
              + sn["sig_int"] ** 2 + spv ** 2)
        d = sn["mB"][i] + al * sn["x1"][i] - be * sn["c"][i] - mu_th
        if sn["chi2mode"] == 0:
            chi2 += (d - M) ** 2 / s2
        else:
            A += d * d / s2
            B += d / s2
            Cc += 1 / s2
        sl += np.log(s2)
    if sn["chi2mode"] != 0:
        chi2 = A - B * B / Cc + np.log(Cc / (2 * np.pi))
    del ll_terms
    return -0.5 * chi2 - (0.5 * sl if sn["add_logdet"] else 0.0)


def em_ref(w, mu, cov, df, X, wbar, flg, idx, N):
    """Rao-Blackwellised EM (Cappe et al. 2008) in plain numpy."""
    K, D = mu.shape
    dens = np.empty((K, len(X)))
    Qs = np.empty((K, len(X)))
    for k in range(K):
        Lk = np.linalg.cholesky(cov[k])
        y = np.linalg.solve(Lk, (X - mu[k]).T)
        Qs[k] = np.sum(y * y, axis=0)
        if df > 0:
            dens[k] = stats.multivariate_t(mu[k], cov[k], df=df).logpdf(X)
        else:
            dens[k] = stats.multivariate_normal(mu[k], cov[k]).logpdf(X)
    lt = np.log(w)[:, None] + dens
    logq = special.logsumexp(lt, axis=0)
    rho = np.exp(lt - logq[None, :])
    v = wbar[None, :] * rho * flg[None, :]
    tau = (df + D) / (df + Qs) if df > 0 else np.ones_like(Qs)
    nw = np.zeros(K)
    nmu = mu.copy()
    ncov = cov.copy()
    cnt = np.bincount(idx, minlength=K)
    dead = np.zeros(K, int)
    for k in range(K):
        s0 = v[k].sum()
        vt = v[k] * tau[k]
        st = vt.sum()
        if cnt[k] < 20 or s0 < 1.0 / N or st <= 0:
            dead[k] = 1
            continue
        m1 = (vt[:, None] * X).sum(0) / st
        dx = X - m1
        S = (vt[:, None, None] * dx[:, :, None] * dx[:, None, :]).sum(0) / s0
        nw[k] = s0
        nmu[k] = m1
        ncov[k] = S
    nw /= nw.sum()
    return nw, nmu, ncov, dead, logq, lt, Qs


def demo_targets(reference):
    """Targets of the reference's two tempering demos, read as text from
    <reference>/Demo/tempering/*/config_pmc; None without a reference tree."""
    if not reference:
        return None
    out = {}
    for name in ("1_mvnorm_2D_temp_none", "2_mixmvnorm_2D_temp_none"):
        path = os.path.join(reference, "Demo", "tempering", name, "config_pmc")
        if not os.path.exists(path):
            return None
        vals = {}
        means, stds = [], []
        for line in open(path):
            t = line.split("#")[0].split()
            if not t:
                continue
            if t[0] == "mean":
                means.append([float(v) for v in t[1:]])
            elif t[0] == "std":
                stds.append([float(v) for v in t[1:]])
            elif t[0] in ("min", "max", "nsamples", "niter", "ncomp", "fsfinal"):
                vals.setdefault(t[0], [float(v) for v in t[1:]])
        out[name] = dict(mean=np.array(means), cov=np.array(stds).reshape(len(stds), 2, 2), **vals)
    return out


def main(argv=None):
    import argparse
    ap = argparse.ArgumentParser(description="Write tests/golden/golden.npz and golden.json.")
    ap.add_argument("--reference", default=os.environ.get("PMCG_REFERENCE"),
                    help="CosmoPMC source tree (for the Demo/tempering targets)")
    args = ap.parse_args(argv)
    rng = np.random.default_rng(20261203)
    g = {}
    meta = {}
    # Philox4x32-10 known-answer vectors (Salmon et al. 2011, Random123 kat_vectors)
    g["philox_ctr"] = np.array([[0, 0, 0, 0], [0xFFFFFFFF] * 4, [0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344]],
                               dtype=np.uint64)
    g["philox_key"] = np.array([[0, 0], [0xFFFFFFFF] * 2, [0xA4093822, 0x299F31D0]], dtype=np.uint64)
    g["philox_out"] = np.array([[0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8],
                                [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD],
                                [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]], dtype=np.uint64)
    # mixture log-pdfs (scipy)
    for tag, df in (("gauss", -1), ("t", 3)):
        w, mu, cov = mixture(rng, 4, 5)
        X = rng.normal(0, 2, (64, 5))
        if df > 0:
            logq = special.logsumexp([np.log(w[k]) + stats.multivariate_t(mu[k], cov[k], df=df).logpdf(X)
                                      for k in range(4)], axis=0)
        else:
            logq = special.logsumexp([np.log(w[k]) + stats.multivariate_normal(mu[k], cov[k]).logpdf(X)
                                      for k in range(4)], axis=0)
        g[f"mix_{tag}_w"], g[f"mix_{tag}_mu"], g[f"mix_{tag}_cov"] = w, mu, cov
        g[f"mix_{tag}_X"], g[f"mix_{tag}_logq"] = X, logq
        meta[f"mix_{tag}_df"] = df
    # luminosity distances (scipy quad)
    cosmo = np.array([[0.3, 0.7, -1.0, 0.7], [0.3, 0.6, -0.9, 0.7], [0.25, 0.85, -1.2, 0.7], [1.0, 0.0, -1.0, 0.7]])
    zs = np.array([0.01, 0.3, 0.9, 1.4])
    g["dl_cosmo"], g["dl_z"] = cosmo, zs
    g["dl_val"] = np.array([[lum_dist_quad(*c, z) for z in zs] for c in cosmo])
    # SN log-likelihoods (independent numpy + quad restatement)
    for tag, mode, logdet in (("full", 0, 0), ("marg", 1, 0), ("logdet", 0, 1)):
        sn = W.sn_data(nsn=40, seed=11, chi2mode=mode, quad_nodes=8)
        if logdet:
            sn["cov6"] = np.tile([0.0225, 0.01, 0.001, 0.0005, -0.0002, 0.0001], (40, 1))
            sn["add_logdet"] = 1
            sn["sig_int"] = 0.1
            sn["v_pec"] = 300.0
        P = np.array([[0.3, 0.7, -1.0, -19.1, 0.14, 3.1], [0.25, 0.6, -0.8, -19.0, 0.2, 2.5],
                      [0.4, 0.9, -1.3, -19.3, 0.1, 3.5]])
        g[f"sn_{tag}_P"] = P
        g[f"sn_{tag}_ll"] = np.array([sn_loglike_ref(sn, p) for p in P])
        for k in ("z", "mB", "x1", "c", "cov6"):
            g[f"sn_{tag}_{k}"] = sn[k]
        meta[f"sn_{tag}"] = {k: sn[k] for k in sn if not isinstance(sn[k], np.ndarray)}
    # template likelihood (numpy solve)
    D, M = 3, 64
    P_ = W.tpl_nphi(D)
    A = rng.normal(0, 1 / np.sqrt(P_), (M, P_))
    idx = np.arange(M)
    Cm = 0.9 ** np.abs(idx[:, None] - idx[None, :])
    dobs = A @ W.tpl_phi(np.full(D, 0.1))[0] + np.linalg.cholesky(Cm) @ rng.standard_normal(M)
    T = rng.uniform(-1, 1, (20, D))
    R = dobs[None, :] - W.tpl_phi(T) @ A.T
    g["tpl_A"], g["tpl_C"], g["tpl_dobs"], g["tpl_T"] = A, Cm, dobs, T
    g["tpl_ll"] = -0.5 * np.einsum("nm,nm->n", R, np.linalg.solve(Cm, R.T).T)
    # weights / evidence / perplexity (logsumexp)
    N = 1000
    lp = rng.normal(-5, 3, N)
    lq = rng.normal(-4, 2, N)
    flg = (rng.uniform(size=N) > 0.1).astype(np.int16)
    beta = 0.7
    lw = np.where(flg == 1, beta * lp - lq, -np.inf)
    ls = special.logsumexp(lw[flg == 1])
    wb = np.where(flg == 1, np.exp(lw - ls), 0.0)
    H = -np.sum(wb[wb > 0] * np.log(wb[wb > 0]))
    g["wt_lp"], g["wt_lq"], g["wt_flg"] = lp, lq, flg
    g["wt_expect"] = np.array([ls, np.max(lw[flg == 1]), np.exp(H) / N, 1 / np.sum(wb ** 2), ls - np.log(N)])
    meta["wt_beta"] = beta
    # EM update (numpy restatement), Gaussian and Student-t, one dead component
    for tag, df in (("gauss", -1), ("t", 4)):
        K, D, N = 3, 3, 3000
        w = np.array([0.5, 0.495, 0.005])
        mu = rng.normal(0, 1, (K, D))
        Aa = rng.normal(0, 0.5, (K, D, D))
        cov = np.einsum("kij,klj->kil", Aa, Aa) + np.eye(D)[None] * 0.3
        idx = rng.choice(K, size=N, p=w).astype(np.int32)
        X = np.array([rng.multivariate_normal(mu[k], cov[k]) for k in idx])
        flg = np.ones(N, np.int16)
        flg[:7] = 0
        lw = -0.5 * np.sum((X - 0.3) ** 2, axis=1) / 2.0
        lw[flg == 0] = -np.inf
        wb = np.exp(lw - special.logsumexp(lw[flg == 1]))
        nw, nmu, ncov, dead, logq, lt, Qs = em_ref(w, mu, cov, df, X, wb, flg, idx, N)
        for k, v in dict(w=w, mu=mu, cov=cov, idx=idx, X=X, flg=flg, wbar=wb, nw=nw, nmu=nmu, ncov=ncov,
                         dead=dead).items():
            g[f"em_{tag}_{k}"] = v
        meta[f"em_{tag}_df"] = df
    # tempering schedule of exec/cosmo_pmc.c:464-495
    bet = []
    for kind in (0, 1, 2):
        for it in range(6):
            if kind == 0 or it == 5:
                b = 1.0
            elif kind == 1:
                b = it / (6 - 2.0) * (1 - 0.05) + 0.05
            else:
                b = np.exp(it / (6 - 2.0) * (-np.log(0.05)) + np.log(0.05))
            bet.append([kind, it, b])
    g["tempering"] = np.array(bet)
    demos = demo_targets(args.reference)
    if demos is not None:
        m1 = demos["1_mvnorm_2D_temp_none"]
        m2 = demos["2_mixmvnorm_2D_temp_none"]
        g["demo1_mean"], g["demo1_cov"] = m1["mean"], m1["cov"]
        g["demo2_mean"], g["demo2_cov"] = m2["mean"], m2["cov"]
        meta["demo_box"] = [m1["min"], m1["max"]]
        meta["demo_analytic_evidence"] = 1.0
        meta["demo2_published_evidence_both_modes"] = 0.998802
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **g)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True, default=float)
    print("wrote", len(g), "arrays")


if __name__ == "__main__":
    main()
