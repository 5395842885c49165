"""Seeded synthetic workloads of the engine's benchmark configurations.

No external dataset is reproduced: every array is drawn from a seeded numpy
generator with the shapes and distributions of the named configuration.

* sn_workload:       SN Ia wCDM, 740 supernovae, D=6, K=10 Gaussian proposal.
* mixture_workload:  D=32, K=64 Student-t (nu=3) proposal with condition 1e6
                     covariances; target a different normalised 16-component
                     Gaussian mixture (so log Z = 0 with no prior box).
* template_workload: D=12, 91 quadratic monomials, 2048 data points, AR(1)
                     covariance (rho=0.9), K=16 proposal in the box [-1,1]^12.
"""
from __future__ import annotations

import numpy as np

C_KMS = 299792.458


def random_orthogonal(rng, D):
    """Q from the QR factorisation of a Gaussian matrix, diagonal of R made positive."""
    A = rng.standard_normal((D, D))
    Q, R = np.linalg.qr(A)
    return Q * np.sign(np.diag(R))[None, :]


def conditioned_covs(rng, K, D, lo_exp, hi_exp):
    ev = np.logspace(lo_exp, hi_exp, D)
    covs = np.empty((K, D, D))
    for k in range(K):
        Q = random_orthogonal(rng, D)
        covs[k] = (Q * ev[None, :]) @ Q.T
        covs[k] = 0.5 * (covs[k] + covs[k].T)
    return covs


def random_pos_proposal(rng, K, bmin, bmax, fmin=0.02, df=-1):
    """Initial proposal by the random-position rule of wrappers/src/param.c:656-683:
    per coordinate r ~ U(fmin*box/2, 0.5*box/2), variance r^4, mean at the box centre
    shifted by U(-1,1)*(box/2 - 2r) when that is positive; equal weights."""
    bmin, bmax = np.asarray(bmin, float), np.asarray(bmax, float)
    D = len(bmin)
    mu = np.empty((K, D))
    covs = np.zeros((K, D, D))
    for k in range(K):
        for i in range(D):
            box = bmax[i] - bmin[i]
            r = rng.uniform(fmin * box / 2.0, 0.5 * box / 2.0)
            covs[k, i, i] = r ** 4
            mu[k, i] = 0.5 * (bmin[i] + bmax[i])
            f = box / 2.0 - 2.0 * r
            if f > 0:
                mu[k, i] += rng.uniform(-1, 1) * f
    return np.full(K, 1.0 / K), mu, covs, df


# ----------------------------------------------------------------- SN Ia
def lum_dist_np(z, om, ode, w0, h, G=8, nsub=64):
    """D_L in Mpc by composite Gauss-Legendre (numpy; data synthesis only)."""
    xg, wg = np.polynomial.legendre.leggauss(G)
    ok = 1.0 - om - ode
    out = np.empty_like(z)
    for t, zz in enumerate(z):
        e = np.linspace(0.0, zz, nsub + 1)
        a, b = e[:-1], e[1:]
        hw, c = 0.5 * (b - a), 0.5 * (a + b)
        zn = c[:, None] + hw[:, None] * xg[None, :]
        an = 1.0 + zn
        f = 1.0 / np.sqrt(om * an ** 3 + ok * an ** 2 + ode * an ** (3 * (1 + w0)))
        I = np.sum(hw[:, None] * wg[None, :] * f)
        if abs(ok) < 1e-10:
            dm = I
        elif ok > 0:
            dm = np.sinh(np.sqrt(ok) * I) / np.sqrt(ok)
        else:
            dm = np.sin(np.sqrt(-ok) * I) / np.sqrt(-ok)
        out[t] = (1 + zz) * C_KMS / (100 * h) * dm
    return out


SN_BOX_MIN = np.array([0.0, 0.0, -3.0, -20.0, 0.0, 1.0])
SN_BOX_MAX = np.array([1.2, 1.5, 0.0, -18.5, 0.4, 5.0])
SN_TRUTH = np.array([0.3, 0.7, -1.0, -19.1, 0.14, 3.1])


def sn_data(nsn=740, seed=740, chi2mode=0, quad_nodes=4, sig_mB=0.15):
    rng = np.random.default_rng(seed)
    z = np.sort(rng.uniform(0.01, 1.4, nsn))
    rng.shuffle(z)
    om, ode, w0, M, al, be = SN_TRUTH
    x1 = rng.standard_normal(nsn)
    c = rng.normal(0.0, 0.1, nsn)
    mu = 5 * np.log10(lum_dist_np(z, om, ode, w0, 0.7)) + 25
    mB = mu + M - al * x1 + be * c + rng.normal(0.0, sig_mB, nsn)
    cov6 = np.zeros((nsn, 6))
    cov6[:, 0] = sig_mB ** 2
    return dict(z=z, mB=mB, x1=x1, c=c, cov6=cov6, sig_int=0.0, v_pec=0.0, h=0.7, chi2mode=chi2mode,
                add_logdet=0, quad_nodes=quad_nodes, ip_om=0, ip_ode=1, ip_w0=2, ip_M=3, ip_alpha=4, ip_beta=5,
                def_om=0.3, def_w0=-1.0, def_M=-19.3, def_alpha=0.0, def_beta=0.0)


def _sn_model_mag(sn, theta):
    """m_B model of every supernova at theta = (Om, Ode, w0, M, alpha, beta), vectorised over z."""
    om, ode, w0, M, al, be = theta
    z = sn["z"]
    xg, wg = np.polynomial.legendre.leggauss(8)
    nsub = 64
    t = np.linspace(0.0, 1.0, nsub + 1)
    e = z[:, None] * t[None, :]
    hw, c = 0.5 * (e[:, 1:] - e[:, :-1]), 0.5 * (e[:, 1:] + e[:, :-1])
    an = 1.0 + c[:, :, None] + hw[:, :, None] * xg[None, None, :]
    ok = 1.0 - om - ode
    f = 1.0 / np.sqrt(om * an ** 3 + ok * an ** 2 + ode * an ** (3 * (1 + w0)))
    I = np.sum(hw[:, :, None] * wg[None, None, :] * f, axis=(1, 2))
    if abs(ok) < 1e-10:
        dm = I
    elif ok > 0:
        dm = np.sinh(np.sqrt(ok) * I) / np.sqrt(ok)
    else:
        dm = np.sin(np.sqrt(-ok) * I) / np.sqrt(-ok)
    dl = (1 + z) * C_KMS / (100 * sn["h"]) * dm
    return 5 * np.log10(dl) + 25 + M - al * sn["x1"] + be * sn["c"]


def sn_fisher(sn, theta, rel_step=1e-4):
    """Fisher matrix J^T S^-1 J of the SN chi^2 (diagonal m_B errors) at theta, central differences."""
    theta = np.asarray(theta, float)
    sig2 = sn["cov6"][:, 0] + sn["sig_int"] ** 2
    J = np.empty((len(sn["z"]), len(theta)))
    for i in range(len(theta)):
        h = rel_step * max(1.0, abs(theta[i]))
        tp, tm = theta.copy(), theta.copy()
        tp[i] += h
        tm[i] -= h
        J[:, i] = (_sn_model_mag(sn, tp) - _sn_model_mag(sn, tm)) / (2 * h)
    return J.T @ (J / sig2[:, None])


def fisher_proposal(rng, K, theta0, F, bmin, bmax, fshift=1.0, frescale=2.0, df=-1, box_frac=None):
    """Initial proposal from a Fisher matrix (the reference's Fisher start): every
    component has covariance frescale * F^-1 and a mean shifted from theta0 by
    fshift * F^-1/2 xi, xi ~ N(0, I), clipped into the box; equal weights.
    box_frac: cap every standard deviation of F^-1 at box_frac (max - min),
    keeping the correlations (a Fisher matrix of a strongly tempered target
    is wider than the prior box)."""
    Cf = np.linalg.inv(F)
    Cf = 0.5 * (Cf + Cf.T)
    bmin, bmax = np.asarray(bmin, float), np.asarray(bmax, float)
    if box_frac is not None:
        sd = np.sqrt(np.diag(Cf))
        f = np.minimum(1.0, box_frac * (bmax - bmin) / sd)
        Cf = Cf * np.outer(f, f)
    L = np.linalg.cholesky(Cf)
    mu = theta0[None, :] + fshift * (rng.standard_normal((K, len(theta0))) @ L.T)
    mu = np.clip(mu, bmin + 1e-3 * (bmax - bmin), bmax - 1e-3 * (bmax - bmin))
    covs = np.repeat((frescale * Cf)[None], K, axis=0)
    return np.full(K, 1.0 / K), mu, covs, df


def sn_workload(nsn=740, K=10, seed=740, chi2mode=0, init="random"):
    """SN Ia run. init="random": the random-position proposal of the box;
    init="fisher": components around the truth with the Fisher covariance
    (a healthy run from the first iteration)."""
    sn = sn_data(nsn, seed, chi2mode)
    rng = np.random.default_rng(seed + 1)
    if init == "fisher":
        F = sn_fisher(sn, SN_TRUTH)
        w, mu, covs, df = fisher_proposal(rng, K, SN_TRUTH, F, SN_BOX_MIN, SN_BOX_MAX)
    else:
        w, mu, covs, df = random_pos_proposal(rng, K, SN_BOX_MIN, SN_BOX_MAX)
    return dict(sn=sn, bmin=SN_BOX_MIN.copy(), bmax=SN_BOX_MAX.copy(), prop=(w, mu, covs, df))


# ----------------------------------------------------------------- mixtures
def mixture_workload(D=32, K=64, Kt=16, nu=3, seed=64, prop_hi=6.0, target_scale=(0.7, 1.3), offset=0.3):
    """Proposal: K Student-t components, means ~ N(0, 4 I), covariances Q diag(logspace(0, prop_hi)) Q^T.

    Target: a different normalised Gaussian mixture of Kt components that lives
    inside the proposal's support: component j sits at proposal component 4j's
    mean shifted by `offset` standard deviations along random directions, with
    the same orientation and eigenvalues scaled by U(target_scale). (A target
    drawn independently of the proposal, with eigenvalues of at most 1e2, makes the
    importance weights degenerate in 32 dimensions: one sample carries all the
    weight and every component's update is singular.)"""
    rng = np.random.default_rng(seed)
    mu = rng.normal(0.0, 2.0, (K, D))
    ev = np.logspace(0.0, prop_hi, D)
    Qs = [random_orthogonal(rng, D) for _ in range(K)]
    covs = np.array([0.5 * ((Q * ev) @ Q.T + ((Q * ev) @ Q.T).T) for Q in Qs])
    stride = max(1, K // Kt)
    mut = np.empty((Kt, D))
    covt = np.empty((Kt, D, D))
    for j in range(Kt):
        k = (j * stride) % K
        mut[j] = mu[k] + (Qs[k] * np.sqrt(ev)) @ (offset * rng.standard_normal(D))
        e = ev * rng.uniform(*target_scale, D)
        c = (Qs[k] * e) @ Qs[k].T
        covt[j] = 0.5 * (c + c.T)
    return dict(prop=(np.full(K, 1.0 / K), mu, covs, nu), target=(np.full(Kt, 1.0 / Kt), mut, covt, -1))


# ----------------------------------------------------------------- template
def tpl_nphi(D):
    return 1 + D + D * (D + 1) // 2


def tpl_phi(theta):
    theta = np.atleast_2d(theta)
    N, D = theta.shape
    cols = [np.ones(N)] + [theta[:, i] for i in range(D)]
    cols += [theta[:, i] * theta[:, j] for i in range(D) for j in range(i, D)]
    return np.stack(cols, axis=1)


def template_workload(D=12, M=2048, K=16, rho=0.9, seed=91):
    rng = np.random.default_rng(seed)
    P = tpl_nphi(D)
    A = rng.normal(0.0, 1.0 / np.sqrt(P), (M, P))
    idx = np.arange(M)
    Cm = rho ** np.abs(idx[:, None] - idx[None, :])
    L = np.linalg.cholesky(Cm)
    theta0 = np.full(D, 0.1)
    dobs = A @ tpl_phi(theta0)[0] + L @ rng.standard_normal(M)
    bmin, bmax = -np.ones(D), np.ones(D)
    w, mu, covs, df = random_pos_proposal(np.random.default_rng(seed + 1), K, bmin, bmax)
    return dict(A=A, C=Cm, dobs=dobs, bmin=bmin, bmax=bmax, prop=(w, mu, covs, df), theta0=theta0)


def template_fisher(tw, theta=None):
    """Fisher matrix J^T C^-1 J of the template likelihood at theta (default the
    truth theta0), J = A dphi/dtheta (exact for the quadratic monomials)."""
    theta = np.asarray(tw["theta0"] if theta is None else theta, float)
    D = len(theta)
    P = tpl_nphi(D)
    dphi = np.zeros((P, D))
    for i in range(D):
        dphi[1 + i, i] = 1.0
    p = 1 + D
    for i in range(D):
        for j in range(i, D):
            dphi[p, i] += theta[j]
            dphi[p, j] += theta[i]
            p += 1
    J = tw["A"] @ dphi
    return J.T @ np.linalg.solve(tw["C"], J)
