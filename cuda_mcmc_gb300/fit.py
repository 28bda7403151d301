"""Fisher-preconditioned Sgr A* fits.

The reference's sampler moves one parameter per proposal with a per-parameter
step that burn-in adapts (src/gpu_mcmc.cu:361-526).  On a posterior whose
parameters are correlated (the crescent's radius, thickness and flux are)
such a walk needs many proposals per independent sample, and chains that
start far from the posterior mass take long to reach it.  This module adds
the gradient-informed schedule (:func:`run_fisher`):

1. a short burn-in with the reference's proposals from the usual uniform
   start;
2. the best replica found so far is polished by bounded L-BFGS on the CUDA
   adjoint (grad.polish), and at the polished point p* the Fisher
   information F (Gauss-Newton, grad.SgraChi2.fisher_gn) plus the uniform
   prior's information 12 / width^2;
3. every replica restarts from p* + N(0, F^-1 / beta) (clipped into the prior
   box): a burn-in restart, so that no chain spends the budget crossing the
   prior box;
4. block proposals p += s_ibeta L z with L L^T = (2.38^2 / k) F^-1 for the
   rest of the burn-in (which adapts s_ibeta, starting at 1/sqrt(beta)) and
   the recorded iterations.

:func:`run_plain` is the reference's schedule with the same iteration budget;
the ESS benchmark workloads compare the two.
"""
from __future__ import annotations

import numpy as np
import torch

from . import grad as _grad


def best_points(job):
    """Per sequence, the parameters of the replica with the lowest chi^2:
    [nseq, nptot] float64."""
    s = job.to_numpy(("pcur", "chi2c"))
    c = s["chi2c"]                                   # [nbeta, nseq]
    ib = np.argmin(c, axis=0)
    return s["pcur"][ib, np.arange(job.nseq)].astype(np.float64)


def run_plain(job, nburn, niter):
    """The reference's schedule: nburn adapted burn-in iterations, niter
    recorded iterations, one-parameter proposals throughout."""
    job.run(nburn, 0, do_init=True)
    job.run(0, niter, itr0=0)


def _box(job):
    pdescr = job.t["pdescr"].cpu().numpy()
    pmin = job.t["pmint"].cpu().numpy().astype(np.float64)
    pmax = job.t["pmaxt"].cpu().numpy().astype(np.float64)
    return pdescr, np.where(pdescr != 0)[0], pmin, pmax


def fisher_at(obj, p, pmin, pmax, ivar):
    """Gauss-Newton Fisher information of chi^2/2 at p over ivar
    (grad.SgraChi2.fisher_gn) plus the uniform prior's Gaussian-equivalent
    information diag(12 / width^2), so that a direction the data do not
    constrain keeps a prior-sized step: float64 [k, k].  (The Hessian of
    chi^2 itself is not used: closure residuals that wrap at +-pi make it
    non-smooth, and far from the optimum it is indefinite.)"""
    width = np.where(pmax > pmin, pmax - pmin, 1.0)
    F = obj.fisher_gn(np.asarray(p, np.float32)[None])[0].double().cpu().numpy()
    F = F[np.ix_(ivar, ivar)]
    # float32 accumulation can leave J^T J slightly indefinite: clip at 0
    w, V = np.linalg.eigh(0.5 * (F + F.T))
    return (V * np.maximum(w, 0.0)) @ V.T + np.diag(12.0 / width[ivar] ** 2)


def covariance(F):
    """F^-1 through the eigen-decomposition (symmetric, positive definite for
    a positive definite F)."""
    w, V = np.linalg.eigh(0.5 * (F + F.T))
    cov = (V / w) @ V.T
    return 0.5 * (cov + cov.T)


def cholesky_psd(A):
    """Lower Cholesky factor of a symmetric positive (semi-)definite A, with
    the smallest diagonal jitter that makes the factorisation succeed."""
    A = 0.5 * (A + A.T)
    jitter = 0.0
    scale = float(np.mean(np.diag(A)))
    for _ in range(12):
        try:
            return np.linalg.cholesky(A + jitter * np.eye(A.shape[0]))
        except np.linalg.LinAlgError:
            jitter = scale * (1e-14 if jitter == 0.0 else 10.0 * jitter / scale)
    raise np.linalg.LinAlgError("covariance is not positive definite")


def restart_near(job, p_star, cov, seed=0, cap=10.0):
    """Burn-in restart: every replica's parameters ivar drawn from
    N(p*, cov * min(1/beta, cap^2)), angles wrapped, clipped into the prior
    box; chi2c recomputed (calc_modchi2) so the sweep can continue."""
    pdescr, ivar, pmin, pmax = _box(job)
    beta = job.t["beta"].cpu().numpy().astype(np.float64)
    pcur = job.t["pcur"].cpu().numpy()
    rng = np.random.default_rng(seed)
    Lc = cholesky_psd(np.asarray(cov, np.float64))
    z = rng.standard_normal((job.nbeta, job.nseq, ivar.size))
    s = np.minimum(1.0 / np.sqrt(beta), cap)
    p = np.asarray(p_star, np.float64)[ivar] + (z @ Lc.T) * s[:, None, None]
    ang = pdescr[ivar] == 2
    p[..., ang] = np.arctan2(np.sin(p[..., ang]), np.cos(p[..., ang]))
    pcur[..., ivar] = np.clip(p, pmin[ivar], pmax[ivar]).astype(np.float32)
    job.set_state(pcur=pcur, flag=np.ones((job.nbeta, job.nseq), np.int32))
    job.eval()
    job.check()


def fisher_setup(job, obj, polish_iter=200, restart=True, seed=0):
    """Steps 2-4 of the Fisher schedule on a job whose chains have had a short
    burn-in: polish the best replica, Fisher information there, optional
    restart of all replicas around it, block proposals.  Returns (p*, F)."""
    pdescr, ivar, pmin, pmax = _box(job)
    s = job.to_numpy(("pcur", "chi2c"))
    ib, iq = np.unravel_index(np.argmin(s["chi2c"]), s["chi2c"].shape)
    p_star = s["pcur"][ib, iq].astype(np.float64)
    if polish_iter > 0:
        p_star = _grad.polish(obj, p_star, pmin, pmax, ivar=ivar, maxiter=polish_iter)[0]
    F = fisher_at(obj, p_star, pmin, pmax, ivar)
    cov = covariance(F)
    if restart:
        restart_near(job, p_star, cov, seed=seed)
    L = cholesky_psd(cov * (2.38 ** 2 / ivar.size))
    job.set_block_proposals(L.astype(np.float32))
    return p_star, F


def run_fisher(job, obj, nburn, niter, first=0.25, graph=False, chunk=500, **kw):
    """Fisher schedule with the same iteration budget as :func:`run_plain`
    (see the module docstring): ``first`` of the burn-in with the reference's
    proposals, then :func:`fisher_setup`, the rest of the burn-in and the
    recorded iterations with block proposals -- with ``graph``, that rest of
    the schedule captured as one CUDA graph of launches of at most ``chunk``
    iterations and replayed once.  Returns (p*, F)."""
    n1 = int(round(first * nburn))
    job.run(n1, 0, do_init=True)
    out = fisher_setup(job, obj, **kw)
    if graph:
        job.graph_schedule(nburn - n1, niter, chunk=chunk, itr0=0).replay()
    else:
        job.run(nburn - n1, 0)
        job.run(0, niter, itr0=0)
    return out


def posterior_summary(pout, slot=0, burn_frac=0.0):
    """Mean, standard deviation and Monte-Carlo standard error (from the
    ESS) of each parameter at temperature slot ``slot`` of
    pout[nprm][nbeta][nseq][niter], pooled over sequences."""
    from .ess import ess
    x = np.asarray(pout)[:, slot]
    n0 = int(burn_frac * x.shape[-1])
    x = x[..., n0:]
    mean = x.mean(axis=(1, 2))
    sd = x.std(axis=(1, 2))
    e = np.array([ess(x[k]) for k in range(x.shape[0])])
    return {"mean": mean, "sd": sd, "ess": e, "mcse": sd / np.sqrt(np.maximum(e, 1.0))}
