"""Fisher-preconditioned Sgr A* fits.

The reference's sampler moves one parameter per proposal with a per-parameter
step that burn-in adapts (src/gpu_mcmc.cu:361-526).  On a posterior whose
parameters are correlated (the crescent's radius, thickness and flux are)
such a walk needs many proposals per independent sample.  This module adds
the gradient-informed schedule:

1. burn-in with the reference's proposals, until the chains sit near the
   posterior mass;
2. per sequence, the best replica's parameters (optionally polished by
   L-BFGS on the CUDA adjoint), and there the observed Fisher information
   F = Hessian(chi^2)/2 from central differences of the adjoint gradient
   (one batched gradient call for all sequences);
3. block proposals p += s_ibeta L z with L L^T = (2.38^2 / k) F^-1 for the
   rest of burn-in (which adapts s_ibeta, starting at 1/sqrt(beta)) and for
   the recorded iterations.

:func:`run_plain` and :func:`run_fisher` run one DeviceJob each way; the ESS
benchmark compares them on the same data and iteration budget.
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


def fisher_block(job, obj, rel_step=1e-3, polish_iter=0, points=None):
    """Set Fisher block proposals on ``job`` (a DeviceJob of the Sgr A* model
    whose data ``obj`` (grad.SgraChi2) holds).  Returns the Cholesky factors
    [nseq, nprm, nprm]."""
    pdescr = job.t["pdescr"].cpu().numpy()
    ivar = np.where(pdescr != 0)[0]
    pmin = job.t["pmint"].cpu().numpy().astype(np.float64)
    pmax = job.t["pmaxt"].cpu().numpy().astype(np.float64)
    P = best_points(job) if points is None else np.asarray(points, np.float64)
    if polish_iter > 0:
        P = np.stack([_grad.polish(obj, p, pmin, pmax, ivar=ivar, maxiter=polish_iter)[0]
                      for p in P])
    width = np.where(pmax > pmin, pmax - pmin, 1.0)
    F = _grad.fisher_many(obj, P, ivar=ivar, beta=1.0, rel_step=rel_step, scale=width)
    # floor the information at (10 prior widths)^-2 so that a direction the
    # data do not constrain still gets a finite step
    floor = 1.0 / (10.0 * width[ivar]) ** 2
    L = np.empty_like(F)
    for q in range(F.shape[0]):
        Fq = F[q] + np.diag(floor)
        L[q] = _grad.proposal_cholesky(Fq)
    job.set_block_proposals(L.astype(np.float32))
    return L


def run_plain(job, nburn, niter):
    """The reference's schedule: nburn adapted burn-in iterations, niter
    recorded iterations, one-parameter proposals throughout."""
    job.run(nburn, 0, do_init=True)
    job.run(0, niter, itr0=0)


def run_fisher(job, obj, nburn, niter, first=0.5, polish_iter=0, rel_step=1e-3):
    """Fisher schedule with the same iteration budget: ``first`` of the
    burn-in with one-parameter proposals, then Fisher block proposals for the
    rest of the burn-in and the recorded iterations."""
    n1 = int(round(first * nburn))
    job.run(n1, 0, do_init=True)
    torch.cuda.synchronize(job.device)
    L = fisher_block(job, obj, rel_step=rel_step, polish_iter=polish_iter)
    job.run(nburn - n1, 0)
    job.run(0, niter, itr0=0)
    return L


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
