"""Effective sample size of MCMC output.

``ess(x)`` for chains x[m, n] (m chains of n draws): Geyer's initial
monotone sequence estimator applied to the multi-chain autocorrelation
    rho_t = 1 - (W - mean_m acov_m(t)) / var_plus,
with W the mean within-chain variance and var_plus the pooled variance
estimate (the formulation of Vehtari, Gelman, Simpson, Carpenter and
Buerkner 2021, "Rank-normalization, folding, and localization", Bayesian
Analysis).  Autocovariances come from FFTs.  ``ess_min`` takes the
reference's ``pout[nprm][nbeta][nseq][niter]`` and returns the minimum over
parameters of the ESS of the coldest (T = 1) slot, pooled over sequences.
"""
from __future__ import annotations

import numpy as np


def _autocov(x):
    n = x.shape[-1]
    xc = x - x.mean(axis=-1, keepdims=True)
    nfft = 1 << (2 * n - 1).bit_length()
    f = np.fft.rfft(xc, nfft, axis=-1)
    ac = np.fft.irfft(f * np.conj(f), nfft, axis=-1)[..., :n]
    return ac / n


def ess(x):
    x = np.asarray(x, np.float64)
    if x.ndim == 1:
        x = x[None]
    m, n = x.shape
    if n < 4:
        return float(m * n)
    acov = _autocov(x)
    w = acov[:, 0].mean() * n / (n - 1.0)
    var_plus = w * (n - 1.0) / n
    if m > 1:
        var_plus += x.mean(axis=1).var(ddof=1)
    if var_plus <= 0:
        return float(m * n)
    rho = 1.0 - (w - acov.mean(axis=0)) / var_plus
    rho[0] = 1.0
    # initial positive sequence of pair sums, made monotone
    t, tau, prev = 0, 0.0, np.inf
    while t + 1 < n:
        p = rho[t] + rho[t + 1]
        if p < 0:
            break
        p = min(p, prev)
        tau += p
        prev = p
        t += 2
    tau = -1.0 + 2.0 * tau
    tau = max(tau, 1.0 / np.log10(m * n + 10.0))
    return float(m * n / tau)


def ess_per_param(pout, slot=0):
    """ESS of each mutable parameter of pout[nprm][nbeta][nseq][niter] at
    temperature slot `slot`, pooled over sequences."""
    pout = np.asarray(pout)
    return np.array([ess(pout[k, slot]) for k in range(pout.shape[0])])


def ess_min(pout, slot=0):
    return float(ess_per_param(pout, slot).min())
