"""Posterior post-processing of a sweep's records.

What the reference does after a fit (src/imgpu.py:453-469 rates; the
histograms, means / standard deviations and best fit of
src/model_obsfit.py:289-553), on the records in the reference's layouts:
``pout [nprm][nbeta][nseq][niter]`` and ``chi2 [nseq][niter]`` (the chi^2 of
temperature slot 0 after each iteration's exchanges).  Inputs may be numpy
arrays or torch tensors (histograms of device tensors are computed on the
device).
"""
from __future__ import annotations

import numpy as np

from .ess import ess


def _np(a):
    try:
        import torch
        if isinstance(a, torch.Tensor):
            return a.detach().cpu().numpy()
    except ImportError:   # pragma: no cover
        pass
    return np.asarray(a)


def summary(pout, chi2=None, slot=0, burn=0, q=(0.025, 0.16, 0.5, 0.84, 0.975), ndof=None):
    """Per mutable parameter at temperature slot ``slot`` (samples of all
    sequences pooled, the first ``burn`` recorded iterations dropped): mean,
    standard deviation, quantiles ``q``, ESS and Monte-Carlo standard error.
    With ``chi2`` also the best fit -- the recorded sample of slot 0 with the
    lowest chi^2 -- its chi^2 and, given ``ndof``, the reduced chi^2."""
    x = _np(pout)[:, slot, :, burn:].astype(np.float64)
    k = x.shape[0]
    flat = x.reshape(k, -1)
    out = {"mean": flat.mean(1), "sd": flat.std(1),
           "quantiles": dict(zip(q, np.quantile(flat, q, axis=1))),
           "ess": np.array([ess(x[i]) for i in range(k)])}
    out["mcse"] = out["sd"] / np.sqrt(np.maximum(out["ess"], 1.0))
    if chi2 is not None:
        if slot != 0:
            raise ValueError("chi2 records belong to slot 0")
        c = _np(chi2)[:, burn:]
        iq, it = np.unravel_index(np.argmin(c), c.shape)
        out["best"] = x[:, iq, it]
        out["best_chi2"] = float(c[iq, it])
        if ndof:
            out["best_chi2_reduced"] = float(c[iq, it]) / ndof
    return out


def histograms(pout, bins=50, slot=0, burn=0, ranges=None):
    """Histogram of each mutable parameter at slot ``slot``: (counts [nprm,
    bins], edges [nprm, bins + 1]); ``ranges`` [nprm, 2] (default: the sample
    range).  Torch tensors are binned on their device."""
    try:
        import torch
        is_t = isinstance(pout, torch.Tensor)
    except ImportError:   # pragma: no cover
        is_t = False
    if is_t:
        x = pout[:, slot, :, burn:].reshape(pout.shape[0], -1).float()
        counts, edges = [], []
        for i in range(x.shape[0]):
            lo, hi = ((float(x[i].min()), float(x[i].max())) if ranges is None
                      else (float(ranges[i][0]), float(ranges[i][1])))
            if hi <= lo:
                hi = lo + 1.0
            counts.append(torch.histc(x[i], bins=bins, min=lo, max=hi).cpu().numpy())
            edges.append(np.linspace(lo, hi, bins + 1))
        return np.stack(counts), np.stack(edges)
    x = _np(pout)[:, slot, :, burn:].reshape(_np(pout).shape[0], -1)
    counts, edges = [], []
    for i in range(x.shape[0]):
        r = None if ranges is None else (ranges[i][0], ranges[i][1])
        c, e = np.histogram(x[i], bins=bins, range=r)
        counts.append(c)
        edges.append(e)
    return np.stack(counts), np.stack(edges)


def rates(n_acpt, n_exch, niter, nseq):
    """Acceptance rate per (parameter, temperature) and exchange rate per
    temperature over the recorded iterations, summed over sequences:
    n_acpt [nprm][nbeta][nseq] / (niter nseq), n_exch [nbeta][nseq] /
    (niter nseq).  (imgpu keeps the reference's expression, src/imgpu.py:453,
    which adds 2 to the sum; these are the plain rates.)"""
    d = float(niter * nseq)
    return _np(n_acpt).sum(axis=-1) / d, _np(n_exch).sum(axis=-1) / d
