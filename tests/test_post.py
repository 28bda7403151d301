"""Posterior post-processing (cuda_mcmc_gb300.post) on synthetic records with
known answers."""
import numpy as np
import torch

from cuda_mcmc_gb300 import post


def _records(seed=0, nprm=3, nbeta=4, nseq=6, niter=4000):
    rng = np.random.default_rng(seed)
    mu, sd = np.array([1.0, -2.0, 0.5]), np.array([0.1, 2.0, 0.01])
    pout = (mu[:, None, None, None] + sd[:, None, None, None] *
            rng.standard_normal((nprm, nbeta, nseq, niter))).astype(np.float32)
    chi2 = rng.uniform(100, 200, (nseq, niter)).astype(np.float32)
    chi2[3, niter // 3] = 50.0
    return pout, chi2, mu, sd


def test_summary_moments_quantiles_and_best_fit():
    pout, chi2, mu, sd = _records()
    s = post.summary(pout, chi2, ndof=25)
    assert np.all(np.abs(s["mean"] - mu) < 5 * s["mcse"])
    assert np.allclose(s["sd"], sd, rtol=0.03)
    assert np.allclose(s["quantiles"][0.5], mu, atol=0.05 * sd + 1e-6)
    assert np.allclose(s["quantiles"][0.84] - s["quantiles"][0.16], 2 * sd, rtol=0.05)
    assert np.all(s["ess"] > 0.5 * pout.shape[2] * pout.shape[3])   # independent draws
    assert np.array_equal(s["best"], pout[:, 0, 3, 4000 // 3].astype(np.float64))
    assert s["best_chi2"] == 50.0 and s["best_chi2_reduced"] == 2.0


def test_histograms_numpy_and_torch_agree():
    pout, _, _, _ = _records(1, niter=500)
    ranges = [(0.5, 1.5), (-8, 4), (0.45, 0.55)]
    c1, e1 = post.histograms(pout, bins=20, ranges=ranges)
    c2, e2 = post.histograms(torch.from_numpy(pout), bins=20, ranges=ranges)
    assert c1.shape == (3, 20) and np.allclose(e1, e2)
    assert np.abs(c1 - c2).max() <= 2          # bin-edge rounding only
    assert c1.sum(1).max() <= pout.shape[2] * pout.shape[3]


def test_rates():
    n_acpt = np.ones((3, 4, 6), np.int32) * 30
    n_exch = np.ones((4, 6), np.int32) * 12
    a, x = post.rates(n_acpt, n_exch, niter=100, nseq=6)
    assert np.allclose(a, 30 * 6 / 600.0) and np.allclose(x, 12 * 6 / 600.0)
