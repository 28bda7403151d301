"""ESS estimator (Geyer initial monotone sequence, multi-chain)."""
import numpy as np

from cuda_mcmc_gb300 import ess


def test_iid_chains_have_full_ess():
    x = np.random.default_rng(0).standard_normal((4, 4000))
    e = ess.ess(x)
    assert 0.85 * 16000 < e < 1.15 * 16000


def test_ar1_chain_matches_its_integrated_autocorrelation_time():
    rng = np.random.default_rng(1)
    phi, n = 0.8, 40000
    y = np.zeros((4, n))
    z = rng.standard_normal((4, n))
    for t in range(1, n):
        y[:, t] = phi * y[:, t - 1] + z[:, t]
    tau = (1 + phi) / (1 - phi)
    assert 0.8 < ess.ess(y) / (4 * n / tau) < 1.2


def test_ess_min_over_parameters_of_the_cold_slot():
    rng = np.random.default_rng(2)
    pout = rng.standard_normal((3, 2, 4, 1000)).astype(np.float32)
    pout[1, 0] = np.cumsum(pout[1, 0], axis=-1) * 0.01   # a random walk: tiny ESS
    assert ess.ess_min(pout) == ess.ess_per_param(pout)[1]
    assert ess.ess_min(pout) < 100
