"""The Fisher schedule (fit.run_fisher) samples the same posterior as the
reference's schedule (fit.run_plain) with more effective samples per
iteration: on one seeded small Sgr A* data set, the two posteriors' means
agree within 5 combined Monte-Carlo standard errors and their widths within
15%, and the Fisher run's minimum ESS is larger."""
import numpy as np
import pytest

from cuda_mcmc_gb300 import fit, synth
from cuda_mcmc_gb300.device import DeviceJob
from cuda_mcmc_gb300.grad import SgraChi2

pytestmark = pytest.mark.gpu


def test_fisher_schedule_matches_the_plain_posterior():
    w = synth.sgra(nvis=400, ncph=120, seed=8, nseq=8, nbeta=8)
    nburn, niter = 2000, 4000
    jp = DeviceJob.from_workload(w, niter_total=niter, seed=21)
    fit.run_plain(jp, nburn, niter)
    jf = DeviceJob.from_workload(w, niter_total=niter, seed=21)
    p_star, F = fit.run_fisher(jf, SgraChi2.from_workload(w), nburn, niter)
    jp.check()
    jf.check()
    sp = fit.posterior_summary(jp.t["pout"].cpu().numpy())
    sf = fit.posterior_summary(jf.t["pout"].cpu().numpy())
    z = np.abs(sp["mean"] - sf["mean"]) / np.sqrt(sp["mcse"] ** 2 + sf["mcse"] ** 2)
    assert z.max() < 5.0, z
    assert np.all(np.abs(np.log(sf["sd"] / sp["sd"])) < np.log(1.15)), sf["sd"] / sp["sd"]
    assert sf["ess"].min() > sp["ess"].min()
    # the polished point is inside the posterior mass
    ivar = np.where(np.asarray(w.pdescr) != 0)[0]
    assert np.all(np.abs(p_star[ivar] - sf["mean"]) < 4 * sf["sd"])
    assert np.all(np.linalg.eigvalsh(F) > 0)
