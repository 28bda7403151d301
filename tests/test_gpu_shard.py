"""Shards of a run's sequences (cmc_job.seq_offset / nseq_total) walk exactly
the unsharded run's chains: two shards run one after the other on one GPU
equal the unsharded job bit for bit (same launch shape)."""
import numpy as np
import pytest

from cuda_mcmc_gb300 import shard, synth
from cuda_mcmc_gb300.device import DeviceJob

pytestmark = pytest.mark.gpu


def test_shards_equal_the_unsharded_run():
    w = synth.sgra(nvis=300, ncph=90, seed=21, nseq=8, nbeta=8)
    nburn, niter = 5, 7
    shape = {"R": 4, "T": 128, "phasor": 1}
    full = DeviceJob.from_workload(w, niter_total=niter, seed=77)
    full.shape = shape
    full.run(nburn, 0, do_init=True)
    full.run(0, niter)
    ref = full.to_numpy()
    local = []
    for s0, s1 in ((0, 3), (3, 8)):
        j = DeviceJob.from_workload(w, niter_total=niter, seed=77, seqs=(s0, s1))
        j.shape = shape
        j.run(nburn, 0, do_init=True)
        j.run(0, niter)
        local.append((0, s0, s1, j.to_numpy()))
    fields = ("pout", "tout", "chi2", "pcur", "chi2c", "rndst", "pstp", "n_acpt", "n_exch")
    got = shard.gather(local, 1, fields=fields)[0]
    for k in fields:
        assert np.array_equal(got[k], ref[k]), k
