"""The allocation-free entry point cmc_run_noalloc (libcmc_sgra.so).

Some callers of this library cannot give it new device memory while they run:
their device memory is reserved up front by another allocator, or a
cudaMalloc / cudaFree would synchronise a latency-critical pipeline between its
stages.  cmc_run_noalloc serves them: it is cmc_run with the packed-data
scratch taken from a fixed 4 MiB array inside the library instead of from
job->work.  These tests call it through the C-ABI and check that it gives
cmc_run's results on two calls in a row (a start and a resume), and that it
refuses a job whose scratch would not fit in the fixed array.

This file sorts last so that a run stopping at the first failure has already
run every other test.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from cuda_mcmc_gb300 import _lib, synth
from cuda_mcmc_gb300.device import DeviceJob

pytestmark = pytest.mark.gpu

CHI2_RTOL = 1e-5


def _noalloc(L):
    f = L.cmc_run_noalloc
    f.argtypes = [C.POINTER(_lib.CmcJob), C.c_void_p]
    f.restype = C.c_int
    return f


def _run_noalloc(L, job, nburn, niter, do_init, itr0):
    j = job.job
    j.do_init = 1 if do_init else 0
    j.nburn, j.niter, j.itr0 = nburn, niter, itr0
    s = torch.cuda.current_stream()
    _lib.check(L, _noalloc(L)(C.byref(j), C.c_void_p(s.cuda_stream)))
    job.check()


def test_noalloc_matches_cmc_run_on_two_calls():
    L = _lib.load("sgra")
    w = synth.sgra(nvis=2000, ncph=600, seed=3, nseq=8, nbeta=32)
    a = DeviceJob.from_workload(w, niter_total=20, seed=7)   # cmc_run, job->work
    b = DeviceJob.from_workload(w, niter_total=20, seed=7)   # cmc_run_noalloc
    calls = [(10, 10, True, 0), (5, 10, False, 10)]
    for nburn, niter, init, itr0 in calls:
        a.run(nburn, niter, do_init=init, itr0=itr0)
        a.check()
        _run_noalloc(L, b, nburn, niter, init, itr0)
        sa, sb = a.to_numpy(), b.to_numpy()
        for f in ("n_acpt", "n_exch", "n_cnt", "n_hist", "tcur", "tout", "flag", "ptentn",
                  "rndst"):
            assert np.array_equal(sa[f], sb[f]), f
        for f in ("pcur", "pout", "pstp", "ptent"):
            assert np.allclose(sa[f], sb[f], rtol=1e-6, atol=0), f
        for f in ("chi2c", "chi2"):
            assert np.allclose(sa[f], sb[f], rtol=CHI2_RTOL, atol=0), f


def test_noalloc_rejects_scratch_beyond_its_array():
    L = _lib.load("sgra")
    w = synth.sgra(nvis=200, ncph=60, seed=1, nseq=1, nbeta=2)
    job = DeviceJob.from_workload(w, niter_total=1)
    big = _lib.CmcJob.from_buffer_copy(job.job)
    nvis = 100_000                       # 100k points need > 4 MiB of packed data
    big.hidat[0] = nvis
    big.ndat = nvis
    big.ncoor = 2 * nvis
    big.ndatm = 2 * 2 * nvis
    big.do_init, big.nburn, big.niter = 1, 1, 0
    rc = _noalloc(L)(C.byref(big), None)
    assert rc == _lib.CMC_ERR_ARG
    assert "4 MiB" in L.cmc_last_error().decode()
