"""The allocation-free entry point cmc_run_noalloc (libcmc_sgra.so).

Some callers of this library cannot give it new device memory while they run:
their device memory is reserved up front by another allocator, or a
cudaMalloc / cudaFree would synchronise a latency-critical pipeline between its
stages.  cmc_run_noalloc serves them: it is cmc_run with the packed-data
scratch taken from a fixed 4 MiB array inside the library instead of from
job->work.  These tests call it through the C-ABI and check that it gives
cmc_run's results on two calls in a row (a start and a resume), and that it
refuses a job whose scratch would not fit in the fixed array.

With 2048 points or more the replicas' closure phases may live in global
memory: inside the fixed array beside the packed data when they fit there,
else in shared memory.  Both placements are compared with cmc_run at the same
launch shape.

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


STATIC_BYTES = 4 << 20


def _compare(a, b):
    sa, sb = a.to_numpy(), b.to_numpy()
    for f in ("pout", "tout", "chi2", "pcur", "chi2c", "pstp", "n_acpt", "n_exch", "n_hist",
              "rndst", "flag"):
        assert np.array_equal(sa[f], sb[f]), f


def _noalloc_shape(L, job):
    """The launch shape cmc_run picks for this job with a job->work of the
    fixed array's size (what cmc_run_noalloc runs)."""
    j = _lib.CmcJob.from_buffer_copy(job.job)
    j.work_bytes = STATIC_BYTES
    R, G, T, P, W = (C.c_int() for _ in range(5))
    sm = C.c_size_t()
    _lib.check(L, L.cmc_query_config(C.byref(j), C.byref(R), C.byref(G), C.byref(T), C.byref(P),
                                     C.byref(sm), C.byref(W)))
    return {"R": R.value, "T": T.value, "phasor": P.value}


def test_noalloc_global_phases_inside_the_array():
    """2500 points, 16 replicas: the phase regions (160 KB) fit in the array
    beside the packed data; forced to phases in global memory, the
    allocation-free call equals cmc_run at the same shape on two calls."""
    L = _lib.load("sgra")
    w = synth.sgra(nvis=2500, ncph=750, seed=5, nseq=2, nbeta=8)
    shape = {"R": 4, "T": 128, "phasor": 2}
    a = DeviceJob.from_workload(w, niter_total=12, seed=9)
    a.shape = shape
    b = DeviceJob.from_workload(w, niter_total=12, seed=9)
    for nburn, niter, init, itr0 in [(6, 6, True, 0), (3, 6, False, 6)]:
        a.run(nburn, niter, do_init=init, itr0=itr0)
        a.check()
        L.cmc_set_config(shape["R"], shape["T"], shape["phasor"])
        try:
            _run_noalloc(L, b, nburn, niter, init, itr0)
        finally:
            L.cmc_set_config(0, 0, -1)
        _compare(a, b)


def test_noalloc_phases_fall_back_to_shared_memory():
    """3000 points at 16 x 32 replicas: the phase regions (6 MB) do not fit in
    the 4 MiB array, so the call keeps the phases in shared memory; it equals
    cmc_run at that launch shape."""
    L = _lib.load("sgra")
    w = synth.sgra(nvis=3000, ncph=900, seed=6, nseq=16, nbeta=32)
    a = DeviceJob.from_workload(w, niter_total=6, seed=4)
    b = DeviceJob.from_workload(w, niter_total=6, seed=4)
    shape = _noalloc_shape(L, b)
    assert shape["phasor"] != 2
    a.shape = shape
    for nburn, niter, init, itr0 in [(3, 3, True, 0), (2, 3, False, 3)]:
        a.run(nburn, niter, do_init=init, itr0=itr0)
        a.check()
        _run_noalloc(L, b, nburn, niter, init, itr0)
        _compare(a, b)


def test_noalloc_rejects_phases_that_fit_nowhere():
    """70,000 points and 1000 closures at 32 temperatures: the packed data
    fits in the array, the phases fit neither there nor in shared memory."""
    L = _lib.load("sgra")
    w = synth.sgra(nvis=70000, ncph=1000, seed=7, nseq=2, nbeta=32)
    job = DeviceJob.from_workload(w, niter_total=1)
    j = job.job
    j.do_init, j.nburn, j.niter, j.itr0 = 1, 1, 0, 0
    rc = _noalloc(L)(C.byref(j), None)
    assert rc == _lib.CMC_ERR_UNSUPPORTED
    assert "4 MiB" in L.cmc_last_error().decode()
