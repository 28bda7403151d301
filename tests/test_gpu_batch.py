"""The batched persistent path (many independent fits in work-list launches).

Each fit of a batch must walk exactly the chain it walks alone: with the same
seed and the same launch shape (the shape of its size class), the batch and a
single-job run of that fit give bit-identical outputs.  The chi^2 traces are
also checked against the FP64 oracle.
"""
import numpy as np
import pytest

import oracle
from cuda_mcmc_gb300 import _lib, synth
from cuda_mcmc_gb300.device import BatchJob, DeviceJob

pytestmark = pytest.mark.gpu

CHI2_RTOL = 1e-5


def _fits():
    # sizes spread over the batch size classes
    sizes = [(120, 36), (700, 210), (2500, 750), (5200, 1560)]
    return [synth.sgra(nvis=nv, ncph=nc, seed=50 + i, nseq=3, nbeta=16)
            for i, (nv, nc) in enumerate(sizes)]


def test_batch_equals_individual_runs_with_the_class_shape():
    fits = _fits()
    nburn, niter = 6, 8
    jobs = [DeviceJob.from_workload(w, niter_total=niter, seed=100 + i) for i, w in enumerate(fits)]
    batch = BatchJob(jobs)
    classes = batch.classes()
    assert sum(c["items"] for c in classes) == sum(w.nseq for w in fits)
    batch.run(nburn, 0, do_init=True)
    batch.run(0, niter)
    batch.check()
    # the batch does not report which class a fit landed in: try each shape
    for i, w in enumerate(fits):
        got = jobs[i].to_numpy()
        ref = DeviceJob.from_workload(w, niter_total=niter, seed=100 + i)
        matched = False
        for c in classes:
            ref2 = DeviceJob.from_workload(w, niter_total=niter, seed=100 + i)
            ref2.shape = {"R": c["R"], "T": c["T"], "phasor": c["phasor"]}
            try:
                ref2.run(nburn, 0, do_init=True)
                ref2.run(0, niter)
                ref2.check()
            except _lib.McmcError:
                continue
            r = ref2.to_numpy()
            # every shape makes the same decisions here (so pout and the
            # generator states agree for all of them); the chi^2 sums of the
            # fit's own class shape match to the bit
            fields = ("pout", "rndst", "chi2", "tout", "pcur", "chi2c", "n_acpt", "n_exch",
                      "n_hist", "pstp")
            if all(np.array_equal(r[f], got[f]) for f in fields):
                matched = True
                break
        assert matched, "fit %d: the batch result matches no single-job run" % i
        # chi^2 trace vs FP64 oracle
        pb = oracle.Problem(w.model, w.coor, w.dat, w.std2r, w.icoor, w.idat, w.nptot,
                            w.imodel, w.npass)
        P = np.stack([got["pout"][:, 0, q, it] for q in range(w.nseq) for it in (0, niter - 1)])
        _, _, _, c2 = oracle.calc_modchi2(pb, P.astype(np.float32))
        c2g = np.array([got["chi2"][q, it] for q in range(w.nseq) for it in (0, niter - 1)])
        assert np.max(np.abs(c2g - c2) / c2) < CHI2_RTOL


def test_batch_rejects_mixed_nbeta():
    a = DeviceJob.from_workload(synth.sgra(nvis=100, ncph=30, nseq=2, nbeta=8), niter_total=1)
    b = DeviceJob.from_workload(synth.sgra(nvis=100, ncph=30, nseq=2, nbeta=16), niter_total=1)
    with pytest.raises(_lib.McmcError, match="nbeta"):
        BatchJob([a, b])


def test_graph_schedule_equals_direct_launches():
    """BatchJob.graph_schedule captures burn-in and recorded chunks in one
    CUDA graph; one replay equals the same launches issued directly."""
    fits = _fits()[:2]
    nburn, niter = 7, 9
    outs = []
    for use_graph in (False, True):
        jobs = [DeviceJob.from_workload(w, niter_total=niter, seed=40 + i)
                for i, w in enumerate(fits)]
        b = BatchJob(jobs)
        b.run(0, 0, do_init=True)
        if use_graph:
            b.graph_schedule(nburn, niter, chunk=4).replay()
        else:
            for n in (4, 3):
                b.run(n, 0)
            for i0, n in ((0, 4), (4, 4), (8, 1)):
                b.run(0, n, itr0=i0)
        b.check()
        outs.append([j.to_numpy() for j in jobs])
    for a, c in zip(*outs):
        for k in ("pout", "tout", "chi2", "pcur", "chi2c", "rndst", "pstp"):
            assert np.array_equal(a[k], c[k]), k


def test_autotune_restores_state_and_keeps_chains_exact():
    """BatchJob.autotune times the shapes of each class on the batch itself
    and restores the state after every trial; the tuned batch still walks each
    fit's single-job chain with the chosen class shape, bit for bit."""
    fits = _fits()
    nburn, niter = 4, 5
    jobs = [DeviceJob.from_workload(w, niter_total=niter, seed=500 + i) for i, w in enumerate(fits)]
    batch = BatchJob(jobs)
    batch.run(0, 0, do_init=True)
    batch.check()
    before = [j.to_numpy() for j in jobs]
    chosen = batch.autotune(iters=1, R_values=(2, 4, 8), T_values=(128, 256))
    after = [j.to_numpy() for j in jobs]
    for a, b in zip(before, after):
        for k in a:
            assert np.array_equal(a[k], b[k]), k
    classes = batch.classes()
    assert [(c["R"], c["T"], c["phasor"]) for c in classes] == \
        [(c["R"], c["T"], c["phasor"]) for c in chosen]
    batch.run(0, 0, do_init=True)     # restart with the tuned shapes from the first chi^2
    batch.run(nburn, 0)
    batch.run(0, niter)
    batch.check()
    for i, w in enumerate(fits):
        got = jobs[i].to_numpy()
        ok = False
        for c in classes:
            ref = DeviceJob.from_workload(w, niter_total=niter, seed=500 + i)
            ref.shape = {"R": c["R"], "T": c["T"], "phasor": c["phasor"]}
            try:
                ref.run(0, 0, do_init=True)
                ref.run(nburn, 0)
                ref.run(0, niter)
                ref.check()
            except _lib.McmcError:
                continue
            r = ref.to_numpy()
            if all(np.array_equal(r[k], got[k]) for k in ("pout", "chi2", "pcur", "chi2c",
                                                           "rndst")):
                ok = True
                break
        assert ok, "fit %d matched no tuned class shape" % i


def test_plugin_model_batch_finds_the_rosenbrock_minimum():
    """A batch of plugin-model fits (Rosenbrock N=4, the reference's
    search_Rosenbrock example) runs through the same persistent launches and
    each fit's best recorded sample lies in the minimum's valley: f(x) < 0.02
    and within 0.2 of (1, 1, 1, 1) (the valley is flat along its curve)."""
    fits = [synth.rosenbrock(n=4, nseq=16, nbeta=32, nburn=1000, niter=2000) for _ in range(3)]
    jobs = [DeviceJob.from_workload(w, niter_total=2000, seed=900 + i) for i, w in enumerate(fits)]
    batch = BatchJob(jobs)
    batch.run(1000, 0, do_init=True)
    batch.run(0, 2000)
    batch.check()
    for j in jobs:
        s = j.to_numpy()
        i = np.argmin(s["chi2"])
        x = s["pout"][:, 0].reshape(4, -1)[:, i].astype(np.float64)
        f = np.sum(100 * (x[1:] - x[:-1] ** 2) ** 2 + (1 - x[:-1]) ** 2)
        assert f < 0.02 and np.all(np.abs(x - 1.0) < 0.2), (x, f)


def test_batch_cancel_stops_a_running_batch():
    """cmc_batch_cancel from the host while a long burn-in runs: the launch
    ends early (no further items, running ones stop at their next
    exchange), every job reports CMC_ERR_CANCELLED, the fits' step counters
    stopped part-way, and the next run (status words reset) runs normally."""
    import time
    import torch
    fits = synth.sgra_batch(nfits=16, seed=9, nseq=8, nbeta=16, nburn=0, niter=0)
    jobs = [DeviceJob.from_workload(w, niter_total=1, seed=40 + i) for i, w in enumerate(fits)]
    batch = BatchJob(jobs)
    batch.run(0, 0, do_init=True)
    batch.check()
    t0 = time.perf_counter()
    batch.run(5, 0)
    batch.check()
    per_iter = (time.perf_counter() - t0) / 5
    n = max(50, int(4.0 / per_iter))          # about 4 s uncancelled
    t0 = time.perf_counter()
    batch.run(n, 0)
    time.sleep(0.3)
    batch.cancel()
    torch.cuda.synchronize()
    elapsed = time.perf_counter() - t0
    assert elapsed < 0.5 * n * per_iter, (elapsed, n * per_iter)
    for j in jobs:
        with pytest.raises(_lib.McmcError) as err:
            j.check()
        assert err.value.code == _lib.CMC_ERR_CANCELLED
    # n_cnt [nprm][nbeta][nseq] starts at 1 and counts each parameter's
    # burn-in proposals: iterations done = (sum over parameters - nprm) / nprm
    # (5 + n uncancelled).  Small fits may finish before the cancel lands;
    # the batch as a whole stopped part-way, some of its sequences in the
    # middle of their burn-in and no fit ran past its schedule
    nprm = fits[0].nprm
    done = np.array([(j.to_numpy(("n_cnt",))["n_cnt"].sum(axis=0) - nprm).mean() / nprm
                     for j in jobs])
    assert done.sum() < 0.9 * len(jobs) * (5 + n), done
    assert np.all(done <= 5 + n) and np.any((done > 5) & (done < 5 + n)), done
    batch.clear_status()
    batch.run(2, 0)
    batch.check()
