"""The spread layout of the sweep (cmc_set_layout 2).

N co-resident CTAs of one cooperative launch share the nbeta*nseq replicas
evenly (R or R - 1 each, sequence-major), and each sequence's exchange runs
on the CTA holding its ibeta = 0 replica, through global memory.  Every
replica's chi^2 is summed by the same threads in the same order as in the
cluster layout when the CTAs have the same thread count, and the draws are
the same, so at equal T the two layouts walk identical chains: every output
is compared bit for bit.  The FP64-oracle and reference-build lock-steps of
the layout are in test_gpu_parity.py and test_gpu_ref_cuda.py.
"""
import numpy as np
import pytest
import torch

from cuda_mcmc_gb300 import mcmc_interf, synth
from cuda_mcmc_gb300.device import DeviceJob, sampler_defaults

pytestmark = pytest.mark.gpu

FIELDS = ("pcur", "chi2c", "flag", "ptent", "ptentn", "pstp", "n_acpt", "n_exch", "n_cnt",
          "n_hist", "tcur", "rndst", "pout", "tout", "chi2", "datm", "chi2m")


def _run(w, shape, seed=5, nburn=3, niter=5, chunks=None, block=None):
    job = DeviceJob.from_workload(w, niter_total=niter, seed=seed)
    job.shape = shape
    if block is not None:
        job.set_block_proposals(block)
    if chunks is None:
        job.run(nburn, niter, do_init=True)
    else:
        first = True
        for nb, ni in chunks:
            job.run(nb, ni, do_init=first)
            first = False
    job.check()
    return job, job.to_numpy(FIELDS)


def _same(a, b):
    for f in FIELDS:
        assert np.array_equal(a[f], b[f]), f


# (cluster shape, spread shape) pairs at equal threads per CTA
PAIRS = {
    "T256_phases": (dict(R=8, T=256, phasor=0, layout=1), dict(R=7, T=256, phasor=0, layout=2)),
    "T128_phasors": (dict(R=4, T=128, phasor=1, layout=1), dict(R=3, T=128, phasor=1, layout=2)),
    "T64_phases_R1": (dict(R=2, T=64, phasor=0, layout=1), dict(R=1, T=64, phasor=0, layout=2)),
}


@pytest.mark.parametrize("name", list(PAIRS))
def test_spread_equals_cluster_layout(name):
    """2000 + 600 data, 8 x 32 replicas: identical chains, records, model
    rows and generator states in both layouts."""
    cl, sp = PAIRS[name]
    w = synth.sgra(nvis=2000, ncph=600, seed=3, nseq=8, nbeta=32)
    jc, a = _run(w, cl)
    js, b = _run(w, sp)
    assert jc.config()["layout"] == "cluster"
    cfg = js.config()
    assert cfg["layout"] == "spread" and cfg["R"] == sp["R"] and cfg["blocks"] == -(-256 // sp["R"])
    _same(a, b)


def test_spread_block_proposals_equal_cluster_layout():
    """Block proposals read each replica's sequence's Cholesky factor: the
    same chains in both layouts."""
    w = synth.sgra(nvis=1000, ncph=300, seed=4, nseq=6, nbeta=16)
    rng = np.random.default_rng(2)
    k = w.nprm
    chol = np.stack([np.linalg.cholesky(np.eye(k) * 1e-4 + 1e-5 * (lambda A: A @ A.T)(
        rng.standard_normal((k, k)))) for _ in range(w.nseq)]).astype(np.float32)
    cl, sp = dict(R=8, T=256, phasor=0, layout=1), dict(R=5, T=256, phasor=0, layout=2)
    _, a = _run(w, cl, block=chol)
    _, b = _run(w, sp, block=chol)
    _same(a, b)


def test_spread_chunked_run_and_graph_equal_single_launch():
    """Resumed launches (state carried through the job arrays) and a captured
    CUDA graph of the schedule run the one-launch chains."""
    w = synth.sgra(nvis=2000, ncph=600, seed=3, nseq=8, nbeta=32)
    sp = dict(R=7, T=256, phasor=0, layout=2)
    _, a = _run(w, sp, nburn=4, niter=6)
    _, b = _run(w, sp, niter=6, chunks=[(2, 0), (2, 0), (0, 3), (0, 3)])
    _same(a, b)
    job = DeviceJob.from_workload(w, niter_total=6, seed=5)
    job.shape = sp
    job.run(0, 0, do_init=True)
    g = job.graph_schedule(4, 6, chunk=3)
    g.replay()
    job.check()
    _same(a, job.to_numpy(FIELDS))


def test_spread_is_the_automatic_choice_at_64x32():
    """At 2000 + 600 data and 64 x 32 replicas the library takes the spread
    layout by itself on a GPU where the cluster layout leaves its busiest SMs
    holding two CTAs of 8 (152 SMs: 256 CTAs); the host-buffer mcmc_cuda call
    then equals a device job forced into the cluster layout at the same
    threads per CTA."""
    w = synth.sgra(nvis=2000, ncph=600, seed=3, nseq=64, nbeta=32, nburn=3, niter=4)
    auto = DeviceJob.from_workload(w, niter_total=w.niter, seed=11)
    cfg = auto.config()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    if sms != 152:
        pytest.skip("the expected pick is stated for 152 SMs")
    assert cfg["layout"] == "spread" and cfg["R"] == 7 and cfg["T"] == 256, cfg
    ref, dev = _run(w, dict(R=8, T=256, phasor=cfg["phasor"], layout=1), seed=11, nburn=w.nburn,
                    niter=w.niter)
    s = sampler_defaults(w.pdescr, w.pmint, w.pmaxt, w.nbeta, w.nseq)
    nrep, nprm = w.nbeta * w.nseq, w.nprm
    pout = np.zeros((nprm, w.nbeta, w.nseq, w.niter), np.float32)
    tout = np.zeros((w.nbeta, w.nseq, w.niter), np.int32)
    chi2 = np.zeros((w.nseq, w.niter), np.float32)
    datm = np.zeros(nrep * (w.ndat + w.nvis), np.float32)
    chi2m = np.zeros((w.nbeta, w.nseq, w.ndat), np.float32)
    rndst = np.zeros((w.nbeta, w.nseq, 48), np.uint8)
    mcmc_interf.use_model("sgra")
    mcmc_interf.mcmcuda(w.coor, w.dat, w.std2r, w.icoor, w.idat, datm, chi2m, s["pdescr"],
                        s["ivar"], s["invar"], s["ptotal"], s["pmint"], s["pmaxt"], pout, tout,
                        chi2, s["chi2c"], s["tcur"], s["flag"], s["n_acpt"], s["n_exch"],
                        s["n_cnt"], s["n_hist"], w.beta(), s["pstp"], s["ptent"], s["ptentn"],
                        s["pcur"], rndst, np.uint64(11), w.imodel, w.coor.size, w.ndat,
                        w.icoor.size, w.idat.size, datm.size, w.nptot, nprm, 100, w.npass,
                        w.nbeta, w.nseq, w.nburn, w.niter)
    assert np.array_equal(pout, dev["pout"])
    assert np.array_equal(tout, dev["tout"])
    assert np.array_equal(chi2, dev["chi2"])
    assert np.array_equal(rndst, dev["rndst"])
    for f in ("pcur", "chi2c", "pstp", "n_acpt", "n_exch", "n_cnt", "n_hist", "tcur"):
        assert np.array_equal(s[f], dev[f]), f
    assert np.array_equal(datm, dev["datm"]) and np.array_equal(chi2m, dev["chi2m"])


def test_spread_global_phases_equal_cluster_layout():
    """Phases in global memory (3000 + 900 data): each spread CTA owns R
    regions, so a one-short CTA's unused slot writes a region nobody reads;
    the chains are the cluster layout's."""
    w = synth.sgra(nvis=3000, ncph=900, seed=6, nseq=8, nbeta=32)
    _, a = _run(w, dict(R=8, T=256, phasor=2, layout=1))
    js, b = _run(w, dict(R=7, T=256, phasor=2, layout=2))
    assert js.config()["phasor"] == 2
    _same(a, b)


GROUPED = {
    # phases in global memory: 8 sequences in groups of 3, 3 and 2, 14 CTAs
    "global_3groups": (dict(R=8, T=256, phasor=2, layout=1),
                       dict(R=7, T=256, phasor=2, layout=2, groups=3)),
    # phases in shared memory, two groups of 4 on 64 CTAs of 2 replicas each
    "shared_2groups_N64": (dict(R=4, T=128, phasor=0, layout=1),
                           dict(R=2, T=128, phasor=0, layout=2, groups=2, blocks=64)),
}


@pytest.mark.parametrize("name", list(GROUPED))
def test_spread_sequence_groups_equal_cluster_layout(name):
    """One spread launch running its sequences in groups, one group after the
    other on all of its CTAs (what bounds the phase regions in use with
    phases in global memory): the sequences' chains are independent, so every
    output equals the cluster layout's, bit for bit, over a chunked run."""
    cl, sp = GROUPED[name]
    w = synth.sgra(nvis=3000, ncph=900, seed=6, nseq=8, nbeta=32)
    _, a = _run(w, cl, nburn=3, niter=6, chunks=[(3, 0), (0, 4), (0, 2)])
    js, b = _run(w, sp, nburn=3, niter=6, chunks=[(3, 0), (0, 4), (0, 2)])
    cfg = js.config()
    assert cfg["layout"] == "spread" and cfg["groups"] == sp["groups"], cfg
    if "blocks" in sp:
        assert cfg["blocks"] == sp["blocks"]
    _same(a, b)


def test_spread_groups_are_the_automatic_choice_beyond_one_wave():
    """More replicas than the resident CTAs hold at 7 per CTA (2000 + 600
    data, 128 x 32 on 152 SMs): the library runs the sequences in two groups
    of 64 on 293 CTAs (1.106e8 evals/s against the cluster layout's 1.009e8
    measured on a GB300); the chains are the cluster layout's."""
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    if sms != 152:
        pytest.skip("the expected pick is stated for 152 SMs")
    w = synth.sgra(nvis=2000, ncph=600, seed=3, nseq=128, nbeta=32)
    job = DeviceJob.from_workload(w, niter_total=2, seed=7)
    cfg = job.config()
    assert cfg["layout"] == "spread" and cfg["groups"] == 2 and cfg["R"] == 7, cfg
    assert cfg["blocks"] == 293
    _, a = _run(w, dict(R=8, T=256, phasor=cfg["phasor"], layout=1), seed=7, nburn=1, niter=2)
    _, b = _run(w, None, seed=7, nburn=1, niter=2)
    _same(a, b)


def test_spread_rejects_what_it_cannot_run():
    """Forced onto a job it cannot hold (more than 32 temperatures), the
    spread layout reports no shape instead of running."""
    from cuda_mcmc_gb300 import _lib
    w = synth.sgra(nvis=200, ncph=60, seed=8, nseq=1, nbeta=64)
    job = DeviceJob.from_workload(w, niter_total=1, seed=1)
    job.shape = dict(R=4, T=128, phasor=0, layout=2)
    with pytest.raises(_lib.McmcError):
        job.config()


def test_spread_wait_that_runs_out_reports_timeout(monkeypatch):
    """A wait that nothing ends: with the test hook CMC_SPREAD_HOLD_SEQ the
    owner of sequence 0 never completes its exchange.  Every CTA's bounded
    wait runs out (about a second), the CTAs leave their iteration loops and
    the launch ends with CMC_ERR_TIMEOUT in the status word; the context stays
    usable and the next launch runs the normal chains."""
    import time
    from cuda_mcmc_gb300 import _lib
    w = synth.sgra(nvis=400, ncph=120, seed=3, nseq=4, nbeta=16)
    shape = dict(R=5, T=128, phasor=0, layout=2)
    job = DeviceJob.from_workload(w, niter_total=2, seed=5)
    job.shape = shape
    monkeypatch.setenv("CMC_SPREAD_HOLD_SEQ", "0")
    t0 = time.perf_counter()
    job.run(2, 2, do_init=True)
    with pytest.raises(_lib.McmcError) as err:
        job.check()
    elapsed = time.perf_counter() - t0
    monkeypatch.delenv("CMC_SPREAD_HOLD_SEQ")
    assert err.value.code == _lib.CMC_ERR_TIMEOUT
    assert elapsed < 30.0
    _, a = _run(w, dict(R=8, T=128, phasor=0, layout=1), nburn=2, niter=2)
    _, b = _run(w, shape, nburn=2, niter=2)
    _same(a, b)


def test_spread_timeout_in_a_group_skips_the_later_groups(monkeypatch):
    """The held sequence in the first of two groups: its waits run out, the
    CTAs start no later group (the abort flag is read once per CTA before
    each), and the launch reports CMC_ERR_TIMEOUT; the next launch runs
    normally."""
    import time
    from cuda_mcmc_gb300 import _lib
    w = synth.sgra(nvis=400, ncph=120, seed=3, nseq=4, nbeta=16)
    shape = dict(R=4, T=128, phasor=0, layout=2, groups=2)
    job = DeviceJob.from_workload(w, niter_total=2, seed=5)
    job.shape = shape
    monkeypatch.setenv("CMC_SPREAD_HOLD_SEQ", "1")
    t0 = time.perf_counter()
    job.run(2, 2, do_init=True)
    with pytest.raises(_lib.McmcError) as err:
        job.check()
    elapsed = time.perf_counter() - t0
    monkeypatch.delenv("CMC_SPREAD_HOLD_SEQ")
    assert err.value.code == _lib.CMC_ERR_TIMEOUT
    assert elapsed < 30.0
    _, a = _run(w, dict(R=8, T=128, phasor=0, layout=1), nburn=2, niter=2)
    _, b = _run(w, shape, nburn=2, niter=2)
    _same(a, b)

