"""Parity of the CUDA path (through the C-ABI) with the oracle and the
reference's own code.

Tolerances (float32 kernels against the FP64 oracle):
  * model amplitudes: |err| <= 1e-5 |V| + 1e-6 Zsp.  The absolute part is a
    few float32 ulps of the zero-spacing flux Zsp: near a visibility null the
    amplitude is a float32 sum of O(Zsp) terms that cancel, so no float32
    evaluation (the reference's own included) is relatively accurate there;
  * model phases: |err| <= 2e-5 + 1e-6 Zsp/|V| rad (the phase error an
    amplitude-scale error of 1e-6 Zsp makes); closure phases: 1e-4 rad;
  * chi^2 of a parameter set: relative 1e-5;
  * decisions (accept / reject / swap): identical, except a decision whose
    uniform draw lies within 1e-3*alpha of its acceptance probability alpha
    (a near tie that float32 chi^2 may legitimately flip).
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from conftest import golden
from cuda_mcmc_gb300 import _lib, mcmc_interf, synth
from cuda_mcmc_gb300.device import BatchJob, DeviceJob

pytestmark = pytest.mark.gpu

AMP_RTOL, AMP_ATOL, PHASE_ATOL, CPH_ATOL = 1e-5, 1e-6, 2e-5, 1e-4
CHI2_RTOL, TIE_RTOL = 1e-5, 1e-3


def _wrap(x):
    return np.angle(np.exp(1j * x))


def _pb(w):
    return oracle.Problem(w.model, w.coor, w.dat, w.std2r, w.icoor, w.idat, w.nptot, w.imodel,
                          w.npass)


@pytest.fixture(scope="module", autouse=True)
def _libs():
    for m in ("sgra", "rosenbrock", "solvsys", "nlsys"):
        _lib.load(m)


# ---------------------------------------------------------------------------
# model + chi^2 (calc_modchi2 / calc_model through the host C-ABI)
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("name", ["sgra_modchi2_m9.npz", "sgra_modchi2_m13.npz",
                                  "sgra_modchi2_cpext.npz"])
def test_calc_modchi2_sgra(name):
    g = golden(name)
    mcmc_interf.use_model("sgra")
    P = g["pcur"]
    nrep, nptot = P.shape
    nvis, ndat = int(g["idat"][0]), g["dat"].size
    datm = np.zeros(nrep * (ndat + nvis), np.float32)
    chi2m = np.zeros((nrep, 1, ndat), np.float32)
    chi2c = np.zeros((nrep, 1), np.float32)
    flag = np.ones((nrep, 1), np.int32)
    mcmc_interf.calcmodchi2(g["coor"], g["dat"], g["std2r"], g["icoor"], g["idat"], datm, chi2m,
                            P.reshape(nrep, 1, nptot).copy(), chi2c, flag, int(g["imodel"]),
                            g["coor"].size, ndat, g["icoor"].size, 3, datm.size, nptot, nrep, 1)
    pb = oracle.Problem("sgra", g["coor"], g["dat"], g["std2r"], g["icoor"], g["idat"], nptot,
                        int(g["imodel"]), 2)
    d, ph, c2m, c2 = oracle.calc_modchi2(pb, P)
    gd = datm[:nrep * ndat].reshape(nrep, ndat)
    gph = datm[nrep * ndat:].reshape(nrep, nvis)
    zsp = P[:, :1]
    amp_err = np.abs(gd[:, :nvis] - d[:, :nvis]) - AMP_RTOL * np.abs(d[:, :nvis])
    assert amp_err.max() <= AMP_ATOL * zsp.min()
    ph_tol = PHASE_ATOL + AMP_ATOL * zsp / np.maximum(np.abs(d[:, :nvis]), 1e-30)
    assert np.all(np.abs(_wrap(gph - ph)) <= ph_tol)
    assert np.abs(_wrap(gd[:, nvis:] - d[:, nvis:])).max() < CPH_ATOL
    assert np.max(np.abs(chi2c.ravel() - c2) / c2) < CHI2_RTOL
    # chi2c is the sum of its chi2m row, as in the reference (calc_chi2)
    assert np.allclose(chi2m.reshape(nrep, ndat).sum(1), chi2c.ravel(), rtol=1e-5)
    # and the reference's own float32 numbers agree to float32 accuracy
    assert np.max(np.abs(chi2c.ravel() - g["chi2c"]) / g["chi2c"]) < CHI2_RTOL


def test_calc_model_sgra():
    w = synth.sgra(nvis=300, ncph=0, seed=9, nseq=1, nbeta=1)
    rng = np.random.default_rng(3)
    P = rng.uniform(synth.SGRA9_PMIN, synth.SGRA9_PMAX, (8, 9)).astype(np.float32)
    nrep, nvis = 8, 300
    idat = np.array([nvis, 0, 0], np.int32)
    datm = np.zeros(nrep * 2 * nvis, np.float32)
    mcmc_interf.use_model("sgra")
    mcmc_interf.calcmodel(w.coor, idat, datm, P.reshape(nrep, 1, 9).copy(), 1, w.coor.size,
                          nvis, 3, datm.size, 9, nrep, 1)
    amp, ph = datm[:nrep * nvis].reshape(nrep, nvis), datm[nrep * nvis:].reshape(nrep, nvis)
    for r in range(nrep):
        a, p = oracle.sgra_vis(1, P[r], w.coor[0::2], w.coor[1::2])
        assert np.max(np.abs(amp[r] - a) - AMP_RTOL * a) <= AMP_ATOL * P[r, 0]
        assert np.all(np.abs(_wrap(ph[r] - p)) <= PHASE_ATOL + AMP_ATOL * P[r, 0] / a)


@pytest.mark.parametrize("w", [synth.rosenbrock(n=4), synth.solvsys(), synth.nlsys()],
                         ids=["rosenbrock", "solvsys", "nlsys"])
def test_calc_modchi2_plugins(w):
    mcmc_interf.use_model(w.model)
    rng = np.random.default_rng(5)
    nrep = 64
    P = rng.uniform(w.pmint, w.pmaxt, (nrep, w.nptot)).astype(np.float32)
    datm = np.zeros(nrep * w.ndat, np.float32)
    chi2m = np.zeros((nrep, 1, w.ndat), np.float32)
    chi2c = np.zeros((nrep, 1), np.float32)
    mcmc_interf.calcmodchi2(w.coor, w.dat, w.std2r, w.icoor, w.idat, datm, chi2m,
                            P.reshape(nrep, 1, -1).copy(), chi2c, np.ones((nrep, 1), np.int32),
                            0, w.coor.size, w.ndat, w.icoor.size, w.idat.size, datm.size,
                            w.nptot, nrep, 1)
    _, _, _, c2 = oracle.calc_modchi2(_pb(w), P)
    assert np.max(np.abs(chi2c.ravel() - c2) / np.maximum(c2, 1e-6)) < CHI2_RTOL


# ---------------------------------------------------------------------------
# the sweep
# ---------------------------------------------------------------------------

def _golden_job(model):
    g = golden("sweep_%s.npz" % model)
    job = DeviceJob(model, g["coor"], g["dat"], g["std2r"], g["icoor"], g["idat"], g["pdescr"],
                    g["pmint"], g["pmaxt"], g["beta"], int(g["nseq"]), int(g["niter"]),
                    imodel=int(g["imodel"]), npass=int(g["npass"]), ptotal=g["ptotal"],
                    pstp=g["pstp0"], rng="injected", streams=(g["u"], g["n"]))
    return g, job


@pytest.mark.parametrize("model", ["sgra", "rosenbrock", "solvsys"])
def test_sweep_matches_reference_decision_for_decision(model):
    """Injected streams: the fused kernel takes every accept / reject / swap
    decision of the reference's own kernels (golden fixtures)."""
    g, job = _golden_job(model)
    job.run(int(g["nburn"]), int(g["niter"]), do_init=True)
    job.check()
    s = job.to_numpy()
    for f in ("n_acpt", "n_exch", "n_cnt", "n_hist", "tcur", "tout", "flag", "ptentn"):
        assert np.array_equal(s[f], g[f]), f
    assert np.array_equal(s["inj_cur"][:, 0], g["cu"]) and np.array_equal(s["inj_cur"][:, 1], g["cn"])
    assert np.allclose(s["pcur"], g["pcur"], rtol=1e-5, atol=1e-6)
    assert np.allclose(s["pout"], g["pout"], rtol=1e-5, atol=1e-6)
    assert np.allclose(s["pstp"], g["pstp"], rtol=1e-6, atol=0)
    assert np.allclose(s["chi2"], g["chi2"], rtol=CHI2_RTOL, atol=1e-5)


def _oracle_state_from(job_state, w, niter_total):
    st = oracle.new_state(w.pdescr, w.pmint, w.pmaxt, w.beta(), w.nseq, niter_total,
                          ptotal=w.ptotal, ndat=w.ndat)
    for f in ("pcur", "flag", "ptent", "ptentn", "pstp", "n_acpt", "n_exch", "n_cnt", "n_hist",
              "tcur"):
        getattr(st, f)[...] = job_state[f]
    st.chi2c = job_state["chi2c"].astype(np.float64)
    return st


def _sgra_cpext(w, seed=12):
    """The workload's visibilities with its closures given as triangle
    corners (cpExt = 1): u1, v1, u2, v2 per closure, the third corner
    -(u1 + u2), -(v1 + v2)."""
    import dataclasses
    rng = np.random.default_rng(seed)
    nvis, ncph = int(w.idat[0]), w.ndat - int(w.idat[0])
    corners = rng.uniform(-6, 6, (ncph, 4)).astype(np.float32)
    return dataclasses.replace(
        w, coor=np.concatenate([w.coor[:2 * nvis], corners.ravel()]).astype(np.float32),
        dat=np.concatenate([w.dat[:nvis], rng.uniform(-3, 3, ncph)]).astype(np.float32),
        std2r=np.concatenate([w.std2r[:nvis], np.full(ncph, 100.0)]).astype(np.float32),
        icoor=np.zeros(1, np.int32), idat=np.array([nvis, 0, 1], np.int32))


def _lockstep(cases, run_one, nburn, niter, seed=77):
    """Lock-step harness.  ``cases`` = [(workload, job)] with injected-stream
    jobs whose state already holds the initialised replicas (do_init run);
    ``run_one(burn)`` runs one burn-in or main iteration of every job (one
    launch per job, or one batch launch).  Before each iteration the FP64
    oracle takes the kernel's state (and stream cursors), runs the same
    iteration with the same draws, and the outcomes are compared: identical
    decisions (acceptances, exchanges, step histories, temperatures, stream
    positions), chi^2 within 1e-5 and parameters within float rounding.
    An iteration that differs must contain a near tie in the oracle's trace
    (|u - alpha| < 1e-3); at most one such iteration is allowed."""
    mismatched = 0
    for step in range(nburn + niter):
        burn = step < nburn
        runs = []
        for w, job in cases:
            s = job.to_numpy()
            st = _oracle_state_from(s, w, job.niter_total)
            ors = oracle.Streams(job.streams[0], job.streams[1], s["inj_cur"][:, 0].copy(),
                                 s["inj_cur"][:, 1].copy())
            tr = oracle.sweep(_pb(w), st, ors, 0, 1 if burn else 0, 0 if burn else 1, trace=True)
            runs.append((st, ors, tr))
        run_one(burn)
        bad = False
        for (w, job), (st, ors, tr) in zip(cases, runs):
            job.check()
            s = job.to_numpy()
            same = (np.array_equal(s["n_acpt"], st.n_acpt) and np.array_equal(s["n_exch"], st.n_exch)
                    and np.array_equal(s["tcur"], st.tcur) and np.array_equal(s["n_hist"], st.n_hist)
                    and np.array_equal(s["inj_cur"][:, 0], ors.cu)
                    and np.array_equal(s["inj_cur"][:, 1], ors.cn))
            if same:
                assert np.allclose(s["pcur"], st.pcur, rtol=1e-6, atol=1e-7)
                assert np.max(np.abs(s["chi2c"] - st.chi2c) / np.maximum(st.chi2c, 1e-6)) < CHI2_RTOL
            else:
                # allowed only when the oracle saw a near tie in this iteration
                alpha_m = np.abs(tr.margin[tr.dec >= 0])
                x_m = np.abs(tr.xmargin)
                assert alpha_m.min(initial=1.0) < TIE_RTOL or x_m.min(initial=1.0) < TIE_RTOL
                bad = True
        mismatched += bad
    assert mismatched <= 1


def _injected_job(w, niter_total, seed=77, shape=None):
    nrep = w.nbeta * w.nseq
    rs = oracle.make_streams(nrep, 4000, 1000, seed)
    job = DeviceJob.from_workload(w, niter_total=niter_total, rng="injected", streams=(rs.u, rs.n))
    job.streams = (rs.u, rs.n)
    job.shape = shape
    return job


def _check_init(w, job):
    """The kernel's init_pcur + first chi^2 against the oracle's."""
    s = job.to_numpy()
    st = oracle.new_state(w.pdescr, w.pmint, w.pmaxt, w.beta(), w.nseq, job.niter_total,
                          ptotal=w.ptotal, ndat=w.ndat)
    if w.pstp0 is not None:
        st.pstp[:] = np.asarray(w.pstp0, np.float32)[:, None, None]
    oracle.sweep(_pb(w), st, oracle.Streams(*job.streams), 1, 0, 0)
    assert np.allclose(s["pcur"], st.pcur, rtol=1e-6, atol=1e-7)
    assert np.max(np.abs(s["chi2c"] - st.chi2c) / np.maximum(st.chi2c, 1e-6)) < CHI2_RTOL


@pytest.mark.parametrize("cfg", ["sgra", "sgra_cpext", "sgra_npass1", "sgra_nbeta64", "nlsys",
                                 "rosenbrock"])
def test_sweep_lockstep_vs_fp64_oracle(cfg):
    """Larger data than the fixtures: from the same state and the same
    injected draws, every iteration of the kernel makes the FP64 oracle's
    decisions (near ties excepted) and reaches its chi^2 within 1e-5.
    Sgr A* with closures from visibility triplets, from triangle corners
    (cpExt = 1), without the closure pass (npass = 1), and with 64
    temperatures (the exchange's shared-memory loop; up to 32 it runs on the
    lanes of one warp)."""
    import dataclasses
    if cfg == "sgra":
        w = synth.sgra(nvis=400, ncph=120, seed=8, nseq=2, nbeta=8)
    elif cfg == "sgra_nbeta64":
        w = synth.sgra(nvis=200, ncph=60, seed=8, nseq=1, nbeta=64)
    elif cfg == "sgra_cpext":
        w = _sgra_cpext(synth.sgra(nvis=400, ncph=120, seed=8, nseq=2, nbeta=8))
    elif cfg == "sgra_npass1":
        w = dataclasses.replace(synth.sgra(nvis=400, ncph=120, seed=8, nseq=2, nbeta=8), npass=1)
    elif cfg == "nlsys":
        w = synth.nlsys(nseq=2, nbeta=8)
    else:
        w = synth.rosenbrock(nseq=2, nbeta=8)
    nburn, niter = 6, 6
    job = _injected_job(w, niter)
    job.run(0, 0, do_init=True)
    job.check()
    _check_init(w, job)
    _lockstep([(w, job)], lambda burn: job.run(1 if burn else 0, 0 if burn else 1, itr0=0),
              nburn, niter)


# Launch shapes the benchmarks run, forced through cmc_set_config:
#   cfg3: 2000 vis + 600 closures at 32 temperatures as the 64 x 32 benchmark
#         runs it -- R = 8 replicas per CTA, clusters of G = 4 CTAs of 256
#         threads, phases in shared memory, the warp-parallel exchange reading
#         chi^2 from three remote CTAs and the parameter rows pulled across
#         the cluster;
#   cfg4: the 20000-visibility shape, R = 4, T = 256, phases in global memory
#         (3000 + 900 data: from 2048 points on the phases may live there);
#   r2g16: R = 2, the largest (non-portable) cluster, G = 16, unit phasors;
#   spread: the spread layout (cmc_set_layout 2), 64 replicas shared by
#         cooperative CTAs of 7 (10 CTAs: 7 7 7 7 6 6 6 6 6 6, the fifth
#         holding both sequences and running the second one's exchange) or of
#         3 (22 CTAs), the exchanges through global memory; with phases in
#         global memory, one region per CTA slot.
SHAPES = {
    "cfg3_R8_T256_smem": (dict(nvis=2000, ncph=600), dict(R=8, T=256, phasor=0)),
    "cfg4_R4_T256_global": (dict(nvis=3000, ncph=900), dict(R=4, T=256, phasor=2)),
    "r2_g16_phasors": (dict(nvis=2000, ncph=600), dict(R=2, T=64, phasor=1)),
    "spread_R7_T256_smem": (dict(nvis=2000, ncph=600), dict(R=7, T=256, phasor=0, layout=2)),
    "spread_R3_T128_phasors": (dict(nvis=2000, ncph=600), dict(R=3, T=128, phasor=1, layout=2)),
    "spread_R7_T256_global": (dict(nvis=3000, ncph=900), dict(R=7, T=256, phasor=2, layout=2)),
}


@pytest.mark.parametrize("name", list(SHAPES))
def test_sweep_lockstep_benchmark_shapes(name):
    """The benchmarked launch shapes (32 temperatures, 2 sequences, 4 + 4
    iterations) make the FP64 oracle's decisions iteration by iteration."""
    sizes, shape = SHAPES[name]
    w = synth.sgra(seed=8, nseq=2, nbeta=32, **sizes)
    job = _injected_job(w, 4, shape=shape)
    cfg = job.config()
    assert (cfg["R"], cfg["T"], cfg["phasor"]) == (shape["R"], shape["T"], shape["phasor"])
    if shape.get("layout") == 2:
        assert cfg["layout"] == "spread" and cfg["blocks"] == -(-64 // shape["R"])
    else:
        assert cfg["G"] == 32 // shape["R"]
    job.run(0, 0, do_init=True)
    job.check()
    _check_init(w, job)
    _lockstep([(w, job)], lambda burn: job.run(1 if burn else 0, 0 if burn else 1, itr0=0), 4, 4)


def test_batch_lockstep_autotuned_classes():
    """Batched fits at their size classes' autotuned launch shapes make the
    FP64 oracle's decisions, fit by fit, iteration by iteration."""
    sizes = [(300, 90), (2600, 780), (5200, 1560)]
    fits = [synth.sgra(nvis=nv, ncph=nc, seed=60 + i, nseq=2, nbeta=16)
            for i, (nv, nc) in enumerate(sizes)]
    jobs = [_injected_job(w, 3, seed=90 + i) for i, w in enumerate(fits)]
    batch = BatchJob(jobs)
    batch.autotune(iters=1)
    for j in jobs:                   # the trials advanced the stream cursors
        j.t["inj_cur"].zero_()
    batch.run(0, 0, do_init=True)
    batch.check()
    for w, j in zip(fits, jobs):
        _check_init(w, j)
    _lockstep(list(zip(fits, jobs)),
              lambda burn: batch.run(1 if burn else 0, 0 if burn else 1, itr0=0), 3, 3)


def test_mcmc_cuda_host_abi_equals_device_api():
    """mcmc_interf.mcmcuda (host buffers, the reference's call) and a
    device-resident job with the same seed produce identical outputs."""
    w = synth.sgra(nvis=300, ncph=90, seed=12, nseq=4, nbeta=8, nburn=20, niter=30)
    seed = 99
    job = DeviceJob.from_workload(w, seed=seed)
    job.run(w.nburn, w.niter, do_init=True)
    job.check()
    dev = job.to_numpy()
    from cuda_mcmc_gb300.device import sampler_defaults
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
                        s["pcur"], rndst, np.uint64(seed), w.imodel, w.coor.size, w.ndat,
                        w.icoor.size, w.idat.size, datm.size, w.nptot, nprm, 100, w.npass,
                        w.nbeta, w.nseq, w.nburn, w.niter)
    assert np.array_equal(pout, dev["pout"])
    assert np.array_equal(tout, dev["tout"])
    assert np.array_equal(chi2, dev["chi2"])
    assert np.array_equal(rndst, dev["rndst"])
    for f in ("pcur", "chi2c", "pstp", "n_acpt", "n_exch", "n_cnt", "n_hist", "tcur"):
        assert np.array_equal(s[f], dev[f]), f
    assert np.array_equal(datm, dev["datm"]) and np.array_equal(chi2m, dev["chi2m"])


def _host_call(w, seed, rndst):
    from cuda_mcmc_gb300.device import sampler_defaults
    s = sampler_defaults(w.pdescr, w.pmint, w.pmaxt, w.nbeta, w.nseq)
    nrep, nprm = w.nbeta * w.nseq, w.nprm
    out = dict(pout=np.zeros((nprm, w.nbeta, w.nseq, w.niter), np.float32),
               tout=np.zeros((w.nbeta, w.nseq, w.niter), np.int32),
               chi2=np.zeros((w.nseq, w.niter), np.float32),
               datm=np.zeros(nrep * (w.ndat + w.nvis), np.float32),
               chi2m=np.zeros((w.nbeta, w.nseq, w.ndat), np.float32), rndst=rndst)
    mcmc_interf.use_model("sgra")
    mcmc_interf.mcmcuda(w.coor, w.dat, w.std2r, w.icoor, w.idat, out["datm"], out["chi2m"],
                        s["pdescr"], s["ivar"], s["invar"], s["ptotal"], s["pmint"], s["pmaxt"],
                        out["pout"], out["tout"], out["chi2"], s["chi2c"], s["tcur"], s["flag"],
                        s["n_acpt"], s["n_exch"], s["n_cnt"], s["n_hist"], w.beta(), s["pstp"],
                        s["ptent"], s["ptentn"], s["pcur"], rndst, np.uint64(seed), w.imodel,
                        w.coor.size, w.ndat, w.icoor.size, w.idat.size, out["datm"].size,
                        w.nptot, nprm, 100, w.npass, w.nbeta, w.nseq, w.nburn, w.niter)
    out.update(s)
    return out


def test_mcmc_cuda_generator_states_are_the_callers_array():
    """rndst goes to the device and back as in the reference
    (src/mcmcjob.cu:724, 765): curand_init rewrites each 48-byte XORWOW
    state's fields in place and leaves its 4 padding bytes (36-39) as the
    caller's.  The output does not depend on what an earlier call left in
    the library's device memory pool (an unrelated 64 x 32 call in between)."""
    w = synth.sgra(nvis=2000, ncph=600, seed=3, nseq=4, nbeta=8, nburn=6, niter=6)
    a = _host_call(w, 4242, np.zeros((w.nbeta, w.nseq, 48), np.uint8))
    big = synth.sgra(nvis=2000, ncph=600, seed=3, nseq=64, nbeta=32, nburn=1, niter=2)
    _host_call(big, 11, np.full((big.nbeta, big.nseq, 48), 0x5C, np.uint8))
    b = _host_call(w, 4242, np.full((w.nbeta, w.nseq, 48), 0xAB, np.uint8))
    assert np.all(b["rndst"][..., 36:40] == 0xAB) and np.all(a["rndst"][..., 36:40] == 0)
    assert np.array_equal(a["rndst"][..., :36], b["rndst"][..., :36])
    assert np.array_equal(a["rndst"][..., 40:], b["rndst"][..., 40:])
    for f in ("pout", "tout", "chi2", "datm", "chi2m", "pcur", "chi2c", "n_acpt", "n_exch",
              "n_cnt", "n_hist", "tcur", "pstp", "flag"):
        assert np.array_equal(a[f], b[f]), f


def test_chunked_run_equals_single_launch():
    w = synth.nlsys(nseq=4, nbeta=8)
    a = DeviceJob.from_workload(w, niter_total=40, seed=5)
    a.run(30, 40, do_init=True)
    b = DeviceJob.from_workload(w, niter_total=40, seed=5)
    b.run(10, 0, do_init=True)
    b.run(20, 15)
    b.run(0, 25)
    a.check()
    b.check()
    sa, sb = a.to_numpy(), b.to_numpy()
    for f in ("pout", "tout", "chi2", "pcur", "chi2c", "rndst", "n_acpt", "n_hist", "pstp"):
        assert np.array_equal(sa[f], sb[f]), f


def test_chi2_trace_is_fp64_chi2_of_recorded_samples():
    """Size-independent property at the benchmark's data size: every recorded
    chi2[iseq, itr] is the chi^2 of the recorded coldest-slot sample."""
    w = synth.sgra(nvis=2000, ncph=600, seed=3, nseq=8, nbeta=32, nburn=30, niter=40)
    job = DeviceJob.from_workload(w, seed=2)
    job.run(w.nburn, w.niter, do_init=True)
    job.check()
    s = job.to_numpy()
    idx = [(q, it) for q in range(w.nseq) for it in range(0, w.niter, 13)]
    P = np.stack([s["pout"][:, 0, q, it] for (q, it) in idx]).astype(np.float32)
    _, _, _, c2 = oracle.calc_modchi2(_pb(w), P)
    c2g = np.array([s["chi2"][q, it] for (q, it) in idx])
    assert np.max(np.abs(c2g - c2) / c2) < CHI2_RTOL
    # every tcur column is a permutation of 0..nbeta-1
    assert all(sorted(s["tcur"][:, q]) == list(range(w.nbeta)) for q in range(w.nseq))
    # each burn-in proposal counts one trial: sum_k n_cnt = nprm + nburn*nprm
    assert np.all(s["n_cnt"].sum(0) == w.nprm * (1 + w.nburn))


def test_known_answers_solvsys_and_rosenbrock():
    w = synth.solvsys(nseq=14, nbeta=32, nburn=400, niter=5000)   # solvsys.py:38-40
    job = DeviceJob.from_workload(w, seed=1)
    job.run(w.nburn, w.niter, do_init=True)
    job.check()
    s = job.to_numpy()
    chi2, pout = s["chi2"].ravel(), s["pout"][:, 0].reshape(2, -1)
    rx = np.array([(-4.0 - np.sqrt(832.0)) / 34.0, (-4.0 + np.sqrt(832.0)) / 34.0])
    best = pout[:, chi2 < 2e-4]
    assert best.shape[1] > 0
    d = np.min(np.abs(best[0][:, None] - rx[None, :]), axis=1)
    assert np.all(d < 0.05)
    # every hit sits on one of the two roots (a coldest chain need not visit both)
    found = {int(np.argmin(np.abs(x - rx))) for x in best[0]}
    assert found and found <= {0, 1}
    w = synth.rosenbrock(n=4, nseq=16, nbeta=32, nburn=1000, niter=5000)
    job = DeviceJob.from_workload(w, seed=2)
    job.run(w.nburn, w.niter, do_init=True)
    job.check()
    s = job.to_numpy()
    i = np.argmin(s["chi2"])
    xbest = s["pout"][:, 0].reshape(4, -1)[:, i]
    assert np.all(np.abs(xbest - 1.0) < 0.1)


def test_errors_are_reported_not_faults():
    w = synth.sgra(nvis=50, ncph=10, seed=1, nseq=1, nbeta=2, nburn=1, niter=1)
    bad = w.icoor.copy()
    bad[0] = 10 ** 6                        # closure index out of range
    job = DeviceJob("sgra", w.coor, w.dat, w.std2r, bad, w.idat, w.pdescr, w.pmint, w.pmaxt,
                    w.beta(), 1, 1, imodel=1, npass=2)
    job.run(1, 1, do_init=True)
    with pytest.raises(_lib.McmcError):
        job.check()
    job2 = DeviceJob.from_workload(w)
    job2.job.imodel = 7
    with pytest.raises(_lib.McmcError, match="imodel"):
        job2.run(1, 1, do_init=True)
    job3 = DeviceJob.from_workload(w)
    job3.job.nbeta = 1
    with pytest.raises(_lib.McmcError, match="nbeta"):
        job3.run(1, 1, do_init=True)


def test_global_memory_phases_equal_shared_memory_phases():
    """Phase storage mode 2 (per-replica phases in global memory, for large
    data sets) stores the same float phases as mode 0 (shared memory): a
    run in each mode with the same R and T gives bit-identical results."""
    w = synth.sgra(nvis=3000, ncph=900, seed=31, nseq=4, nbeta=8)
    out = []
    for ph in (0, 2):
        job = DeviceJob.from_workload(w, niter_total=6, seed=5)
        job.shape = {"R": 4, "T": 128, "phasor": ph}
        assert job.config()["phasor"] == ph
        job.run(4, 0, do_init=True)
        job.run(0, 6)
        job.check()
        out.append(job.to_numpy())
    for k in ("pout", "tout", "chi2", "pcur", "chi2c", "pstp", "n_acpt", "n_exch", "rndst",
              "datm", "chi2m"):
        assert np.array_equal(out[0][k], out[1][k]), k


def test_calc_modchi2_beyond_shared_memory_uses_global_phases():
    """60,000 visibilities: one replica's phases (240 KB) exceed shared
    memory; with cmc_work_bytes() of scratch the evaluation keeps them in
    global memory and matches the FP64 oracle."""
    w = synth.sgra(nvis=60000, ncph=2000, seed=32, nseq=1, nbeta=2)
    job = DeviceJob.from_workload(w, niter_total=1, seed=5)
    P = np.stack([w.truth, w.truth * np.float32(1.02)])[:, None, :].astype(np.float32)
    job.set_state(pcur=P, flag=np.ones((2, 1), np.int32))
    job.eval()
    job.check()
    s = job.to_numpy(("chi2c",))
    _, _, _, c64 = oracle.calc_modchi2(_pb(w), P.reshape(2, -1))
    assert np.max(np.abs(s["chi2c"].ravel() - c64) / c64) < CHI2_RTOL
