"""Parity with the reference's own CUDA build, in the production generator mode.

The reference's src/gpu_mcmc.cu (unchanged, with
examples/sgra_model_fit/model.cuh) is compiled for sm_103a by
oracle/ref_build.py and run on the same GPU by oracle/ref_gpu.py, which
launches its kernels in run_mcmc's order (src/gpu_mcmc.cu:682-763).  Both
sides draw from cuRAND XORWOW generators seeded by curand_init(seed, ist, 0)
(:228-239), so with the same seed the library must walk the reference's
chains: the same draws in the same order (the k redraw, Box-Muller normals,
the exchange drawing from the ibeta = 0 generator, :361-411, :426-474,
:533-626), hence identical generator states, counters, temperatures and
decisions, with chi^2 and parameters equal to float32 rounding.

Tolerances: chi^2 relative 1e-5 (both are float32 sums of 2600 float32
terms); parameters 1e-6 relative + 1e-7; a decision may differ only where
it is a near tie: where the reference's own uniform u lies so close to its
acceptance probability alpha = min(1, e^x) that chi^2 values within the 1e-5
tolerance can move it across, |ln u - x| <= beta/2 * 1e-5 * (chi2_new +
chi2_cur), or within the 1e-3 of the other lock-step tests.  That is checked
by re-running the iteration of the reference kernel by kernel and reading
each decision's u and chi^2 values.
"""
import numpy as np
import pytest

from cuda_mcmc_gb300 import mcmc_interf, synth
from cuda_mcmc_gb300.device import DeviceJob, sampler_defaults

pytestmark = pytest.mark.gpu

ref_gpu = pytest.importorskip("oracle.ref_gpu")
if not ref_gpu.available("sgra"):
    pytest.skip("the reference's CUDA build is not present (oracle/ref_build.py "
                "builds it where the reference tree is)", allow_module_level=True)

CHI2_RTOL, TIE_RTOL = 1e-5, 1e-3
STATE = ("pcur", "chi2c", "flag", "ptent", "ptentn", "pstp", "n_acpt", "n_exch", "n_cnt",
         "n_hist", "tcur", "rndst")
EXACT = ("n_acpt", "n_exch", "n_cnt", "n_hist", "tcur", "pstp", "flag", "ptentn", "rndst")


def _ref_job(w, niter, seed, nburn=0):
    st = sampler_defaults(w.pdescr, w.pmint, w.pmaxt, w.nbeta, w.nseq, ptotal=w.ptotal,
                          pstp=w.pstp0)
    return ref_gpu.RefGpuJob("sgra", w.coor, w.dat, w.std2r, w.icoor, w.idat, w.beta(), st,
                             w.nseq, niter, seed, imodel=w.imodel, npass=w.npass, nburn=nburn)


def _seq(a, f, q):
    return a[f][:, q] if f in ("n_exch", "tcur", "flag", "ptentn", "rndst") else a[f][..., q]


def test_init_matches_reference_cuda_build():
    """init_rng + init_pcur + the first chi^2: identical generator states,
    the same prior draws, chi^2 to float32 accuracy."""
    w = synth.sgra(nvis=2000, ncph=600, seed=3, nseq=4, nbeta=32)
    ref = _ref_job(w, 1, seed=77)
    ref.init()
    r = ref.to_numpy()
    job = DeviceJob.from_workload(w, niter_total=1, seed=77)
    job.run(0, 0, do_init=True)
    job.check()
    s = job.to_numpy()
    assert np.array_equal(r["rndst"], s["rndst"])
    assert np.allclose(r["pcur"], s["pcur"], rtol=1e-6, atol=1e-7)
    assert np.max(np.abs(r["chi2c"] - s["chi2c"]) / r["chi2c"]) < CHI2_RTOL


CASES = {
    # 8 temperatures: one CTA per sequence
    "2000vis_4x8": (dict(nseq=4, nbeta=8), None, 6, 6),
    # 32 temperatures at the 64 x 32 benchmark's launch shape (R = 8, G = 4,
    # T = 256, phases in shared memory: the warp-parallel exchange over DSMEM)
    "2000vis_2x32_R8_G4": (dict(nseq=2, nbeta=32), dict(R=8, T=256, phasor=0), 4, 4),
    # the library's own choice at 32 temperatures
    "2000vis_4x32": (dict(nseq=4, nbeta=32), None, 3, 3),
    # the spread layout: 128 replicas in 19 cooperative CTAs of 6-7, CTAs
    # spanning two sequences, the exchanges through global memory
    "2000vis_4x32_spread_R7": (dict(nseq=4, nbeta=32), dict(R=7, T=256, phasor=0, layout=2), 3, 3),
}


@pytest.mark.parametrize("name", list(CASES))
def test_curand_lockstep_vs_reference_cuda_build(name):
    """Iteration by iteration from the reference's state (generator states
    included): the library's sweep makes the reference kernels' decisions and
    leaves identical generator states, counters and temperatures."""
    dims, shape, nburn, niter = CASES[name]
    w = synth.sgra(nvis=2000, ncph=600, seed=3, **dims)
    seed = 4242
    ref = _ref_job(w, niter, seed, nburn)
    ref.init()
    job = DeviceJob.from_workload(w, niter_total=niter, seed=seed)
    job.shape = shape
    if shape:
        c = job.config()
        assert (c["R"], c["T"], c["phasor"]) == (shape["R"], shape["T"], shape["phasor"])
    mismatched = 0
    for step in range(nburn + niter):
        burn = step < nburn
        itr = step if burn else step - nburn
        pre = ref.to_numpy(STATE)
        job.set_state(**pre)
        ref.iteration(burn, itr)
        job.run(1 if burn else 0, 0 if burn else 1, itr0=itr)
        job.check()
        r, s = ref.to_numpy(), job.to_numpy()
        bad = [q for q in range(w.nseq)
               if not all(np.array_equal(_seq(r, f, q), _seq(s, f, q)) for f in EXACT)]
        good = [q for q in range(w.nseq) if q not in bad]
        if good:
            assert np.allclose(r["pcur"][:, good], s["pcur"][:, good], rtol=1e-6, atol=1e-7)
            c2r, c2s = r["chi2c"][:, good], s["chi2c"][:, good]
            assert np.max(np.abs(c2r - c2s) / c2r) < CHI2_RTOL
            if not burn:
                assert np.array_equal(r["tout"][:, good, itr], s["tout"][:, good, itr])
                assert np.allclose(r["pout"][:, :, good, itr], s["pout"][:, :, good, itr],
                                   rtol=1e-6, atol=1e-7)
                c2r, c2s = r["chi2"][good, itr], s["chi2"][good, itr]
                assert np.max(np.abs(c2r - c2s) / c2r) < CHI2_RTOL
        if bad:
            # every differing sequence must hold a near tie of the reference
            ref.set_state(**pre)
            margin = ref.iteration_trace(burn, itr, chi2_rtol=CHI2_RTOL, floor=TIE_RTOL)
            for q in bad:
                assert margin[q] <= 1.0, "sequence %d differs without a near tie" % q
            mismatched += len(bad)
    # near ties are rare: a small share of the sequence-iterations at most
    assert mismatched <= max(2, w.nseq * (nburn + niter) // 8)


def test_mcmc_cuda_equals_reference_mcmc_cuda_run():
    """The drop-in entry point itself: mcmc_cuda with host buffers (the
    reference's call, src/mcmcjob.cu:475-545) against the reference's
    run_mcmc on the same inputs and seed -- every output of a whole run."""
    w = synth.sgra(nvis=2000, ncph=600, seed=3, nseq=4, nbeta=8, nburn=6, niter=6)
    seed = 4242
    ref = _ref_job(w, w.niter, seed, w.nburn)
    ref.run(w.nburn, w.niter)
    r = ref.to_numpy()
    s = sampler_defaults(w.pdescr, w.pmint, w.pmaxt, w.nbeta, w.nseq, ptotal=w.ptotal,
                         pstp=w.pstp0)
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
    assert np.array_equal(rndst, r["rndst"])
    assert np.array_equal(tout, r["tout"])
    for f in ("n_acpt", "n_exch", "n_cnt", "n_hist", "tcur", "pstp", "ptentn"):
        assert np.array_equal(s[f], r[f]), f
    assert np.allclose(pout, r["pout"], rtol=1e-6, atol=1e-7)
    assert np.allclose(s["pcur"], r["pcur"], rtol=1e-6, atol=1e-7)
    assert np.max(np.abs(chi2 - r["chi2"]) / r["chi2"]) < CHI2_RTOL
    assert np.max(np.abs(s["chi2c"] - r["chi2c"]) / r["chi2c"]) < CHI2_RTOL


def test_calc_modchi2_vs_reference_cuda_build():
    """run_calcmodchi2 of the reference (float32 j0f/j1f/jnf model) and the
    library's calc_modchi2 on the same parameter sets."""
    w = synth.sgra(nvis=2000, ncph=600, seed=3, nseq=8, nbeta=8)
    rng = np.random.default_rng(11)
    P = rng.uniform(synth.SGRA9_PMIN, synth.SGRA9_PMAX, (w.nbeta, w.nseq, 9)).astype(np.float32)
    ref = _ref_job(w, 1, seed=1)
    ref.set_state(pcur=P, flag=np.ones((w.nbeta, w.nseq), np.int32))
    ref.calc_modchi2()
    r = ref.to_numpy(("chi2c", "datm"))
    nrep, nvis, ndat = w.nbeta * w.nseq, w.nvis, w.ndat
    datm = np.zeros(nrep * (ndat + nvis), np.float32)
    chi2m = np.zeros((w.nbeta, w.nseq, ndat), np.float32)
    chi2c = np.zeros((w.nbeta, w.nseq), np.float32)
    mcmc_interf.use_model("sgra")
    mcmc_interf.calcmodchi2(w.coor, w.dat, w.std2r, w.icoor, w.idat, datm, chi2m, P.copy(),
                            chi2c, np.ones((w.nbeta, w.nseq), np.int32), 1, w.coor.size, ndat,
                            w.icoor.size, w.idat.size, datm.size, 9, w.nbeta, w.nseq)
    assert np.max(np.abs(chi2c - r["chi2c"]) / r["chi2c"]) < CHI2_RTOL
    amp_r = r["datm"][:nrep * ndat].reshape(nrep, ndat)[:, :nvis]
    amp_s = datm[:nrep * ndat].reshape(nrep, ndat)[:, :nvis]
    zsp = P.reshape(nrep, 9)[:, :1]
    assert np.all(np.abs(amp_s - amp_r) <= 2e-5 * np.abs(amp_r) + 2e-6 * zsp)
