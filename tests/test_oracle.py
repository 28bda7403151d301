"""Pin the CPU oracle (oracle/oracle.c) against the reference's own code.

The golden fixtures were produced by the reference's kernels and model.cuh
files compiled for the CPU (tests/golden/make_golden.py).  The reference
computes in float32 (with glibc's double Bessel functions on the host), the
oracle in float64, so model values agree to float32 accuracy and every
accept / reject / swap decision of the injected-stream sweeps agrees exactly.
"""
import numpy as np
import pytest

import oracle
from conftest import golden
from cuda_mcmc_gb300 import synth

MODCHI2 = ["sgra_modchi2_m9.npz", "sgra_modchi2_m13.npz", "sgra_modchi2_cpext.npz"]


def _wrap(x):
    return np.angle(np.exp(1j * x))


@pytest.mark.parametrize("name", MODCHI2)
def test_oracle_model_matches_reference(name):
    g = golden(name)
    P = g["pcur"]
    nrep, nvis, ndat = P.shape[0], int(g["idat"][0]), g["dat"].size
    pb = oracle.Problem("sgra", g["coor"], g["dat"], g["std2r"], g["icoor"], g["idat"],
                        P.shape[1], int(g["imodel"]), 2)
    d, ph, c2m, c2 = oracle.calc_modchi2(pb, P)
    rd = g["datm"][:nrep * ndat].reshape(nrep, ndat)
    rph = g["datm"][nrep * ndat:].reshape(nrep, nvis)
    zsp = P[:, :1]
    # float32 model vs float64: relative 5e-5 (amplitudes below 1e-3 Zsp
    # are compared absolutely at that scale: the reference's float sums of
    # O(Zsp) ring terms carry ~1e-7 Zsp of rounding)
    amp_err = np.abs(rd[:, :nvis] - d[:, :nvis]) / np.maximum(np.abs(d[:, :nvis]), 1e-3 * zsp)
    assert amp_err.max() < 5e-5
    assert np.abs(_wrap(rph - ph)).max() < 5e-5
    assert np.abs(_wrap(rd[:, nvis:] - d[:, nvis:])).max() < 5e-5
    assert np.max(np.abs(g["chi2c"] - c2) / c2) < 2e-6
    assert np.max(np.abs(g["chi2m"] - c2m) / np.maximum(c2m, 1.0)) < 1e-3


def test_oracle_sgra9_matches_numpy_xringaus():
    """sgra_model9 against an independent FP64 NumPy/SciPy restatement of
    xringaus (src/obsdatafit.py:1476-1608) used by the data generator."""
    rng = np.random.default_rng(0)
    u, v = rng.uniform(-9, 9, 500), rng.uniform(-9, 9, 500)
    for _ in range(5):
        prm = synth.sgra_truth(rng)
        a1, p1 = synth._sgra9_vis_np(prm, u, v)
        a2, p2 = oracle.sgra_vis(1, prm, u, v)
        assert np.max(np.abs(a1 - a2)) < 1e-12 * max(1.0, a2.max())
        assert np.max(np.abs(_wrap(p1 - p2))) < 1e-9


@pytest.mark.parametrize("model", ["sgra", "rosenbrock", "solvsys"])
def test_oracle_sweep_matches_reference(model):
    g = golden("sweep_%s.npz" % model)
    nseq, nburn, niter = int(g["nseq"]), int(g["nburn"]), int(g["niter"])
    nptot = g["pdescr"].size
    pb = oracle.Problem(model, g["coor"], g["dat"], g["std2r"], g["icoor"], g["idat"], nptot,
                        int(g["imodel"]), int(g["npass"]))
    st = oracle.new_state(g["pdescr"], g["pmint"], g["pmaxt"], g["beta"], nseq, niter,
                          ptotal=g["ptotal"], ndat=g["dat"].size)
    st.pstp[:] = g["pstp0"]
    rs = oracle.Streams(g["u"], g["n"])
    oracle.sweep(pb, st, rs, 1, nburn, niter)
    for f in ("n_acpt", "n_exch", "n_cnt", "n_hist", "tcur", "tout", "flag", "ptentn"):
        assert np.array_equal(getattr(st, f), g[f]), f
    assert np.array_equal(rs.cu, g["cu"]) and np.array_equal(rs.cn, g["cn"])
    assert np.allclose(st.pcur, g["pcur"], rtol=1e-5, atol=1e-6)
    assert np.allclose(st.pout, g["pout"], rtol=1e-5, atol=1e-6)
    assert np.allclose(st.pstp, g["pstp"], rtol=1e-6, atol=0)
    assert np.allclose(st.chi2, g["chi2"], rtol=1e-4, atol=1e-5)


def test_known_answers():
    """The examples' closed-form answers: solvsys roots
    (examples/solvsys/solvsys.py:59-62) and the Rosenbrock minimum."""
    w = synth.solvsys()
    pb = oracle.Problem("solvsys", w.coor, w.dat, w.std2r, w.icoor, w.idat, 2)
    rx1 = (-4.0 - np.sqrt(832.0)) / 34.0
    rx2 = (-4.0 + np.sqrt(832.0)) / 34.0
    roots = np.array([[rx1, np.sqrt(1 - rx1 ** 2)], [rx2, np.sqrt(1 - rx2 ** 2)]], np.float32)
    _, _, _, c2 = oracle.calc_modchi2(pb, roots)
    assert np.all(c2 < 1e-12)
    w = synth.rosenbrock(n=4)
    pb = oracle.Problem("rosenbrock", w.coor, w.dat, w.std2r, w.icoor, w.idat, 4)
    _, _, _, c2 = oracle.calc_modchi2(pb, np.ones((1, 4), np.float32))
    assert c2[0] == 0.0


def test_injected_stream_exhaustion_is_reported():
    w = synth.solvsys(nseq=1, nbeta=2)
    pb = oracle.Problem("solvsys", w.coor, w.dat, w.std2r, w.icoor, w.idat, 2)
    st = oracle.new_state(w.pdescr, w.pmint, w.pmaxt, w.beta(), 1, 5, ndat=2)
    rs = oracle.make_streams(2, 6, 2, 1)
    with pytest.raises(RuntimeError, match="exhausted"):
        oracle.sweep(pb, st, rs, 1, 5, 5)


@pytest.mark.parametrize("name", ["sgra_modchi2_m9.npz", "sgra_modchi2_cpext.npz"])
def test_float32_port_matches_reference_chi2(name):
    """The float32 arithmetic of the CPU baseline (oracle.c OR_ARITH_F32)
    gives the reference's own float chi^2 (golden fixtures) and the FP64
    chi^2 to float32 accuracy."""
    g = golden(name)
    P = g["pcur"]
    pb = oracle.Problem("sgra", g["coor"], g["dat"], g["std2r"], g["icoor"], g["idat"],
                        P.shape[1], int(g["imodel"]), 2, arith=1)
    c32 = oracle.chi2_f32(pb, P)
    assert np.max(np.abs(c32 - g["chi2c"]) / g["chi2c"]) < 1e-5
    _, _, _, c64 = oracle.calc_modchi2(pb, P)
    assert np.max(np.abs(c32 - c64) / c64) < 1e-5


def test_float32_sweep_makes_the_fp64_decisions():
    """The CPU baseline's sweep (float32 model) takes the FP64 checker's
    decisions on the same injected streams."""
    w = synth.sgra(nvis=300, ncph=90, seed=4, nseq=2, nbeta=8)
    out = []
    for arith in (0, 1):
        pb = oracle.Problem(w.model, w.coor, w.dat, w.std2r, w.icoor, w.idat, w.nptot,
                            w.imodel, w.npass, arith=arith)
        st = oracle.new_state(w.pdescr, w.pmint, w.pmaxt, w.beta(), w.nseq, 4,
                              ptotal=w.ptotal, ndat=w.ndat)
        oracle.sweep(pb, st, oracle.make_streams(16, 2000, 500, 3), 1, 4, 4)
        out.append(st)
    for f in ("n_acpt", "n_exch", "tcur", "n_hist"):
        assert np.array_equal(getattr(out[0], f), getattr(out[1], f)), f
    assert np.max(np.abs(out[0].chi2c - out[1].chi2c) / out[0].chi2c) < 1e-5
