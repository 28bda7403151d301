"""The high-level Python API (imgpu) and its data helpers.

CPU: uv-file parsing, closure building, the reference's defaults in the
Mcgpu state.  GPU: the examples' compute sections through Mcgpu /
Mcgpu_Sgra, checked against the FP64 oracle.
"""
import glob
import os

import numpy as np
import pytest

import itertools

import oracle
from cuda_mcmc_gb300 import imgpu, synth
from oracle.ref_build import REF_ROOT

REF_UV = sorted(glob.glob(os.path.join(REF_ROOT, "examples", "sgra_model_fit", "*_uvdata.txt")))


def _closures_loop(phase, tsec, blin):
    """The reference's triangle loop (src/imgpu.py:1229-1325) restated
    literally: per equal-time span, every combination of its sorted
    antennas, each baseline's first row found by search."""
    ibeg, iend = imgpu.get_time_indices(tsec)
    cphs, cpix, trid, tcp = [], [], [], []
    bls = np.asarray(blin)
    for i0, i1 in zip(ibeg, iend):
        bl = bls[i0:i1].astype(int)
        ant = np.unique(bl)
        for a1, a2, a3 in (ant[list(t)] for t in itertools.combinations(range(ant.size), 3)):
            ib1 = i0 + int(np.where((bl[:, 0] == a1) & (bl[:, 1] == a2))[0][0])
            ib2 = i0 + int(np.where((bl[:, 0] == a1) & (bl[:, 1] == a3))[0][0])
            ib3 = i0 + int(np.where((bl[:, 0] == a2) & (bl[:, 1] == a3))[0][0])
            ph = phase[ib1] + phase[ib2] - phase[ib3]
            cphs.append(np.arctan2(np.sin(ph), np.cos(ph)))
            cpix.append((ib1, ib2, ib3))
            trid.append(a1 + imgpu.PK3I * (a2 + imgpu.PK3I * a3))
            tcp.append(tsec[i0])
    return (np.array(cphs, np.float32), np.array(cpix, np.int32).reshape(-1, 3),
            np.array(trid, np.int32), np.array(tcp, float))


def _wrap(x):
    return np.angle(np.exp(1j * x))


def test_read_uvdata_roundtrip(tmp_path):
    f = str(tmp_path / "obs_uvdata.txt")
    truth, uv = synth.write_uvdata(f, nant=5, ntimes=6)
    ulam, vlam, wlam, amp, phase, blin, tsec, sig, chan, wei = imgpu.read_uvdata(f)
    assert ulam.size == uv.shape[0] == 6 * 10
    # file in kilolambda -> megalambda here; the Sgr A* class scales to Glambda
    assert np.allclose(1e-3 * ulam, uv[:, 0], atol=1e-5)
    assert np.allclose(1e-3 * vlam, uv[:, 1], atol=1e-5)
    assert np.all(np.abs(phase) <= np.pi + 1e-6)
    assert blin.shape == (60, 2) and blin.min() == 1 and blin.max() == 5
    assert len(set(tsec.tolist())) == 6
    assert np.all(sig > 0)


def test_calc_closures_triangles(tmp_path):
    f = str(tmp_path / "obs_uvdata.txt")
    synth.write_uvdata(f, nant=5, ntimes=4)
    _, _, _, amp, phase, blin, tsec, _, _, _ = imgpu.read_uvdata(f)
    cphs, cpix, trid, tcp = imgpu.calc_closures(phase, tsec, blin)
    assert cphs.size == 4 * imgpu.cbinom(5, 3)
    ref = phase[cpix[:, 0]] + phase[cpix[:, 1]] - phase[cpix[:, 2]]
    assert np.allclose(_wrap(cphs - ref), 0, atol=1e-6)
    # triangle (a1, a2, a3): rows are baselines a1-a2, a1-a3, a2-a3
    assert np.all(blin[cpix[:, 0], 0] == blin[cpix[:, 1], 0])
    assert np.all(blin[cpix[:, 0], 1] == blin[cpix[:, 2], 0])
    assert np.all(blin[cpix[:, 1], 1] == blin[cpix[:, 2], 1])


def test_calc_closures_matches_the_reference_loop():
    """Spans with different antenna sets, a repeated baseline row (the first
    one counts), spans under 3 rows (skipped) and unsorted baselines."""
    rng = np.random.default_rng(4)
    rows_b, rows_t = [], []
    for it, ants in enumerate([(1, 2, 3, 4, 5), (2, 3, 5, 7), (1, 3), (1, 2, 4, 6, 8, 9)]):
        bl = [(a, b) for a, b in itertools.combinations(ants, 2)]
        rng.shuffle(bl)
        if it == 0:
            bl.append(bl[0])                      # repeated baseline: first row wins
        rows_b += bl
        rows_t += [1000.0 + 60 * it] * len(bl)
    blin = np.array(rows_b, np.int32)
    tsec = np.array(rows_t, np.float32)
    phase = rng.uniform(-np.pi, np.pi, len(rows_b)).astype(np.float32)
    got = imgpu.calc_closures(phase, tsec, blin)
    ref = _closures_loop(phase, tsec, blin)
    assert got[0].size == imgpu.cbinom(5, 3) + imgpu.cbinom(4, 3) + imgpu.cbinom(6, 3)
    for g, r in zip(got[1:], ref[1:]):
        assert np.array_equal(g, r)
    assert np.allclose(_wrap(got[0] - ref[0]), 0, atol=2e-6)
    # a triangle whose baseline is missing fails as the reference's loop does
    keep = np.arange(len(rows_b)) != 1           # row 1's baseline occurs once
    with pytest.raises(IndexError):
        imgpu.calc_closures(phase[keep], tsec[keep], blin[keep])
    with pytest.raises(IndexError):
        _closures_loop(phase[keep], tsec[keep], blin[keep])


def test_helpers():
    assert imgpu.cbinom(6, 3) == 20 and imgpu.cbinom(2, 3) == -1
    c = imgpu.combgen(6, 3)
    assert c.shape == (20, 3) and c[5].tolist() == [0, 2, 4]
    ib, ie = imgpu.get_time_indices(np.array([0, 0, 0, 1, 1, 2, 2, 2, 2], float))
    assert ib == [0, 5] and ie == [3, 9]


@pytest.mark.skipif(not REF_UV, reason="reference uv files not present")
def test_read_reference_uv_files():
    for f in REF_UV:
        ulam, vlam, wlam, amp, phase, blin, tsec, sig, chan, wei = imgpu.read_uvdata(f)
        assert 200 < ulam.size < 400
        base = 1e-3 * np.sqrt(ulam ** 2 + vlam ** 2)
        assert base.max() < 12.0
        cphs, cpix, trid, tcp = imgpu.calc_closures(phase, tsec, blin)
        assert cphs.size > 0
        ref = phase[cpix[:, 0]] + phase[cpix[:, 1]] - phase[cpix[:, 2]]
        assert np.allclose(_wrap(cphs - ref), 0, atol=1e-5)
        loop = _closures_loop(phase, tsec, blin)
        for g, r in zip((cpix, trid, tcp), loop[1:]):
            assert np.array_equal(g, r)
        assert np.allclose(_wrap(cphs - loop[0]), 0, atol=2e-6)


def test_mcgpu_defaults_follow_the_reference():
    m = imgpu.Mcgpu(coor=np.array([2, 2, 0.25, 0.5], np.float32), dat=np.array([1, 0.5]),
                    pdescr=np.array([1, 1]), pmint=np.array([-5.0, -5.0]),
                    pmaxt=np.array([5.0, 5.0]), nbeta=8, nseq=3, seed=1, model="solvsys")
    assert m.pcur.shape == (8, 3, 2) and np.all(m.pcur == 0.0)
    assert np.allclose(m.pstp, 0.2)
    assert m.beta[0] == 1.0 and np.isclose(m.beta[-1], 1e-4, rtol=1e-5)
    assert np.all(m.n_cnt == 1) and m.tcur[:, 1].tolist() == list(range(8))
    assert m.ndatm == 8 * 3 * 2 and m.invar.tolist() == [0, 1]


@pytest.mark.gpu
def test_solvsys_example_replay():
    """examples/solvsys/solvsys.py:38-62 through imgpu.Mcgpu."""
    m = imgpu.Mcgpu(coor=np.array([2, 2, 0.25, 0.5], np.float32), dat=np.array([1, 0.5]),
                    pdescr=np.array([1, 1]), pmint=np.array([-5.0, -5.0]),
                    pmaxt=np.array([5.0, 5.0]), nbeta=32, nseq=14, nburn=400, niter=5000,
                    seed=3, model="solvsys")
    m.burnin_and_search()
    assert m.pout.shape == (2, 14 * 5000) and m.chi2.shape == (14 * 5000,)
    best = m.pout[:, m.chi2 < 0.0002]
    rx = np.array([(-4.0 - np.sqrt(832.0)) / 34.0, (-4.0 + np.sqrt(832.0)) / 34.0])
    assert best.shape[1] > 0
    assert np.all(np.min(np.abs(best[0][:, None] - rx[None]), axis=1) < 0.05)
    assert m.rate_acpt.shape == (32, 14)


@pytest.mark.gpu
def test_sgra_fit_from_uv_file(tmp_path):
    f = str(tmp_path / "obs_uvdata.txt")
    truth, uv = synth.write_uvdata(f, nant=6, ntimes=20, seed=4)
    m = imgpu.Mcgpu_Sgra(f, imodel=1, nseq=4, nbeta=16, nburn=40, niter=60, seed=11,
                         pdescr=synth.SGRA9_PDESCR, pmint=synth.SGRA9_PMIN,
                         pmaxt=synth.SGRA9_PMAX, ecph=np.radians(5.0))
    assert m.error == "" and m.cpExt == 0 and m.ncph == 20 * imgpu.cbinom(6, 3)
    assert m.burnin_and_search() == 0
    # the recorded chi^2 of a sample equals calcmodchi2 of it, and FP64
    k = int(np.argmin(m.chi2))
    p = m.pout[:, k].astype(np.float32)
    chi2c, mvicp, mpha, chi2m, datm = m.calcmodchi2(p)
    assert np.isclose(chi2c, m.chi2[k], rtol=1e-5)
    pb = oracle.Problem("sgra", m.coor, m.dat, m.std2r, m.icoor, m.idat, 9, 1, 2)
    _, _, _, c2 = oracle.calc_modchi2(pb, p[None])
    assert np.isclose(chi2c, c2[0], rtol=1e-5)
    # calcmodel on a grid, interleaved layout, against FP64
    g = np.linspace(-6, 6, 9).astype(np.float32)
    U, V = np.meshgrid(g, g)
    mamp, mph = m.calcmodel(U, V, p, imodel=1, uv_layout="interleaved")
    a, ph = oracle.sgra_vis(1, p, U.ravel(), V.ravel())
    assert np.max(np.abs(mamp.ravel() - a) - 1e-5 * a) <= 1e-6 * p[0]


@pytest.mark.gpu
def test_search_rosenbrock_api_example_replay():
    """examples/search_Rosenbrock/search_Rosenbrock_api.py:60-160 (compute
    section, Python 3): the arrays built as the example builds them, one
    mcmc_interf.mcmcuda call on the Rosenbrock plugin, and the example's
    result -- the minimum chi^2 sample at (1, 1)."""
    from cuda_mcmc_gb300 import mcmc_interf as mi
    from numpy import array, float32, int32, uint8, uint64, where, zeros, ones_like, arange
    nseq, nbeta, niter, nburn = int32(14), int32(32), int32(1000), int32(400)
    seed = uint64(12345)
    imodel = 0
    pdescr = array((1, 1), dtype=int32)
    ptotal = array((0., 0.), dtype=float32)
    nptot = len(ptotal)
    pmint = array((-5., -5.), dtype=float32)
    pmaxt = array((5., 5.), dtype=float32)
    ivar = where(pdescr != 0)[0].astype(int32)
    nprm = len(ivar)
    pmin, pmax = pmint[ivar], pmaxt[ivar]
    invar = zeros(nptot, dtype=int32)
    ip = 0
    for i in range(nptot):
        if pdescr[i] != 0:
            invar[i] = ip
            ip = ip + 1
        else:
            invar[i] = -1
    nadj = int32(100)
    beta1, betan = float32(1.), float32(0.0001)
    npass = 1
    coor = array((2, 2, 0.25, 0.5), dtype=float32); ncoor = len(coor)
    icoor = zeros(1, dtype=int32); nicoor = len(coor)      # the example's over-read
    dat = zeros(1, dtype=float32); ndat = len(dat)
    std2r = ones_like(dat, dtype=float32)
    idat = zeros(1, dtype=int32); nidat = len(idat)
    datm = zeros((nbeta * nseq * ndat), dtype=float32); ndatm = len(datm)
    chi2m = zeros((nbeta, nseq, ndat), dtype=float32)
    rndst = zeros((nbeta, nseq, 48), dtype=uint8)
    beta = zeros((nbeta), dtype=float32)
    pstp = zeros((nprm, nbeta, nseq), dtype=float32)
    pout = zeros((nprm, nbeta, nseq, niter), dtype=float32)
    tout = zeros((nbeta, nseq, niter), dtype=int32)
    chi2 = zeros((nseq, niter), dtype=float32)
    flag = zeros((nbeta, nseq), dtype=int32)
    tcur = zeros((nbeta, nseq), dtype=int32)
    chi2c = zeros((nbeta, nseq), dtype=float32)
    n_cnt = zeros((nprm, nbeta, nseq), dtype=int32)
    n_acpt = zeros((nprm, nbeta, nseq), dtype=int32)
    n_exch = zeros((nbeta, nseq), dtype=int32)
    n_hist = zeros((nadj, nprm, nbeta, nseq), dtype=int32)
    ptentn = zeros((nbeta, nseq), dtype=int32)
    ptent = zeros((nbeta, nseq), dtype=float32)
    pcur = zeros((nbeta, nseq, nptot), dtype=float32)
    for i in range(nbeta):
        for j in range(nseq):
            pcur[i, j, :] = ptotal
            for k in range(nprm):
                pcur[i, j, ivar[k]] = pmin[k] + (pmax[k] - pmin[k]) / 2.
    pmid = (pmax - pmin) / 50.
    for i in range(nprm):
        pstp[i, :, :] = pmid[i]
    n0_nbeta = arange(nbeta)
    for i in range(nseq):
        tcur[:, i] = n0_nbeta
    bstp = (betan / beta1) ** (1.0 / float(nbeta - 1))
    for i in range(nbeta):
        beta[i] = beta1 * bstp ** i
    n_cnt[:] = float32(1.)
    mi.use_model("rosenbrock")
    with pytest.warns(RuntimeWarning, match="zero-padded"):
        mi.mcmcuda(coor, dat, std2r, icoor, idat, datm, chi2m, pdescr, ivar, invar, ptotal,
                   pmint, pmaxt, pout, tout, chi2, chi2c, tcur, flag, n_acpt, n_exch, n_cnt,
                   n_hist, beta, pstp, ptent, ptentn, pcur, rndst, uint64(seed), int32(imodel),
                   int32(ncoor), int32(ndat), int32(nicoor), int32(nidat), int32(ndatm),
                   int32(nptot), int32(nprm), int32(nadj), int32(npass), int32(nbeta),
                   int32(nseq), int32(nburn), int32(niter))
    mi.reset_gpu()
    mi.use_model("sgra")
    c2 = chi2.flatten()
    po = pout[:, 0, :, :].reshape((nprm, nseq * niter))
    im = c2.argmin()
    assert np.all(np.abs(po[:, im] - 1.0) < 0.05), po[:, im]
    assert (c2 < 0.00001).sum() > 0
