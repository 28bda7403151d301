"""Generate the golden fixtures in tests/golden/ from the REFERENCE's own code.

Run in a container that has the reference tree (it is not needed afterwards):

    python tests/golden/make_golden.py

oracle/ref_build.py compiles the reference's src/gpu_mcmc.cu kernels and its
examples' model.cuh files for the CPU (oracle/_ref/libref_<model>.so);
oracle/ref.py drives them in the order of run_calcmodchi2 / run_mcmc with
injected random streams.  The fixtures store the inputs and the reference's
float32 outputs:

  sgra_modchi2_m9.npz     calc_modchi2, sgra_model9, closures from phases
  sgra_modchi2_m13.npz    calc_modchi2, sgra_model13
  sgra_modchi2_cpext.npz  calc_modchi2, sgra_model9, closures from uv triangles
  sweep_<model>.npz       run_mcmc with injected streams: final state + traces
                          (models: sgra, rosenbrock (2-D), solvsys)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import ref  # noqa: E402
from cuda_mcmc_gb300 import synth  # noqa: E402


def sgra_params(rng, n, imodel):
    """n parameter sets inside the prior plus the model's edge cases."""
    if imodel == 1:
        lo, hi = synth.SGRA9_PMIN.astype(np.float64), synth.SGRA9_PMAX.astype(np.float64)
        P = rng.uniform(lo, hi, (n, 9))
        P[0, 2] = 0.0            # rq = 0: no inner disk (Rin == 0 branch)
        P[1, 7] = 0.0            # gq = 0: Gaussian off
        P[2, 5] = 0.0            # gax = 0: Gaussian off
        P[3, 7] = 1.0            # gq = 1: Gaussian only
        P[4, 3] = 0.0            # ecc = 0: concentric
        P[5, 4] = 1.0            # fade = 1: uniform ring
    else:
        lo = np.array([1.0, 20, 0.0, 0.0, 0.0, 0.0, 0.1, 0.05, 0.0, -np.pi, -np.pi, -np.pi, -np.pi])
        hi = np.array([3.0, 40, 0.99, 1.0, 1.0, 1.0, 2.5, 1.0, 1.0, np.pi, np.pi, np.pi, np.pi])
        P = rng.uniform(lo, hi, (n, 13))
        P[0, 2] = 0.0            # rq = 0
        P[1, 8] = 0.0            # gq = 0
        P[2, 8] = 1.0            # gq = 1: Gaussian only (model.cuh:204-210)
        P[3, 6] = 0.0            # gax = 0
    return P.astype(np.float32)


def modchi2_fixture(name, imodel, cpext, seed):
    w = synth.sgra(nvis=120, ncph=40, seed=seed, nseq=1, nbeta=1, imodel=1)
    nvis, ncph = w.nvis, w.ndat - w.nvis
    coor = w.coor.copy()
    coor[0:2] = 0.0                        # a zero baseline: the rho -> 0 limits
    coor[2:4] = np.float32(3e-8)           # below the 1e-7 threshold as well
    icoor = w.icoor
    if cpext:
        tri = w.icoor.reshape(ncph, 3)
        uv = coor.reshape(-1, 2)
        ext = np.concatenate([uv[tri[:, 0]], uv[tri[:, 1]]], axis=1).ravel()
        coor = np.concatenate([coor, ext]).astype(np.float32)
        icoor = np.zeros(1, np.int32)
    rng = np.random.default_rng(seed + 100)
    P = sgra_params(rng, 16, imodel)
    idat = np.array([nvis, 16 * w.ndat, cpext], np.int32)
    pb = oracle.Problem("sgra", coor, w.dat, w.std2r, icoor, idat, P.shape[1], imodel, 2)
    datm, chi2m, chi2c = ref.calc_modchi2(pb, P)
    np.savez_compressed(os.path.join(HERE, name), coor=coor, dat=w.dat, std2r=w.std2r,
                        icoor=icoor, idat=idat, pcur=P, imodel=np.int32(imodel),
                        datm=datm, chi2m=chi2m, chi2c=chi2c)
    print(name, "chi2c", chi2c[:4])


def sweep_fixture(model, w, nburn, niter, seed):
    nrep = w.nbeta * w.nseq
    steps = nburn + niter
    rs = oracle.make_streams(nrep, w.nprm + steps * (2 * w.nprm + 3 * w.nbeta) + 64,
                             steps * w.nprm + 8, seed)
    u, n = rs.u.copy(), rs.n.copy()
    st = oracle.new_state(w.pdescr, w.pmint, w.pmaxt, w.beta(), w.nseq, niter,
                          ptotal=w.ptotal, pstp=None, ndat=w.ndat)
    if w.pstp0 is not None:
        st.pstp[:] = np.asarray(w.pstp0, np.float32)[:, None, None]
    pstp0 = st.pstp.copy()
    pb = oracle.Problem(model, w.coor, w.dat, w.std2r, w.icoor, w.idat, w.nptot, w.imodel, w.npass)
    datm, chi2m = ref.sweep(pb, st, rs, 1, nburn, niter)
    np.savez_compressed(
        os.path.join(HERE, "sweep_%s.npz" % model),
        coor=w.coor, dat=w.dat, std2r=w.std2r, icoor=w.icoor, idat=w.idat, pdescr=w.pdescr,
        pmint=w.pmint, pmaxt=w.pmaxt, ptotal=w.ptotal, beta=w.beta(), pstp0=pstp0,
        imodel=np.int32(w.imodel), npass=np.int32(w.npass), nseq=np.int32(w.nseq),
        nburn=np.int32(nburn), niter=np.int32(niter), u=u, n=n,
        pcur=st.pcur, chi2c=st.chi2c.astype(np.float32), flag=st.flag, ptent=st.ptent,
        ptentn=st.ptentn, pstp=st.pstp, n_acpt=st.n_acpt, n_exch=st.n_exch, n_cnt=st.n_cnt,
        n_hist=st.n_hist, tcur=st.tcur, pout=st.pout, tout=st.tout, chi2=st.chi2,
        cu=rs.cu, cn=rs.cn)
    print("sweep_%s: accepts %d exchanges %d" % (model, st.n_acpt.sum(), st.n_exch.sum()))


def main():
    if not ref.ref_build.available():
        sys.exit("the reference tree is not present; nothing generated")
    ref.ref_build.build()
    modchi2_fixture("sgra_modchi2_m9.npz", 1, 0, 21)
    modchi2_fixture("sgra_modchi2_m13.npz", 2, 0, 22)
    modchi2_fixture("sgra_modchi2_cpext.npz", 1, 1, 23)
    ws = synth.sgra(nvis=60, ncph=20, seed=31, nseq=2, nbeta=4)
    sweep_fixture("sgra", ws, 8, 8, 41)
    wr = synth.rosenbrock(n=2, nseq=3, nbeta=4)
    sweep_fixture("rosenbrock", wr, 25, 25, 42)
    wv = synth.solvsys(nseq=3, nbeta=4)
    sweep_fixture("solvsys", wv, 25, 25, 43)


if __name__ == "__main__":
    main()
