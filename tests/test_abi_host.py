"""CPU tests of the C-ABI libraries and the host layer (no GPU compute).

* every library loads and exports every function include/cuda_mcmc.h
  declares (cmc_run_noalloc and the gradient entry points: libcmc_sgra.so
  only; cmc_module_set: libcmc_module.so only), with the job layout the
  Python mirror expects;
* mcmc_interf validates its arguments like the reference's Cython signatures
  (dtype / ndim errors) before anything reaches the device;
* the launch-shape query rejects impossible sizes without a GPU.
"""
import ctypes as C
import os
import re

import numpy as np
import pytest

from cuda_mcmc_gb300 import _build, _lib, mcmc_interf, synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBS = ("sgra", *_build.BUILTIN_PLUGINS, "module")


def declared_functions():
    text = open(os.path.join(ROOT, "include", "cuda_mcmc.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b([a-z_][a-z0-9_]*)\s*\(", text)
    keywords = {"if", "for", "while", "sizeof", "return", "defined"}
    return sorted({n for n in names if n not in keywords})


def exported(path):
    import subprocess
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True,
                         text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if " T " in line}


@pytest.mark.parametrize("name", LIBS)
def test_library_exports_every_declared_symbol(name):
    L = _lib.load(name)
    syms = exported(_build.lib_path(name))
    want = set(declared_functions())
    if name != "sgra":
        for only_sgra in ("cmc_run_noalloc", "cmc_grad", "cmc_grad_work_bytes", "cmc_fisher",
                          "cmc_fisher_work_bytes"):
            want.discard(only_sgra)
    if name != "module":
        want.discard("cmc_module_set")
    assert want, "no declarations parsed"
    missing = want - syms
    assert not missing, "missing exports: %s" % sorted(missing)
    assert L.cmc_sizeof_job() == C.sizeof(_lib.CmcJob)
    assert L.cmc_abi_version() == 3
    assert L.cmc_model_name().decode() == name


def test_header_declares_the_reference_entry_points():
    d = declared_functions()
    for f in ("mcmc_cuda", "calc_modchi2", "calc_model", "cmc_run", "cmc_eval",
              "cmc_run_noalloc"):
        assert f in d


def _args(w, nbeta=4, nseq=2, niter=3, **over):
    from cuda_mcmc_gb300.device import sampler_defaults
    s = sampler_defaults(w.pdescr, w.pmint, w.pmaxt, nbeta, nseq)
    nrep, nprm = nbeta * nseq, w.nprm
    a = dict(coor=w.coor, dat=w.dat, std2r=w.std2r, icoor=w.icoor, idat=w.idat,
             datm=np.zeros(nrep * (w.ndat + w.nvis), np.float32),
             chi2m=np.zeros((nbeta, nseq, w.ndat), np.float32), pdescr=s["pdescr"],
             ivar=s["ivar"], invar=s["invar"], ptotal=s["ptotal"], pmint=s["pmint"],
             pmaxt=s["pmaxt"], pout=np.zeros((nprm, nbeta, nseq, niter), np.float32),
             tout=np.zeros((nbeta, nseq, niter), np.int32),
             chi2=np.zeros((nseq, niter), np.float32), chi2c=s["chi2c"], tcur=s["tcur"],
             flag=s["flag"], n_acpt=s["n_acpt"], n_exch=s["n_exch"], n_cnt=s["n_cnt"],
             n_hist=s["n_hist"], beta=synth.geometric_betas(nbeta), pstp=s["pstp"],
             ptent=s["ptent"], ptentn=s["ptentn"], pcur=s["pcur"],
             rndst=np.zeros((nbeta, nseq, 48), np.uint8), seed=1, imodel=w.imodel,
             ncoor=w.coor.size, ndat=w.ndat, nicoor=w.icoor.size, nidat=w.idat.size,
             ndatm=nrep * (w.ndat + w.nvis), nptot=w.nptot, nprm=nprm, nadj=100, npass=w.npass,
             nbeta=nbeta, nseq=nseq, nburn=2, niter=niter)
    a.update(over)
    return a


def test_mcmcuda_rejects_wrong_dtype_and_ndim_before_the_device():
    w = synth.sgra(nvis=20, ncph=6, nseq=2, nbeta=4)
    a = _args(w)
    with pytest.raises(ValueError, match="dtype"):
        mcmc_interf.mcmcuda(**{**a, "coor": a["coor"].astype(np.float64)})
    with pytest.raises(ValueError, match="dimensions"):
        mcmc_interf.mcmcuda(**{**a, "pout": a["pout"].reshape(-1)})
    with pytest.raises(ValueError, match="writes"):
        mcmc_interf.mcmcuda(**{**a, "pout": np.zeros((1, 1, 1, 1), np.float32)})
    with pytest.raises(TypeError):
        mcmc_interf.mcmcuda(**{**a, "dat": list(a["dat"])})


def test_short_inputs_are_padded_with_a_warning():
    a = np.array([1, 2], np.int32)
    with pytest.warns(RuntimeWarning, match="zero-padded"):
        b = mcmc_interf._arr(a, np.int32, 1, "icoor", 4)
    assert b.tolist() == [1, 2, 0, 0]


def test_query_rejects_impossible_shapes_without_gpu():
    L = _lib.load("sgra")
    j = _lib.CmcJob()
    rc = L.cmc_run(C.byref(j), None)          # all-zero job: sizes invalid
    assert rc == _lib.CMC_ERR_ARG
    assert "nbeta" in L.cmc_last_error().decode()
