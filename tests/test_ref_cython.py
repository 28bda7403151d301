"""The reference's own Cython bridge, src/mcmc_interf.pyx, on this library.

The reference's Python API reaches its CUDA code through mcmc_interf, a Cython
module that declares the three entry points from "mcmc.h" and is linked with
the CUDA library (src/mcmc_interf.pyx:213-343, src/setup_mcmc.py:10-18).
Dropping this library in means building that .pyx unchanged with this
repository's include/ on the include path and libcmc_sgra.so on the link
line.  oracle/ref_build.py turns the .pyx into C with Cython where the
reference tree is (Cython is not on the GPU host); these tests compile that C
into an extension here and on the GPU host, import it, and (on a GPU) check
that its mcmcuda / calcmodchi2 / calcmodel give the results of this
package's own mcmc_interf.  Its reset_gpu calls cudaDeviceReset, which would
tear down the context PyTorch shares, and is not called.
"""
import importlib.util
import os
import subprocess
import sys
import sysconfig

import numpy as np
import pytest

from oracle import ref_build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bridge(tmp_path):
    src = ref_build.cython_path()
    if not os.path.isfile(src):
        pytest.skip("the Cython output of the reference's mcmc_interf.pyx is not present "
                    "(oracle/ref_build.py makes it where the reference tree is)")
    from cuda_mcmc_gb300 import _build
    lib = _build.build(["sgra"])["sgra"]
    libdir = os.path.dirname(lib)
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    so = os.path.join(str(tmp_path), "mcmc_interf" + sysconfig.get_config_var("EXT_SUFFIX"))
    cmd = ["gcc", "-shared", "-fPIC", "-O2", "-w", "-I", sysconfig.get_paths()["include"],
           "-I", np.get_include(), "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(cuda, "include"), src, "-o", so,
           "-L", libdir, "-lcmc_sgra", "-Wl,-rpath," + libdir,
           "-L", os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.join(cuda, "lib64")]
    subprocess.run(cmd, check=True)
    spec = importlib.util.spec_from_file_location("mcmc_interf", so)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_reference_bridge_builds_against_this_library(tmp_path):
    mod = _bridge(tmp_path)
    for f in ("mcmcuda", "calcmodchi2", "calcmodel", "reset_gpu"):
        assert callable(getattr(mod, f))


@pytest.mark.gpu
def test_reference_bridge_runs_this_library(tmp_path):
    from cuda_mcmc_gb300 import mcmc_interf, synth
    from cuda_mcmc_gb300.device import sampler_defaults
    mod = _bridge(tmp_path)
    w = synth.sgra(nvis=500, ncph=150, seed=12, nseq=4, nbeta=8, nburn=10, niter=20)
    nrep, nprm = w.nbeta * w.nseq, w.nprm
    out = []
    for bridge in (mod, mcmc_interf):
        if bridge is mcmc_interf:
            mcmc_interf.use_model("sgra")
        s = sampler_defaults(w.pdescr, w.pmint, w.pmaxt, w.nbeta, w.nseq)
        pout = np.zeros((nprm, w.nbeta, w.nseq, w.niter), np.float32)
        tout = np.zeros((w.nbeta, w.nseq, w.niter), np.int32)
        chi2 = np.zeros((w.nseq, w.niter), np.float32)
        datm = np.zeros(nrep * (w.ndat + w.nvis), np.float32)
        chi2m = np.zeros((w.nbeta, w.nseq, w.ndat), np.float32)
        rndst = np.zeros((w.nbeta, w.nseq, 48), np.uint8)
        bridge.mcmcuda(w.coor, w.dat, w.std2r, w.icoor, w.idat, datm, chi2m, s["pdescr"],
                       s["ivar"], s["invar"], s["ptotal"], s["pmint"], s["pmaxt"], pout, tout,
                       chi2, s["chi2c"], s["tcur"], s["flag"], s["n_acpt"], s["n_exch"],
                       s["n_cnt"], s["n_hist"], w.beta(), s["pstp"], s["ptent"], s["ptentn"],
                       s["pcur"], rndst, np.uint64(31), w.imodel, w.coor.size, w.ndat,
                       w.icoor.size, w.idat.size, datm.size, w.nptot, nprm, 100, w.npass,
                       w.nbeta, w.nseq, w.nburn, w.niter)
        c2m = np.zeros((w.nbeta, w.nseq, w.ndat), np.float32)
        dm = np.zeros(nrep * (w.ndat + w.nvis), np.float32)
        c2c = np.zeros((w.nbeta, w.nseq), np.float32)
        bridge.calcmodchi2(w.coor, w.dat, w.std2r, w.icoor, w.idat, dm, c2m, s["pcur"], c2c,
                           np.ones((w.nbeta, w.nseq), np.int32), w.imodel, w.coor.size, w.ndat,
                           w.icoor.size, w.idat.size, dm.size, w.nptot, w.nbeta, w.nseq)
        dm2 = np.zeros(nrep * 2 * w.nvis, np.float32)
        bridge.calcmodel(w.coor, w.idat, dm2, s["pcur"], w.imodel, w.coor.size, w.nvis,
                         w.idat.size, dm2.size, w.nptot, w.nbeta, w.nseq)
        out.append(dict(s, pout=pout, tout=tout, chi2=chi2, datm=datm, chi2m=chi2m, rndst=rndst,
                        c2c=c2c, dm=dm, dm2=dm2))
    a, b = out
    assert a["n_acpt"].sum() > 0
    for k in a:
        assert np.array_equal(a[k], b[k]), k
