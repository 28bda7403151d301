"""mcmc_interf -- the reference's Python interface module, for Python 3.

Same four functions as the reference's Cython module (src/mcmc_interf.pyx):
``mcmcuda`` (:230-281), ``calcmodchi2`` (:294-313), ``calcmodel`` (:325-336)
and ``reset_gpu`` (:342-343), with the same argument lists, dtypes and
in-place output semantics: every output array is written in place.

Differences a caller can see:
  * the model is chosen at run time with :func:`use_model` (or the
    ``CUDA_MCMC_MODEL`` environment variable) instead of being compiled into
    the module; the default is the built-in Sgr A* model;
  * errors raise :class:`McmcError` (the reference prints and calls exit(1));
  * an INPUT array shorter than its size argument (e.g. the reference's
    examples pass nicoor = 4 with a one-element icoor) is zero-padded to that
    size instead of being read past its end; a short OUTPUT array raises;
  * ``reset_gpu`` synchronises the device instead of destroying the CUDA
    context (cudaDeviceReset), so that other users of the context (PyTorch)
    keep working.
"""
from __future__ import annotations

import os
import warnings

import numpy as np

from . import _lib
from ._lib import McmcError

__all__ = ["mcmcuda", "calcmodchi2", "calcmodel", "reset_gpu", "use_model", "McmcError"]

_current = {"lib": None, "name": None}


def use_model(model: str = "sgra"):
    """Select the model library: a built-in name (sgra, rosenbrock, solvsys,
    nlsys) or the path of a library built with ``_build.build_plugin``."""
    if os.path.sep in model or model.endswith(".so"):
        L = _lib.load_path(model)
    else:
        L = _lib.load(model)
    _current["lib"] = L
    _current["name"] = model
    return L


def _L():
    if _current["lib"] is None:
        use_model(os.environ.get("CUDA_MCMC_MODEL", "sgra"))
    return _current["lib"]


def _arr(a, dtype, ndim, name, n=None, output=False):
    if not isinstance(a, np.ndarray):
        raise TypeError("%s must be a numpy.ndarray" % name)
    if a.dtype != dtype:
        raise ValueError("Buffer dtype mismatch for %s: expected %s, got %s"
                         % (name, np.dtype(dtype).name, a.dtype.name))
    if a.ndim != ndim:
        raise ValueError("Buffer has wrong number of dimensions for %s (expected %d, got %d)"
                         % (name, ndim, a.ndim))
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("%s must be C-contiguous" % name)
    if n is not None and a.size < n:
        if output:
            raise ValueError("%s has %d elements; the call writes %d" % (name, a.size, n))
        warnings.warn("%s has %d elements but its size argument is %d: passing a zero-padded "
                      "copy" % (name, a.size, n), RuntimeWarning, stacklevel=3)
        b = np.zeros(n, dtype)
        b[:a.size] = a.ravel()
        return b
    return a


def _p(a, t):
    return a.ctypes.data_as(t)


def mcmcuda(coor, dat, std2r, icoor, idat, datm, chi2m, pdescr, ivar, invar, ptotal, pmint,
            pmaxt, pout, tout, chi2, chi2c, tcur, flag, n_acpt, n_exch, n_cnt, n_hist, beta,
            pstp, ptent, ptentn, pcur, rndst, seed, imodel, ncoor, ndat, nicoor, nidat, ndatm,
            nptot, nprm, nadj, npass, nbeta, nseq, nburn, niter):
    """Run the MCMC-RE sweep (burn-in + main stage); outputs are written in place."""
    f4, i4 = np.float32, np.int32
    ncoor, ndat, nicoor, nidat, ndatm = int(ncoor), int(ndat), int(nicoor), int(nidat), int(ndatm)
    nptot, nprm, nadj, npass = int(nptot), int(nprm), int(nadj), int(npass)
    nbeta, nseq, nburn, niter = int(nbeta), int(nseq), int(nburn), int(niter)
    nrep = nbeta * nseq
    coor = _arr(coor, f4, 1, "coor", ncoor)
    dat = _arr(dat, f4, 1, "dat", ndat)
    std2r = _arr(std2r, f4, 1, "std2r", ndat)
    icoor = _arr(icoor, i4, 1, "icoor", nicoor)
    idat = _arr(idat, i4, 1, "idat", nidat)
    datm = _arr(datm, f4, 1, "datm", ndatm, output=True)
    chi2m = _arr(chi2m, f4, 3, "chi2m", nrep * ndat, output=True)
    pdescr = _arr(pdescr, i4, 1, "pdescr", nptot)
    ivar = _arr(ivar, i4, 1, "ivar", nprm)
    invar = _arr(invar, i4, 1, "invar", nptot)
    ptotal = _arr(ptotal, f4, 1, "ptotal", nptot)
    pmint = _arr(pmint, f4, 1, "pmint", nptot)
    pmaxt = _arr(pmaxt, f4, 1, "pmaxt", nptot)
    pout = _arr(pout, f4, 4, "pout", nprm * nrep * niter, output=True)
    tout = _arr(tout, i4, 3, "tout", nrep * niter, output=True)
    chi2 = _arr(chi2, f4, 2, "chi2", nseq * niter, output=True)
    chi2c = _arr(chi2c, f4, 2, "chi2c", nrep, output=True)
    tcur = _arr(tcur, i4, 2, "tcur", nrep, output=True)
    flag = _arr(flag, i4, 2, "flag", nrep, output=True)
    n_acpt = _arr(n_acpt, i4, 3, "n_acpt", nprm * nrep, output=True)
    n_exch = _arr(n_exch, i4, 2, "n_exch", nrep, output=True)
    n_cnt = _arr(n_cnt, i4, 3, "n_cnt", nprm * nrep, output=True)
    n_hist = _arr(n_hist, i4, 4, "n_hist", nadj * nprm * nrep, output=True)
    beta = _arr(beta, f4, 1, "beta", nbeta)
    pstp = _arr(pstp, f4, 3, "pstp", nprm * nrep, output=True)
    ptent = _arr(ptent, f4, 2, "ptent", nrep, output=True)
    ptentn = _arr(ptentn, i4, 2, "ptentn", nrep, output=True)
    pcur = _arr(pcur, f4, 3, "pcur", nrep * nptot, output=True)
    rndst = _arr(rndst, np.uint8, 3, "rndst", nrep * 48, output=True)
    L = _L()
    F, I, U = _lib._fp, _lib._ip, _lib._u8p
    rc = L.mcmc_cuda_v2(
        _p(coor, F), _p(dat, F), _p(std2r, F), _p(icoor, I), _p(idat, I), _p(datm, F),
        _p(chi2m, F), _p(pdescr, I), _p(ivar, I), _p(invar, I), _p(ptotal, F), _p(pmint, F),
        _p(pmaxt, F), _p(pout, F), _p(tout, I), _p(chi2, F), _p(chi2c, F), _p(tcur, I),
        _p(flag, I), _p(n_acpt, I), _p(n_exch, I), _p(n_cnt, I), _p(n_hist, I), _p(beta, F),
        _p(pstp, F), _p(ptent, F), _p(ptentn, I), _p(pcur, F), _p(rndst, U),
        int(np.uint64(seed)), int(imodel), ncoor, ndat, nicoor, nidat, ndatm, nptot, nprm, nadj,
        npass, nbeta, nseq, nburn, niter)
    _lib.check(L, rc)


def calcmodchi2(coor, dat, std2r, icoor, idat, datm, chi2m, pcur, chi2c, flag, imodel, ncoor,
                ndat, nicoor, nidat, ndatm, nptot, nbeta, nseq):
    """Model values, chi^2 terms and chi^2 for nbeta*nseq parameter sets (in place)."""
    f4, i4 = np.float32, np.int32
    ncoor, ndat, nicoor, nidat, ndatm = int(ncoor), int(ndat), int(nicoor), int(nidat), int(ndatm)
    nptot, nbeta, nseq = int(nptot), int(nbeta), int(nseq)
    nrep = nbeta * nseq
    coor = _arr(coor, f4, 1, "coor", ncoor)
    dat = _arr(dat, f4, 1, "dat", ndat)
    std2r = _arr(std2r, f4, 1, "std2r", ndat)
    icoor = _arr(icoor, i4, 1, "icoor", nicoor)
    idat = _arr(idat, i4, 1, "idat", nidat)
    datm = _arr(datm, f4, 1, "datm", ndatm, output=True)
    chi2m = _arr(chi2m, f4, 3, "chi2m", nrep * ndat, output=True)
    pcur = _arr(pcur, f4, 3, "pcur", nrep * nptot)
    chi2c = _arr(chi2c, f4, 2, "chi2c", nrep, output=True)
    flag = _arr(flag, i4, 2, "flag", nrep)
    L = _L()
    F, I = _lib._fp, _lib._ip
    rc = L.calc_modchi2_v2(_p(coor, F), _p(dat, F), _p(std2r, F), _p(icoor, I), _p(idat, I),
                           _p(datm, F), _p(chi2m, F), _p(pcur, F), _p(chi2c, F), _p(flag, I),
                           int(imodel), ncoor, ndat, nicoor, nidat, ndatm, nptot, nbeta, nseq)
    _lib.check(L, rc)


def calcmodel(coor, idat, datm, pcur, imodel, ncoor, ndat, nidat, ndatm, nptot, nbeta, nseq):
    """Model values only (pass 0) for nbeta*nseq parameter sets (datm in place)."""
    f4, i4 = np.float32, np.int32
    ncoor, ndat, nidat, ndatm = int(ncoor), int(ndat), int(nidat), int(ndatm)
    nptot, nbeta, nseq = int(nptot), int(nbeta), int(nseq)
    coor = _arr(coor, f4, 1, "coor", ncoor)
    idat = _arr(idat, i4, 1, "idat", nidat)
    datm = _arr(datm, f4, 1, "datm", ndatm, output=True)
    pcur = _arr(pcur, f4, 3, "pcur", nbeta * nseq * nptot)
    L = _L()
    F, I = _lib._fp, _lib._ip
    rc = L.calc_model_v2(_p(coor, F), _p(idat, I), _p(datm, F), _p(pcur, F), int(imodel), ncoor,
                         ndat, nidat, ndatm, nptot, nbeta, nseq)
    _lib.check(L, rc)


def reset_gpu():
    """Wait for the device (the reference resets it; see the module docstring)."""
    L = _L()
    _lib.check(L, L.cmc_reset_gpu())
