"""imgpu -- the reference's high-level Python API, for Python 3.

Classes ``Mcgpu`` (any model) and ``Mcgpu_Sgra`` (the Sgr A* crescent fit)
with the constructor arguments, attributes and methods of the reference's
src/imgpu.py (:240-571 and :585-1067), running on this library through
``mcmc_interf``; and the data helpers ``read_uvdata`` (:1375-1474),
``calc_closures`` (:1229-1325), ``get_time_indices`` (:1184-1225),
``find_triangles`` (:1160-1180), ``combgen`` (:1103-1156), ``cbinom``
and ``count_lines`` (:1329-1371).

Behaviour kept from the reference (so that its scripts give the same
numbers):
  * defaults: nbeta=32, nseq=14, nburn=300, niter=500, nadj=100; betas
    geometric from 1 (the ``beta1`` argument does not move the first beta) to
    ``betan`` = 1e-4; pcur at the prior centres; pstp = (pmax - pmin)/50;
    n_cnt = 1; a time-based seed when none is given;
  * ``rate_acpt`` / ``rate_exch`` use Python's built-in ``sum(array, 2)``
    (the sum over the first axis plus 2), divided by niter*nseq;
  * ``Mcgpu_Sgra.calcmodel`` packs coor as [u..., v...] while the model reads
    [u0, v0, u1, v1, ...]; pass ``uv_layout="interleaved"`` for model values
    at the given (u, v) points;
  * when any sigma in a uv file is zero, all are set to 1
    (``if all(fsig) == 0``), as the reference does.
Differences: ``Mcgpu_Sgra`` also works without a uv file when ``amp`` (and
``ulam``, ``vlam``) are given; ``calc_closures`` returns empty arrays instead
of failing when there are no triangles; ``Mcgpu_Sgra.burnin_and_search`` also
sets the flattened ``pout`` / ``chi2`` that ``Mcgpu`` sets.
"""
from __future__ import annotations

import builtins
import itertools
import os
import re
import time
from calendar import timegm
from time import strptime

import numpy as np

from . import mcmc_interf as mi

PK2I = 2 ** 15
PK3I = 2 ** 10
_NUM = re.compile(r"[+-]?\d+\.?\d*[eE][+-]?\d+|[+-]?\d*\.?\d+[eE][+-]?\d+|"
                  r"[+-]?\d+\.?\d*|[+-]?\d*\.?\d+|[+-]?\d+")


def _rates(n_acpt, n_exch, niter, nseq):
    nitsq = np.float32(niter * nseq)
    # the reference calls Python's built-in sum here (src/imgpu.py:453-455)
    return builtins.sum(n_acpt, 2) / nitsq, builtins.sum(n_exch, 2) / nitsq


class Mcgpu(object):
    """MCMC-RE for any model library (see ``mcmc_interf.use_model``)."""

    def __init__(self, coor=None, dat=None, std2r=None, icoor=None, idat=None,
                 pdescr=None, ptotal=None, pmint=None, pmaxt=None,
                 beta=None, beta1=None, betan=None,
                 seed=None, imodel=0, npass=1,
                 nadj=100, nbeta=32, nseq=14, nburn=300, niter=500, model=None):
        if model is not None:
            mi.use_model(model)
        self.dat = np.zeros(1, np.float32) if dat is None else np.asarray(dat).astype(np.float32)
        ndat = np.int32(np.size(dat))
        self.std2r = (np.ones_like(self.dat, dtype=np.float32) if std2r is None
                      else np.asarray(std2r).astype(np.float32))
        self.coor = np.zeros(1, np.float32) if coor is None else np.asarray(coor).astype(np.float32)
        ncoor = np.int32(np.size(coor))
        self.icoor = (np.zeros(1, np.int32) if icoor is None
                      else np.asarray(icoor).astype(np.int32))
        nicoor = np.int32(np.size(icoor))
        self.idat = np.zeros(1, np.int32) if idat is None else np.int32(np.atleast_1d(idat))
        nidat = np.int32(np.size(idat))
        self.datm = np.zeros(nbeta * nseq * ndat, np.float32)
        ndatm = np.int32(np.size(self.datm))
        self.chi2m = np.zeros((nbeta, nseq, ndat), np.float32)
        self.pdescr = np.int32(pdescr)
        self.nptot = nptot = np.int32(len(pdescr))
        self.ptotal = (np.zeros(nptot, np.float32) if ptotal is None
                       else np.asarray(ptotal).astype(np.float32))
        self.pmint = np.asarray(pmint).astype(np.float32)
        self.pmaxt = np.asarray(pmaxt).astype(np.float32)
        self.ivar = ivar = np.where(self.pdescr != 0)[0].astype(np.int32)
        self.nprm = nprm = np.int32(len(ivar))
        self.pmin = pmin = self.pmint[ivar]
        self.pmax = pmax = self.pmaxt[ivar]
        self.invar = np.full(nptot, -1, np.int32)
        self.invar[ivar] = np.arange(nprm, dtype=np.int32)
        if seed is None:
            nstates = np.int32(nseq * nbeta)
            self.seed = np.uint64(np.trunc(1e6 * time.time() % (10 * nstates)))
        else:
            self.seed = np.uint64(seed)
        self.ncoor, self.ndat, self.nidat = np.int32(ncoor), np.int32(ndat), np.int32(nidat)
        self.nicoor, self.ndatm = np.int32(nicoor), np.int32(ndatm)
        self.nadj, self.nbeta, self.npass = np.int32(nadj), np.int32(nbeta), np.int32(npass)
        self.nseq, self.nburn, self.niter = np.int32(nseq), np.int32(nburn), np.int32(niter)
        self.imodel = np.int32(imodel)
        self.pstp = np.zeros((nprm, nbeta, nseq), np.float32)
        self.pout_4d = np.zeros((nprm, nbeta, nseq, niter), np.float32)
        self.tout = np.zeros((nbeta, nseq, niter), np.int32)
        self.chi2_2d = np.zeros((nseq, niter), np.float32)
        self.flag = np.zeros((nbeta, nseq), np.int32)
        self.tcur = np.zeros((nbeta, nseq), np.int32)
        self.chi2c = np.zeros((nbeta, nseq), np.float32)
        self.n_cnt = np.zeros((nprm, nbeta, nseq), np.int32)
        self.n_acpt = np.zeros((nprm, nbeta, nseq), np.int32)
        self.n_exch = np.zeros((nbeta, nseq), np.int32)
        self.n_hist = np.zeros((nadj, nprm, nbeta, nseq), np.int32)
        self.ptentn = np.zeros((nbeta, nseq), np.int32)
        self.ptent = np.zeros((nbeta, nseq), np.float32)
        self.pcur = np.zeros((nbeta, nseq, nptot), np.float32)
        self.rndst = np.zeros((nbeta, nseq, 48), np.uint8)
        self.pcur[:, :, :] = self.ptotal
        self.pcur[:, :, ivar] = pmin + (pmax - pmin) / np.float32(2.0)
        self.pstp[:, :, :] = ((pmax - pmin) / 50.0).astype(np.float32)[:, None, None]
        self.tcur[:, :] = np.arange(nbeta, dtype=np.int32)[:, None]
        self.beta1 = np.float32(1.0) if beta1 is None else np.float32(beta1)
        self.betan = np.float32(0.0001) if betan is None else np.float32(betan)
        if beta is None:
            # the first temperature is 1 whatever beta1 says (src/imgpu.py:412-418)
            bstp = (self.betan / np.float32(1.0)) ** (1.0 / np.float32(nbeta - 1))
            self.beta = np.array([bstp ** i for i in range(nbeta)], np.float32)
        else:
            self.beta = np.asarray(beta).astype(np.float32)
        self.n_cnt[:] = 1

    def _mcmcuda(self):
        mi.mcmcuda(self.coor, self.dat, self.std2r, self.icoor, self.idat, self.datm, self.chi2m,
                   self.pdescr, self.ivar, self.invar, self.ptotal, self.pmint, self.pmaxt,
                   self.pout_4d, self.tout, self.chi2_2d, self.chi2c, self.tcur, self.flag,
                   self.n_acpt, self.n_exch, self.n_cnt, self.n_hist, self.beta, self.pstp,
                   self.ptent, self.ptentn, self.pcur, self.rndst, self.seed, self.imodel,
                   self.ncoor, self.ndat, self.nicoor, self.nidat, self.ndatm, self.nptot,
                   self.nprm, self.nadj, self.npass, self.nbeta, self.nseq, self.nburn,
                   self.niter)
        mi.reset_gpu()

    def burnin_and_search(self):
        self._mcmcuda()
        self.rate_acpt, self.rate_exch = _rates(self.n_acpt, self.n_exch, self.niter, self.nseq)
        self.chi2 = self.chi2_2d.flatten()
        self.pout = self.pout_4d[:, 0, :, :].reshape((self.nprm, self.nseq * self.niter))
        return 0

    @staticmethod
    def _prm_shape(prm_in):
        prm = np.asarray(prm_in, dtype=np.float32)
        sh = prm.shape
        if prm.ndim == 1:
            return prm, sh, 1, 1, sh[0]
        if prm.ndim == 2:
            return prm, sh, sh[0], 1, sh[1]
        if prm.ndim == 3:
            return prm, sh, sh[0], sh[1], sh[2]
        raise ValueError("calcmodchi2(): input parameter array has > 3 or < 1 dimensions")

    def calcmodchi2(self, prm_in, imodel=None):
        """Model values datm and chi^2 terms chi2m for the parameter sets in
        prm_in (1D [nptot], 2D [n, nptot] or 3D [nbeta, nseq, nptot])."""
        prm, sh, nbeta, nseq, nptot = self._prm_shape(prm_in)
        ndat = self.ndat
        ndatm = nbeta * nseq * ndat
        pcur = np.ascontiguousarray(prm.reshape((nbeta, nseq, nptot)))
        datm = np.zeros(ndatm, np.float32)
        chi2m = np.zeros((nbeta, nseq, ndat), np.float32)
        chi2c = np.zeros((nbeta, nseq), np.float32)
        flag = np.ones((nbeta, nseq), np.int32)
        imod = self.imodel if imodel is None else imodel
        mi.calcmodchi2(self.coor, self.dat, self.std2r, self.icoor, self.idat, datm, chi2m, pcur,
                       chi2c, flag, imod, self.ncoor, self.ndat, self.nicoor, self.nidat, ndatm,
                       nptot, nbeta, nseq)
        mi.reset_gpu()
        if len(sh) < 3:
            datm = datm.squeeze()
            chi2m = chi2m.squeeze()
        return datm, chi2m

    def reset_gpu(self):
        mi.reset_gpu()


class Mcgpu_Sgra(Mcgpu):
    """The Sgr A* crescent + Gaussian fit to visibility amplitudes and
    closure phases (imodel 1: sgra_model9, 2: sgra_model13)."""

    def __init__(self, uvfile=None, imodel=1, npass=2, nseq=14, nbeta=32, nburn=100, niter=100,
                 seed=1234, beta1=1.0, betan=0.0001, pdescr=None, ptotal=None, pmint=None,
                 pmaxt=None, ulam=None, vlam=None, blin=None, amp=None, phase=None, cphs=None,
                 cpix=None, uvcp=None, eamp=None, ecph=None, tsec=None, chan=None, wei=None,
                 wlam=None, nadj=100, use_cphs=True, model="sgra"):
        super().__init__(pdescr=pdescr, ptotal=ptotal, pmint=pmint, pmaxt=pmaxt, beta1=beta1,
                         betan=betan, seed=seed, imodel=imodel, npass=npass, nadj=nadj,
                         nbeta=nbeta, nseq=nseq, nburn=nburn, niter=niter, model=model)
        f32 = lambda x: None if x is None else np.asarray(x, np.float32)
        self.error = ""
        self.uvfile = uvfile
        self.imodel = imodel
        self.ulam, self.vlam, self.wlam = f32(ulam), f32(vlam), f32(wlam)
        self.uvcp, self.amp, self.phase = f32(uvcp), f32(amp), f32(phase)
        self.eamp, self.ecph = f32(eamp), f32(ecph)
        self.blin = None if blin is None else np.asarray(blin, np.int32)
        self.tsec, self.wei = f32(tsec), f32(wei)
        self.fsig = None
        self.chan = chan
        self.use_cphs = bool(use_cphs)
        if uvfile is not None:
            (self.ulam, self.vlam, self.wlam, self.amp, self.phase, self.blin, self.tsec,
             self.fsig, self.chan, self.wei) = read_uvdata(uvfile)
            self.ulam = 1e-3 * self.ulam
            self.vlam = 1e-3 * self.vlam
        elif self.amp is None:
            raise ValueError("Mcgpu_Sgra needs a uvfile or the amp, ulam and vlam arrays")
        if self.fsig is not None and not builtins.all(self.fsig):
            self.fsig[:] = 1.0        # noiseless simulation (src/imgpu.py:630)
        self.eamp = np.ones_like(self.amp)
        if eamp is None:
            if self.fsig is not None and builtins.all(self.fsig):
                self.eamp = np.copy(self.fsig)
            else:
                self.error = "Some sigmas in uv file are zeros." if self.fsig is not None \
                    else "1-sigma amplitude errors eamp not given"
                return
        elif np.isscalar(eamp):
            if eamp == 0:
                self.error = "1-sigma visibility amplitude error eamp is zero."
                return
            self.eamp[:] = eamp
        elif len(eamp) == len(self.amp):
            if not builtins.all(eamp):
                self.error = "Some of eamp elements are zero."
                return
            self.eamp = np.array(eamp, np.float32)
        else:
            self.error = ("number of 1-sigma errors in parameter eamp (%d) differs from number "
                          "of visibility amplitudes in self.amp (%d)." % (len(eamp), len(self.amp)))
            return
        self.base = np.sqrt(self.ulam ** 2 + self.vlam ** 2)
        self.cphs = None if cphs is None else np.asarray(cphs, np.float32)
        self.cpix = None if cpix is None else np.asarray(cpix, np.int32)
        self.trid = None
        self.tcphsec = None
        if self.phase is None or (np.all(self.phase == 0) and cphs is None):
            self.use_cphs = False
        self.nvis = nvis = np.int32(len(self.amp))
        self.nmph = nbeta * nseq * nvis
        self.cpExt = 0
        if self.use_cphs:
            if cphs is None:
                self.cpExt = 0
                self.cphs, self.cpix, self.trid, self.tcphsec = calc_closures(
                    self.phase, self.tsec, self.blin)
            else:
                self.cpExt = 1
            self.ncph = ncph = np.int32(len(self.cphs))
            self.vicp = np.hstack((self.amp, self.cphs))
            self.nvicp = nvis + ncph
            self.nchi2m = nchi2m = nbeta * nseq * self.nvicp
            self.npass = np.int32(2)
        else:
            self.ncph = ncph = 0
            self.vicp = np.copy(self.amp)
            self.nvicp = nvis
            self.nchi2m = nchi2m = nbeta * nseq * nvis
        if self.use_cphs:
            self.ecph = np.ones(ncph, np.float32)
            if ecph is None:
                self.error = "Closure phase 1-sigma error(s) not provided in parameter ecph."
                return
            elif np.isscalar(ecph):
                if ecph == 0:
                    self.error = "Closure phase 1-sigma error ecph is zero."
                    return
                self.ecph[:] = ecph
            elif len(ecph) == len(self.ecph):
                if not builtins.all(ecph):
                    self.error = "Some of ecph elements are zero."
                    return
                self.ecph = np.array(ecph, np.float32)
            else:
                self.error = ("number of 1-sigma errors in parameter ecph (%d) differs from "
                              "number of closure phases in self.cphs (%d)." % (len(ecph), ncph))
                return
        else:
            self.ecph = None
        self.ndat = ndat = np.int32(nvis + ncph)
        self.nidat = np.int32(3)
        self.ndatm = np.int32(nbeta * nseq * (ndat + nvis))
        self.seed = np.uint64(seed)
        self.dat = np.empty(ndat, np.float32)
        self.std2r = np.ones(ndat, np.float32)
        self.std2r[:nvis] = 1.0 / self.eamp ** 2
        if self.use_cphs:
            self.std2r[nvis:] = 1.0 / self.ecph ** 2
            if self.cpExt == 0:
                self.ncoor, self.nicoor = np.int32(2 * nvis), np.int32(3 * ncph)
            else:
                self.ncoor, self.nicoor = np.int32(2 * nvis + 4 * ncph), np.int32(0)
        else:
            self.ncoor, self.nicoor = np.int32(2 * nvis), np.int32(0)
        self.coor = np.empty(self.ncoor, np.float32)
        self.icoor = np.empty(self.nicoor, np.int32)
        self.idat = np.empty(3, np.int32)
        self.datm = np.zeros(self.ndatm, np.float32)
        self.chi2m = np.zeros((nbeta, nseq, ndat), np.float32)
        self.mvicp = np.zeros((nbeta, nseq, ndat), np.float32)
        self.mpha = np.zeros((nbeta, nseq, nvis), np.float32)
        self.coor[:2 * nvis] = np.vstack((self.ulam, self.vlam)).T.flatten()
        if self.use_cphs:
            if self.cpExt:
                self.coor[2 * nvis:] = np.asarray(self.uvcp, np.float32).flatten()
            else:
                self.icoor[:] = np.asarray(self.cpix).flatten()
            self.dat[:nvis] = self.amp
            self.dat[nvis:] = self.cphs
        else:
            self.dat[:] = self.amp
        self.idat[:] = nvis, nchi2m, self.cpExt

    def burnin_and_search(self):
        if self.error != "":
            print("Cannot burnin and search: first fix the error: " + self.error)
            return 1
        self._mcmcuda()
        self.mvicp = self.datm[:self.nchi2m].reshape((self.nbeta, self.nseq, self.ndat))
        self.mpha = self.datm[self.nchi2m:].reshape((self.nbeta, self.nseq, self.nvis))
        self.rate_acpt, self.rate_exch = _rates(self.n_acpt, self.n_exch, self.niter, self.nseq)
        self.chi2 = self.chi2_2d.flatten()
        self.pout = self.pout_4d[:, 0, :, :].reshape((self.nprm, self.nseq * self.niter))
        return 0

    def calcmodchi2(self, prm_in, imodel=None):
        """chi2c, mvicp (model amplitudes + closures), mpha (model phases),
        chi2m and datm for the parameter sets in prm_in."""
        if self.error != "":
            print("First fix the error: " + self.error)
            return 1
        prm, sh, nbeta, nseq, nptot = self._prm_shape(prm_in)
        ndat, nvis = self.ndat, self.nvis
        pcur = np.ascontiguousarray(prm.reshape((nbeta, nseq, nptot)))
        ndatm = nbeta * nseq * (ndat + nvis)
        datm = np.zeros(ndatm, np.float32)
        chi2m = np.zeros((nbeta, nseq, ndat), np.float32)
        chi2c = np.zeros((nbeta, nseq), np.float32)
        flag = np.ones((nbeta, nseq), np.int32)
        imod = imodel if imodel in (1, 2) else self.imodel
        mi.calcmodchi2(self.coor, self.dat, self.std2r, self.icoor, self.idat, datm, chi2m, pcur,
                       chi2c, flag, imod, self.ncoor, self.ndat, self.nicoor, self.nidat, ndatm,
                       nptot, nbeta, nseq)
        mi.reset_gpu()
        nchi2m = nbeta * nseq * ndat
        mvicp = datm[:nchi2m].reshape((nbeta, nseq, ndat))
        mpha = datm[nchi2m:].reshape((nbeta, nseq, nvis))
        if len(sh) == 1:
            chi2c = chi2c[0, 0]
            mvicp, mpha, chi2m = mvicp.flatten(), mpha.flatten(), chi2m.flatten()
        return chi2c, mvicp, mpha, chi2m, datm

    def calcmodel(self, ulam, vlam, prm_in, imodel=2, uv_layout="reference"):
        """Model amplitudes and phases on a 2-D (u, v) grid for the parameter
        sets in prm_in.  uv_layout="reference" packs coor as the reference
        does ([u..., v...]); "interleaved" gives the model at the given points."""
        ul, vl = np.asarray(ulam).flatten(), np.asarray(vlam).flatten()
        uv_sh = np.shape(ulam)
        udim, vdim = uv_sh[0], uv_sh[1]
        prm, psh, nbeta, nseq, nptot = self._prm_shape(prm_in)
        if len(psh) == 1:
            mamp_sh = uv_sh
        elif len(psh) == 2:
            mamp_sh = (nbeta, udim, vdim)
        else:
            mamp_sh = (nbeta, nseq, udim, vdim)
        imod = imodel if imodel in (1, 2) else self.imodel
        pcur = np.ascontiguousarray(prm.reshape((nbeta, nseq, nptot)))
        ndat = nvis = len(ul)
        ncoor = 2 * nvis
        ndatm = nbeta * nseq * 2 * nvis
        nmamp = nbeta * nseq * nvis
        datm = np.zeros(ndatm, np.float32)
        coor = np.empty(ncoor, np.float32)
        if uv_layout == "interleaved":
            coor[0::2], coor[1::2] = ul, vl
        else:
            coor[:nvis], coor[nvis:] = ul, vl
        idat = np.array((nvis, 0, 0), np.int32)
        mi.calcmodel(coor, idat, datm, pcur, imod, ncoor, ndat, len(idat), ndatm, nptot, nbeta,
                     nseq)
        mi.reset_gpu()
        return datm[:nmamp].reshape(mamp_sh), datm[nmamp:].reshape(mamp_sh)


# ---------------------------------------------------------------------------
# data helpers
# ---------------------------------------------------------------------------

def cbinom(n, m):
    """Number of m-subsets of an n-set; -1 for invalid arguments."""
    if n < 0 or m < 0 or m > n:
        return -1
    from math import comb
    return comb(n, m)


def combgen(n, m):
    """All m-subsets of range(n) as rows of a [cbinom(n, m), m] int array, in
    lexicographic order (the reference's recursive generator's order)."""
    rows = list(itertools.combinations(range(n), m))
    return np.array(rows, dtype=int).reshape(len(rows), m)


def find_triangles(antennas):
    """All antenna triangles and their ids a1 + PK3I*(a2 + PK3I*a3)."""
    ant = np.asarray(antennas)
    itri = combgen(ant.size, 3)
    tri = ant[itri] if len(itri) else np.empty((0, 3), int)
    trid = tri[:, 0] + PK3I * (tri[:, 1] + PK3I * tri[:, 2])
    return tri, trid


def get_time_indices(tsec):
    """Begin / end row indices of the equal-time spans of tsec that hold at
    least 3 rows."""
    tsec = np.asarray(tsec)
    itim = np.where(np.diff(tsec))[0] + 1
    itim = np.hstack((0, itim, len(tsec)))
    ditim = np.diff(itim)
    ibeg = [int(itim[i]) for i in range(len(ditim)) if ditim[i] >= 3]
    iend = [int(itim[i + 1]) for i in range(len(ditim)) if ditim[i] >= 3]
    return ibeg, iend


_TRIANGLES = {}


def _triangle_slots(na):
    """All index triplets i < j < k of range(na), in itertools.combinations
    order, as an [ntri, 3] array (cached per na)."""
    t = _TRIANGLES.get(na)
    if t is None:
        t = np.array(list(itertools.combinations(range(na), 3)), np.int64).reshape(-1, 3)
        _TRIANGLES[na] = t
    return t


def calc_closures(phase, tsec, blin):
    """Closure phases phi(a1a2) + phi(a1a3) - phi(a2a3) of every antenna
    triangle of every equal-time span: returns cphs, cpix (row triplets),
    trid (triangle ids) and tcphsec (times).

    The reference's loop (src/imgpu.py:1229-1325), vectorised per span: the
    span's antennas sorted (np.unique), the first row of every baseline a-b
    in a [na, na] table, all triangles of the span at once in
    itertools.combinations order.  As in the reference, every triangle of a
    span's antennas must have its three baselines in the span (IndexError
    otherwise)."""
    empty = (np.array([], np.float32), np.zeros((0, 3), np.int32), np.array([], np.int32),
             np.array([], np.float32))
    if len(phase) < 3:
        return empty
    ibeg, iend = get_time_indices(tsec)
    if not ibeg:
        return empty
    phase = np.asarray(phase)
    bls = np.asarray(blin)
    cphs, cpix, trid, tcp = [], [], [], []
    for i0, i1 in zip(ibeg, iend):
        bl = bls[i0:i1].astype(np.int64)
        ant = np.unique(bl)
        na = ant.size
        if na < 3:
            continue
        slot = np.searchsorted(ant, bl)
        key = slot[:, 0] * na + slot[:, 1]
        ukey, first = np.unique(key, return_index=True)   # first row of each baseline
        row = np.full(na * na, -1, np.int64)
        row[ukey] = i0 + first
        tri = _triangle_slots(na)
        ib1 = row[tri[:, 0] * na + tri[:, 1]]
        ib2 = row[tri[:, 0] * na + tri[:, 2]]
        ib3 = row[tri[:, 1] * na + tri[:, 2]]
        if (ib1 < 0).any() or (ib2 < 0).any() or (ib3 < 0).any():
            raise IndexError("calc_closures: a triangle of the span at rows %d-%d lacks one of "
                             "its baselines" % (i0, i1 - 1))
        ph = phase[ib1] + phase[ib2] - phase[ib3]
        cphs.append(np.arctan2(np.sin(ph), np.cos(ph)))
        cpix.append(np.stack([ib1, ib2, ib3], 1))
        a = ant[tri]
        trid.append(a[:, 0] + PK3I * (a[:, 1] + PK3I * a[:, 2]))
        tcp.append(np.full(tri.shape[0], tsec[i0], float))
    if not cphs:
        return empty
    return (np.concatenate(cphs).astype(np.float32),
            np.concatenate(cpix).astype(np.int32).reshape(-1, 3),
            np.concatenate(trid).astype(np.int32), np.concatenate(tcp))


def count_lines(filename, numcount=None):
    """Number of lines of a text file, or (numcount given) of the lines that
    hold exactly numcount numbers."""
    n = 0
    with open(filename, "r") as f:
        for row in f:
            if numcount is None or len(_NUM.findall(row)) == numcount:
                n += 1
    return n


def read_uvdata(uv_file):
    """Read a uv data text file (one visibility per row: time, u, v, w in
    kilolambda, baseline aa-bb, channel, (amplitude, phase in degrees), weight,
    sigma).  Returns ulam, vlam, wlam (megalambda), amp, phase (radians),
    blin [n, 2], tsec (seconds since the epoch), sig, chan, wei."""
    n = count_lines(uv_file)
    amp, phase, sig = (np.zeros(n, np.float32) for _ in range(3))
    ulam, vlam, wlam, wei, tsec = (np.zeros(n, np.float32) for _ in range(5))
    chan = np.zeros(n, np.int32)
    blin = np.zeros((n, 2), np.int32)
    i = 0
    with open(uv_file, "r") as fp:
        for row in fp:
            nums = _NUM.findall(row)
            if len(nums) != 15:
                continue
            u, v, w = float(nums[5]), float(nums[6]), float(nums[7])
            chan[i], amp[i], phase[i] = float(nums[10]), float(nums[11]), float(nums[12])
            weig, sig[i] = float(nums[13]), float(nums[14])
            if weig != 0.0:
                wei[i] = weig
                ulam[i], vlam[i], wlam[i] = 1e-3 * u, 1e-3 * v, 1e-3 * w
                phase[i] = np.radians(phase[i])
                t = timegm(strptime(row[:17], "%Y:%j:%H:%M:%S"))
                if row[18:20].isdigit():
                    t = t + 0.01 * np.float32(row[18:20])
                tsec[i] = t
                blin[i, :] = int(nums[8]), -int(nums[9])
            i += 1
    if i == 0:
        e = np.array([], dtype=np.int32)
        return e, e, e, e, e, e, e, e, e, e
    return (ulam[:i], vlam[:i], wlam[:i], amp[:i], phase[:i], blin[:i], tsec[:i], sig[:i],
            chan, wei)
