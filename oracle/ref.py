"""ctypes access to oracle/_ref/libref_<model>.so (the reference's own kernels
compiled for the CPU by oracle/ref_build.py).

TEST INFRASTRUCTURE ONLY: used in this container to pin the oracle and to
generate the committed fixtures under tests/golden/.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import ref_build
from . import Problem, SweepState, Streams

_libs = {}
_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)


def available(model: str) -> bool:
    return os.path.exists(ref_build.lib_path(model)) or ref_build.available()


def lib(model: str):
    if model not in _libs:
        path = ref_build.lib_path(model)
        if not os.path.exists(path):
            ref_build.build()
        L = C.CDLL(path)
        L.ref_mcmc.restype = C.c_int
        L.ref_calc_modchi2.restype = C.c_int
        L.ref_calc_model.restype = C.c_int
        _libs[model] = L
    return _libs[model]


def _f(a):
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_fp)


def _i(a):
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_ip)


def calc_modchi2(pb: Problem, pcur):
    """The reference's calc_modchi2 on the CPU; returns (datm, chi2m, chi2c) float32."""
    pcur = np.ascontiguousarray(pcur, np.float32)
    nrep = pcur.size // pb.nptot
    nvis = pb.nvis
    ndatm = nrep * (pb.ndat + nvis)
    datm = np.zeros(ndatm, np.float32)
    chi2m = np.zeros(nrep * pb.ndat, np.float32)
    chi2c = np.zeros(nrep, np.float32)
    flag = np.ones(nrep, np.int32)
    rc = lib(pb.model).ref_calc_modchi2(
        _f(pb.coor), _f(pb.dat), _f(pb.std2r), _i(pb.icoor), _i(pb.idat), _f(datm),
        _f(chi2m), _f(pcur), _f(chi2c), _i(flag), int(pb.imodel), int(pb.coor.size),
        pb.ndat, int(pb.icoor.size), int(pb.idat.size), ndatm, int(pb.nptot), nrep, 1)
    if rc:
        raise RuntimeError("ref_calc_modchi2 failed")
    return datm, chi2m.reshape(nrep, pb.ndat), chi2c


def sweep(pb: Problem, st: SweepState, rs: Streams, do_init, nburn, niter, itr0=0):
    """The reference's kernels in run_mcmc order, on the CPU, with injected
    streams.  Updates ``st`` in place (chi2c is kept float32 internally)."""
    nrep = st.nbeta * st.nseq
    nvis = pb.nvis
    ndatm = nrep * (pb.ndat + nvis)
    datm = np.zeros(ndatm, np.float32)
    chi2m = np.zeros(nrep * pb.ndat, np.float32)
    chi2c = np.ascontiguousarray(st.chi2c, np.float32)
    cursors = np.ascontiguousarray(np.stack([rs.cu, rs.cn], axis=1), np.int32)
    ptotal = np.zeros(pb.nptot, np.float32)
    rc = lib(pb.model).ref_mcmc(
        _f(pb.coor), _f(pb.dat), _f(pb.std2r), _i(pb.icoor), _i(pb.idat), _f(datm), _f(chi2m),
        _i(st.pdescr), _i(st.ivar), _i(st.invar), _f(ptotal), _f(st.pmint), _f(st.pmaxt),
        _f(st.pout), _i(st.tout), _f(st.chi2), _f(chi2c), _i(st.tcur), _i(st.flag),
        _i(st.n_acpt), _i(st.n_exch), _i(st.n_cnt), _i(st.n_hist), _f(st.beta), _f(st.pstp),
        _f(st.ptent), _i(st.ptentn), _f(st.pcur), _i(cursors), _f(rs.u), _f(rs.n),
        int(rs.u.shape[1]), int(rs.n.shape[1]), int(pb.imodel), int(pb.coor.size), pb.ndat,
        int(pb.icoor.size), int(pb.idat.size), ndatm, int(pb.nptot), st.nprm,
        int(st.n_hist.shape[0]), int(pb.npass), st.nbeta, st.nseq, int(nburn), int(niter),
        int(do_init), int(itr0), int(st.pout.shape[-1]))
    if rc == 2:
        raise RuntimeError("reference sweep: injected random stream exhausted")
    if rc:
        raise RuntimeError("ref_mcmc failed")
    rs.cu[:] = cursors[:, 0]
    rs.cn[:] = cursors[:, 1]
    st.chi2c = chi2c.astype(np.float64)
    return datm, chi2m
