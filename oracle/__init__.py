"""CPU oracle for the cuda_mcmc MCMC-RE hot path.

TEST INFRASTRUCTURE ONLY.  This package is the checker: the tests,
``__graft_entry__.smoke()`` and bench.py's ``cpu_baseline`` / ``--impl
reference`` legs load it; the ``cuda_mcmc_gb300`` product never imports it.

``oracle.c`` restates, in C with FP64 model arithmetic, the reference's
models (examples/sgra_model_fit/model.cuh, examples/search_Rosenbrock/model.cuh,
examples/solvsys/model.cuh), its chi^2 term (src/gpu_mcmc.cu:299-323) and its
sweep (src/gpu_mcmc.cu:245-626 in the order of run_mcmc, :682-763) driven by
injected random streams.  ``oracle/ref_build.py`` additionally compiles the
reference's own ``model.cuh`` files and kernels for the host (into
``oracle/_ref/``) so that this restatement can be pinned against them.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")

MODEL_SGRA, MODEL_ROSEN, MODEL_SOLVSYS, MODEL_NLSYS = 1, 2, 3, 4
MODEL_IDS = {"sgra": MODEL_SGRA, "rosenbrock": MODEL_ROSEN,
             "solvsys": MODEL_SOLVSYS, "nlsys": MODEL_NLSYS}
OK, ERR_ARG, ERR_STREAM = 0, 1, 2

_lib = None


def build(force: bool = False) -> str:
    """Compile oracle.c into oracle/_build/liboracle.so (gcc, -O2, no fast-math)."""
    src = os.path.join(HERE, "oracle.c")
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src)):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    # -ffp-contract=off: keep every float expression as written; the fused
    # multiply-adds the restatement wants are spelled out with fmaf().
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-std=c99", "-ffp-contract=off",
           "-D_DEFAULT_SOURCE", src, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_bp = C.POINTER(C.c_byte)


class _Problem(C.Structure):
    _fields_ = [("model", C.c_int), ("imodel", C.c_int), ("ncoor", C.c_int),
                ("ndat", C.c_int), ("nicoor", C.c_int), ("nidat", C.c_int),
                ("nptot", C.c_int), ("npass", C.c_int),
                ("coor", _fp), ("dat", _fp), ("std2r", _fp),
                ("icoor", _ip), ("idat", _ip), ("arith", C.c_int)]


class _Streams(C.Structure):
    _fields_ = [("u", _fp), ("n", _fp), ("lu", C.c_int), ("ln", C.c_int),
                ("cu", _ip), ("cn", _ip), ("overflow", C.c_int)]


class _SweepState(C.Structure):
    _fields_ = [("nprm", C.c_int), ("nadj", C.c_int), ("nbeta", C.c_int),
                ("nseq", C.c_int), ("niter_total", C.c_int),
                ("pdescr", _ip), ("ivar", _ip), ("invar", _ip),
                ("pmint", _fp), ("pmaxt", _fp), ("beta", _fp),
                ("pcur", _fp), ("chi2c", _dp), ("flag", _ip), ("ptent", _fp),
                ("ptentn", _ip), ("pstp", _fp), ("n_acpt", _ip), ("n_exch", _ip),
                ("n_cnt", _ip), ("n_hist", _ip), ("tcur", _ip),
                ("pout", _fp), ("tout", _ip), ("chi2", _fp),
                ("datm", _dp), ("chi2m", _dp),
                ("tr_dec", _bp), ("tr_margin", _dp), ("tr_xk", _bp),
                ("tr_xdec", _bp), ("tr_xmargin", _dp),
                ("prop_mode", C.c_int), ("prop_chol", _fp)]


def _declare(L):
    L.or_sgra_vis.argtypes = [C.c_int, _dp, C.c_int, _dp, _dp, _dp, _dp]
    L.or_sgra_vis.restype = C.c_int
    L.or_calc_modchi2.argtypes = [C.POINTER(_Problem), C.c_int, _fp, _ip, _dp, _dp, _dp, _dp]
    L.or_calc_modchi2.restype = C.c_int
    L.or_calc_model.argtypes = [C.POINTER(_Problem), C.c_int, _fp, _dp, _dp]
    L.or_calc_model.restype = C.c_int
    L.or_chi2_d.argtypes = [C.POINTER(_Problem), C.c_int, _dp, _dp]
    L.or_chi2_d.restype = C.c_int
    L.or_chi2_f32.argtypes = [C.POINTER(_Problem), C.c_int, _fp, _dp]
    L.or_chi2_f32.restype = C.c_int
    L.or_sweep.argtypes = [C.POINTER(_Problem), C.POINTER(_SweepState),
                           C.POINTER(_Streams), C.c_int, C.c_int, C.c_int, C.c_int]
    L.or_sweep.restype = C.c_int
    for f in ("or_sizeof_problem", "or_sizeof_sweep_state", "or_sizeof_streams"):
        getattr(L, f).restype = C.c_int
    assert L.or_sizeof_problem() == C.sizeof(_Problem)
    assert L.or_sizeof_sweep_state() == C.sizeof(_SweepState)
    assert L.or_sizeof_streams() == C.sizeof(_Streams)


def _ptr(a, t):
    if a is None:
        return C.cast(None, t)
    assert a.flags["C_CONTIGUOUS"], "oracle buffers must be C-contiguous"
    return a.ctypes.data_as(t)


@dataclass
class Problem:
    """A model + data set in the reference's array conventions."""
    model: str
    coor: np.ndarray
    dat: np.ndarray
    std2r: np.ndarray
    icoor: np.ndarray
    idat: np.ndarray
    nptot: int
    imodel: int = 1
    npass: int = 1
    arith: int = 0          # 0: FP64 model (the checker); 1: float32, as the reference computes
    _keep: list = field(default_factory=list, repr=False)

    def __post_init__(self):
        self.coor = np.ascontiguousarray(self.coor, np.float32)
        self.dat = np.ascontiguousarray(self.dat, np.float32)
        self.std2r = np.ascontiguousarray(self.std2r, np.float32)
        self.icoor = np.ascontiguousarray(self.icoor, np.int32)
        self.idat = np.ascontiguousarray(self.idat, np.int32)
        if self.icoor.size == 0:
            self.icoor = np.zeros(1, np.int32)
        if self.idat.size == 0:
            self.idat = np.zeros(1, np.int32)

    @property
    def ndat(self):
        return int(self.dat.size)

    @property
    def nvis(self):
        return int(self.idat[0]) if self.model == "sgra" else 0

    def c(self):
        return _Problem(MODEL_IDS[self.model], int(self.imodel), int(self.coor.size),
                        self.ndat, int(self.icoor.size), int(self.idat.size),
                        int(self.nptot), int(self.npass),
                        _ptr(self.coor, _fp), _ptr(self.dat, _fp), _ptr(self.std2r, _fp),
                        _ptr(self.icoor, _ip), _ptr(self.idat, _ip), int(self.arith))


def sgra_vis(imodel, prm, u, v):
    """FP64 sgra_model9 (imodel=1) / sgra_model13 (imodel=2) at uv points."""
    u = np.ascontiguousarray(u, np.float64).ravel()
    v = np.ascontiguousarray(v, np.float64).ravel()
    prm = np.ascontiguousarray(prm, np.float64).ravel()
    amp = np.empty_like(u)
    pha = np.empty_like(u)
    rc = lib().or_sgra_vis(int(imodel), _ptr(prm, _dp), u.size, _ptr(u, _dp),
                           _ptr(v, _dp), _ptr(amp, _dp), _ptr(pha, _dp))
    if rc != OK:
        raise ValueError("or_sgra_vis: imodel must be 1 or 2")
    return amp, pha


def calc_modchi2(pb: Problem, pcur, flag=None, chi2m=None):
    """FP64 calc_modchi2 for pcur[..., nptot]; returns (datm, phase, chi2m, chi2c)."""
    pcur = np.ascontiguousarray(pcur, np.float32)
    nrep = pcur.size // pb.nptot
    datm = np.zeros((nrep, pb.ndat), np.float64)
    phase = np.zeros((nrep, max(pb.nvis, 1)), np.float64)
    chi2m = (np.zeros((nrep, pb.ndat), np.float64) if chi2m is None
             else np.ascontiguousarray(chi2m, np.float64).reshape(nrep, pb.ndat).copy())
    chi2c = np.zeros(nrep, np.float64)
    fl = None if flag is None else np.ascontiguousarray(flag, np.int32).ravel()
    cp = pb.c()
    rc = lib().or_calc_modchi2(C.byref(cp), nrep, _ptr(pcur, _fp), _ptr(fl, _ip),
                               _ptr(datm, _dp), _ptr(phase, _dp), _ptr(chi2m, _dp),
                               _ptr(chi2c, _dp))
    if rc != OK:
        raise ValueError("or_calc_modchi2 failed (%d)" % rc)
    return datm, phase[:, :pb.nvis], chi2m, chi2c


def calc_model(pb: Problem, pcur):
    """FP64 calc_model (pass 0 only); returns (datm, phase)."""
    pcur = np.ascontiguousarray(pcur, np.float32)
    nrep = pcur.size // pb.nptot
    datm = np.zeros((nrep, pb.ndat), np.float64)
    phase = np.zeros((nrep, max(pb.nvis, 1)), np.float64)
    cp = pb.c()
    rc = lib().or_calc_model(C.byref(cp), nrep, _ptr(pcur, _fp), _ptr(datm, _dp),
                             _ptr(phase, _dp))
    if rc != OK:
        raise ValueError("or_calc_model failed (%d)" % rc)
    return datm, phase[:, :pb.nvis]


def chi2_d(pb: Problem, p):
    """FP64 chi^2 at FP64 parameters p[..., nptot] (calc_modchi2's terms,
    src/gpu_mcmc.cu:305-323, without rounding p to float)."""
    p = np.ascontiguousarray(p, np.float64)
    shape = p.shape[:-1]
    p = p.reshape(-1, pb.nptot)
    out = np.zeros(p.shape[0], np.float64)
    cp = pb.c()
    L = lib()
    # rows split over the host threads (ctypes releases the GIL)
    nth = max(1, min(os.cpu_count() or 1, p.shape[0] // 8))
    bounds = np.linspace(0, p.shape[0], nth + 1).astype(int)

    def part(i):
        a, b = bounds[i], bounds[i + 1]
        if b <= a:
            return OK
        return L.or_chi2_d(C.byref(cp), int(b - a), _ptr(p[a:b], _dp), _ptr(out[a:b], _dp))

    if nth == 1:
        rcs = [part(0)]
    else:
        from concurrent.futures import ThreadPoolExecutor
        with ThreadPoolExecutor(nth) as ex:
            rcs = list(ex.map(part, range(nth)))
    if any(rc != OK for rc in rcs):
        raise ValueError("or_chi2_d failed (%s)" % rcs)
    return out.reshape(shape)


def chi2_f32(pb: Problem, pcur):
    """chi^2 of parameter sets in the float32 arithmetic of the reference's
    kernels (sgra_model9 only): float64 [nrep]."""
    pcur = np.ascontiguousarray(pcur, np.float32)
    nrep = pcur.size // pb.nptot
    out = np.zeros(nrep, np.float64)
    cp = pb.c()
    if lib().or_chi2_f32(C.byref(cp), nrep, _ptr(pcur, _fp), _ptr(out, _dp)) != OK:
        raise ValueError("or_chi2_f32: sgra_model9 problems only")
    return out


def chi2_grad_fd(pb: Problem, p, h):
    """Central differences of chi2_d: (chi2(p + h_k e_k) - chi2(p - h_k e_k)) / 2 h_k
    for every parameter k; p[nrep, nptot], h[nptot] -> [nrep, nptot]."""
    p = np.asarray(p, np.float64).reshape(-1, pb.nptot)
    h = np.broadcast_to(np.asarray(h, np.float64), (pb.nptot,))
    n, k = p.shape
    pp = np.repeat(p[:, None, :], 2 * k, axis=1)
    for j in range(k):
        pp[:, 2 * j, j] += h[j]
        pp[:, 2 * j + 1, j] -= h[j]
    c = chi2_d(pb, pp)
    return (c[:, 0::2] - c[:, 1::2]) / (2.0 * h)


@dataclass
class SweepState:
    """Sampler state in the reference's layouts (see src/gpu_mcmc.cu:100-188)."""
    pdescr: np.ndarray
    ivar: np.ndarray
    invar: np.ndarray
    pmint: np.ndarray
    pmaxt: np.ndarray
    beta: np.ndarray
    pcur: np.ndarray      # [nbeta, nseq, nptot] f32
    chi2c: np.ndarray     # [nbeta, nseq] f64
    flag: np.ndarray
    ptent: np.ndarray
    ptentn: np.ndarray
    pstp: np.ndarray      # [nprm, nbeta, nseq] f32
    n_acpt: np.ndarray
    n_exch: np.ndarray
    n_cnt: np.ndarray
    n_hist: np.ndarray    # [nadj, nprm, nbeta, nseq]
    tcur: np.ndarray
    pout: np.ndarray      # [nprm, nbeta, nseq, niter_total]
    tout: np.ndarray
    chi2: np.ndarray      # [nseq, niter_total]
    datm: np.ndarray = None
    chi2m: np.ndarray = None

    @property
    def nbeta(self):
        return self.pcur.shape[0]

    @property
    def nseq(self):
        return self.pcur.shape[1]

    @property
    def nprm(self):
        return int(self.ivar.size)

    def copy(self):
        kw = {k: (None if v is None else np.array(v, copy=True)) for k, v in self.__dict__.items()}
        return SweepState(**kw)


def new_state(pdescr, pmint, pmaxt, beta, nseq, niter, nadj=100, ptotal=None,
              pstp=None, ndat=0):
    """Initial state following imgpu.Mcgpu.__init__ (src/imgpu.py:259-424)."""
    pdescr = np.asarray(pdescr, np.int32)
    nptot = pdescr.size
    ivar = np.where(pdescr != 0)[0].astype(np.int32)
    nprm = ivar.size
    invar = np.full(nptot, -1, np.int32)
    invar[ivar] = np.arange(nprm, dtype=np.int32)
    pmint = np.asarray(pmint, np.float32)
    pmaxt = np.asarray(pmaxt, np.float32)
    beta = np.asarray(beta, np.float32)
    nbeta = beta.size
    ptotal = np.zeros(nptot, np.float32) if ptotal is None else np.asarray(ptotal, np.float32)
    pcur = np.empty((nbeta, nseq, nptot), np.float32)
    pcur[:] = ptotal
    pcur[:, :, ivar] = pmint[ivar] + (pmaxt[ivar] - pmint[ivar]) / np.float32(2.0)
    if pstp is None:
        st = np.empty((nprm, nbeta, nseq), np.float32)
        st[:] = ((pmaxt[ivar] - pmint[ivar]) / 50.0).astype(np.float32)[:, None, None]
    else:
        st = np.ascontiguousarray(pstp, np.float32).copy()
    tcur = np.empty((nbeta, nseq), np.int32)
    tcur[:] = np.arange(nbeta, dtype=np.int32)[:, None]
    return SweepState(
        pdescr=pdescr, ivar=ivar, invar=invar, pmint=pmint, pmaxt=pmaxt, beta=beta,
        pcur=pcur, chi2c=np.zeros((nbeta, nseq), np.float64),
        flag=np.zeros((nbeta, nseq), np.int32), ptent=np.zeros((nbeta, nseq), np.float32),
        ptentn=np.zeros((nbeta, nseq), np.int32), pstp=st,
        n_acpt=np.zeros((nprm, nbeta, nseq), np.int32), n_exch=np.zeros((nbeta, nseq), np.int32),
        n_cnt=np.ones((nprm, nbeta, nseq), np.int32),
        n_hist=np.zeros((nadj, nprm, nbeta, nseq), np.int32), tcur=tcur,
        pout=np.zeros((nprm, nbeta, nseq, max(niter, 1)), np.float32),
        tout=np.zeros((nbeta, nseq, max(niter, 1)), np.int32),
        chi2=np.zeros((nseq, max(niter, 1)), np.float32),
        datm=np.zeros((nbeta, nseq, max(ndat, 1)), np.float64),
        chi2m=np.zeros((nbeta, nseq, max(ndat, 1)), np.float64))


@dataclass
class Streams:
    """Injected uniforms (0,1] and normals per replica, with cursors."""
    u: np.ndarray    # [nrep, lu] f32
    n: np.ndarray    # [nrep, ln] f32
    cu: np.ndarray = None
    cn: np.ndarray = None

    def __post_init__(self):
        self.u = np.ascontiguousarray(self.u, np.float32)
        self.n = np.ascontiguousarray(self.n, np.float32)
        if self.cu is None:
            self.cu = np.zeros(self.u.shape[0], np.int32)
        if self.cn is None:
            self.cn = np.zeros(self.n.shape[0], np.int32)


def make_streams(nrep, lu, ln, seed):
    """Seeded uniforms strictly inside (0,1) and standard normals (float32)."""
    rng = np.random.default_rng(seed)
    u = rng.random((nrep, lu), dtype=np.float32)
    u = np.where(u == 0.0, np.float32(0.5), u).astype(np.float32)
    n = rng.standard_normal((nrep, ln), dtype=np.float32)
    return Streams(u, n)


@dataclass
class Trace:
    dec: np.ndarray
    margin: np.ndarray
    xk: np.ndarray
    xdec: np.ndarray
    xmargin: np.ndarray


def sweep(pb: Problem, st: SweepState, rs: Streams, do_init, nburn, niter, itr0=0,
          trace=False, prop_chol=None):
    """Run the restated sweep in place on ``st``; returns a Trace or None.
    ``prop_chol`` [nseq, nprm, nprm] switches to the library's block
    proposals (lower Cholesky factor per sequence, scaled by pstp[0])."""
    nrep = st.nbeta * st.nseq
    nstep = nburn + niter
    tr = None
    if trace:
        tr = Trace(dec=np.zeros((nstep, st.nprm, nrep), np.int8),
                   margin=np.zeros((nstep, st.nprm, nrep), np.float64),
                   xk=np.zeros((nstep, st.nseq, st.nbeta), np.int8),
                   xdec=np.zeros((nstep, st.nseq, st.nbeta), np.int8),
                   xmargin=np.zeros((nstep, st.nseq, st.nbeta), np.float64))
    for name in ("pcur", "flag", "ptent", "ptentn", "pstp", "n_acpt", "n_exch", "n_cnt",
                 "n_hist", "tcur", "pout", "tout", "chi2"):
        assert getattr(st, name).flags["C_CONTIGUOUS"], name
    st.chi2c = np.ascontiguousarray(st.chi2c, np.float64)
    chol = None if prop_chol is None else np.ascontiguousarray(prop_chol, np.float32)
    if chol is not None and chol.shape != (st.nseq, st.nprm, st.nprm):
        raise ValueError("prop_chol must be [nseq, nprm, nprm]")
    cst = _SweepState(
        st.nprm, int(st.n_hist.shape[0]), st.nbeta, st.nseq, int(st.pout.shape[-1]),
        _ptr(st.pdescr, _ip), _ptr(st.ivar, _ip), _ptr(st.invar, _ip),
        _ptr(st.pmint, _fp), _ptr(st.pmaxt, _fp), _ptr(st.beta, _fp),
        _ptr(st.pcur, _fp), _ptr(st.chi2c, _dp), _ptr(st.flag, _ip), _ptr(st.ptent, _fp),
        _ptr(st.ptentn, _ip), _ptr(st.pstp, _fp), _ptr(st.n_acpt, _ip), _ptr(st.n_exch, _ip),
        _ptr(st.n_cnt, _ip), _ptr(st.n_hist, _ip), _ptr(st.tcur, _ip),
        _ptr(st.pout, _fp), _ptr(st.tout, _ip), _ptr(st.chi2, _fp),
        _ptr(st.datm, _dp), _ptr(st.chi2m, _dp),
        _ptr(tr.dec if tr else None, _bp), _ptr(tr.margin if tr else None, _dp),
        _ptr(tr.xk if tr else None, _bp), _ptr(tr.xdec if tr else None, _bp),
        _ptr(tr.xmargin if tr else None, _dp),
        0 if prop_chol is None else 1, _ptr(chol, _fp))
    cs = _Streams(_ptr(rs.u, _fp), _ptr(rs.n, _fp), rs.u.shape[1], rs.n.shape[1],
                  _ptr(rs.cu, _ip), _ptr(rs.cn, _ip), 0)
    cp = pb.c()
    rc = lib().or_sweep(C.byref(cp), C.byref(cst), C.byref(cs), int(do_init), int(nburn),
                        int(niter), int(itr0))
    if rc == ERR_STREAM:
        raise RuntimeError("oracle sweep: injected random stream exhausted")
    if rc != OK:
        raise ValueError("oracle sweep: bad arguments (%d)" % rc)
    return tr
