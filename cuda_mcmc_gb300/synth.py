"""Seeded synthetic workloads in the reference's array conventions.

Each generator returns a :class:`Workload`: the model name, the data arrays
exactly as ``mcmc_interf.mcmcuda`` takes them (``coor, dat, std2r, icoor,
idat``), the parameter description (``pdescr, pmint, pmaxt, ptotal``) and the
sampler sizes.  The shapes and value distributions are the five benchmark
workloads of this project:

1. N-dimensional Rosenbrock (N=4) in the reference's Rosenbrock convention:
   one datum, ``dat = 0``, model value f(x) so chi^2 = f(x)^2
   (examples/search_Rosenbrock/model.cuh:40-41 generalised to N dims).
2. The n=8 nonlinear system r_k = sum_j A_kj sin x_j + B_kj x_j^2 - b_k.
3. Sgr A* crescent + Gaussian (sgra_model9): 2000 visibility amplitudes at
   |uv| ~ U(0.5, 8) Glambda with uniform position angles, 600 closure phases
   on random triangles of those points, amplitude noise N(0, 0.03) relative
   and closure-phase noise N(0, 5 deg).
4. The same model at 20000 visibilities and 6000 closure phases.
5. 1024 independent crescent fits with nvis ~ logU(500, 50000) and
   ncph = 0.3 nvis.

Amplitude sigmas are 0.03*|V_true| + 0.002 Jy: the additive floor keeps the
weights finite at visibility nulls, where a purely relative sigma would make
1/sigma^2 unbounded.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

# sgra_model9 parameter order (examples/sgra_model_fit/model.cuh:348-356)
SGRA9_NAMES = ("Zsp", "Re", "rq", "ecc", "fade", "gax", "aq", "gq", "th")
SGRA9_PMIN = np.array([1.0, 20.0, 0.0, 0.0, 0.0, 0.1, 0.05, 0.0, -np.pi], np.float32)
SGRA9_PMAX = np.array([3.0, 40.0, 0.99, 1.0, 1.0, 2.5, 1.0, 1.0, np.pi], np.float32)
SGRA9_TRUTH_LO = np.array([1.5, 25.0, 0.3, 0.2, 0.2, 0.3, 0.3, 0.1, -2.5])
SGRA9_TRUTH_HI = np.array([2.5, 35.0, 0.7, 0.8, 0.8, 1.5, 0.9, 0.5, 2.5])
SGRA9_PDESCR = np.array([1, 1, 1, 1, 1, 1, 1, 1, 2], np.int32)


def geometric_betas(nbeta: int, beta1: float = 1.0, betan: float = 1e-4) -> np.ndarray:
    """beta[i] = beta1 * (betan/beta1)^(i/(nbeta-1)), as imgpu.Mcgpu does
    (src/imgpu.py:412-418)."""
    if nbeta == 1:
        return np.array([beta1], np.float32)
    bstp = (betan / beta1) ** (1.0 / np.float32(nbeta - 1))
    return np.array([beta1 * bstp ** i for i in range(nbeta)], np.float32)


@dataclass
class Workload:
    name: str
    model: str                 # built-in model library: sgra, rosenbrock, solvsys, nlsys
    coor: np.ndarray
    dat: np.ndarray
    std2r: np.ndarray
    icoor: np.ndarray
    idat: np.ndarray
    pdescr: np.ndarray
    pmint: np.ndarray
    pmaxt: np.ndarray
    ptotal: np.ndarray
    imodel: int = 1
    npass: int = 1
    nseq: int = 16
    nbeta: int = 32
    nburn: int = 1000
    niter: int = 5000
    betan: float = 1e-4
    pstp0: np.ndarray = None   # initial step per mutable parameter (None: range/50)
    truth: np.ndarray = None
    extra: dict = field(default_factory=dict)

    @property
    def ndat(self) -> int:
        return int(self.dat.size)

    @property
    def nptot(self) -> int:
        return int(self.pdescr.size)

    @property
    def nprm(self) -> int:
        return int(np.count_nonzero(self.pdescr))

    @property
    def nvis(self) -> int:
        return int(self.idat[0]) if self.model == "sgra" else 0

    def beta(self) -> np.ndarray:
        return geometric_betas(self.nbeta, 1.0, self.betan)

    def with_sizes(self, **kw) -> "Workload":
        d = dict(self.__dict__)
        d.update(kw)
        return Workload(**d)


def rosenbrock(n: int = 4, nseq: int = 16, nbeta: int = 32, nburn: int = 1000,
               niter: int = 5000) -> Workload:
    """Config 1: f(x) = sum_{i<N-1} 100 (x_{i+1}-x_i^2)^2 + (1-x_i)^2 on [-5,5]^N."""
    return Workload(
        name="rosenbrock%d" % n, model="rosenbrock",
        coor=np.zeros(1, np.float32), dat=np.zeros(1, np.float32),
        std2r=np.ones(1, np.float32), icoor=np.zeros(1, np.int32),
        idat=np.zeros(1, np.int32), pdescr=np.ones(n, np.int32),
        pmint=np.full(n, -5.0, np.float32), pmaxt=np.full(n, 5.0, np.float32),
        ptotal=np.zeros(n, np.float32), imodel=0, npass=1, nseq=nseq, nbeta=nbeta,
        nburn=nburn, niter=niter, betan=1e-3, pstp0=np.full(n, 0.5, np.float32),
        truth=np.ones(n, np.float32))


def solvsys(nseq: int = 14, nbeta: int = 32, nburn: int = 400, niter: int = 5000) -> Workload:
    """The reference's two-equation example: x^2 + y^2 = 1, -0.25 x + y = 0.5
    (examples/solvsys/solvsys.py:22-28)."""
    return Workload(
        name="solvsys", model="solvsys",
        coor=np.array([2, 2, 0.25, 0.5], np.float32), dat=np.array([1, 0.5], np.float32),
        std2r=np.ones(2, np.float32), icoor=np.zeros(1, np.int32),
        idat=np.zeros(1, np.int32), pdescr=np.array([1, 1], np.int32),
        pmint=np.array([-5.0, -5.0], np.float32), pmaxt=np.array([5.0, 5.0], np.float32),
        ptotal=np.zeros(2, np.float32), imodel=0, npass=1, nseq=nseq, nbeta=nbeta,
        nburn=nburn, niter=niter)


def nlsys(n: int = 8, seed: int = 2, nseq: int = 64, nbeta: int = 32, nburn: int = 2000,
          niter: int = 10000) -> Workload:
    """Config 2: r_k = sum_j A_kj sin x_j + B_kj x_j^2 - b_k, A, B ~ N(0,1),
    b from a hidden x* ~ U(-1,1)^n; coor = [A | B] row-major, dat = b."""
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, n)).astype(np.float32)
    B = rng.standard_normal((n, n)).astype(np.float32)
    xs = rng.uniform(-1, 1, n).astype(np.float32)
    b = (A.astype(np.float64) @ np.sin(xs.astype(np.float64))
         + B.astype(np.float64) @ (xs.astype(np.float64) ** 2)).astype(np.float32)
    return Workload(
        name="nlsys%d" % n, model="nlsys",
        coor=np.concatenate([A.ravel(), B.ravel()]).astype(np.float32), dat=b,
        std2r=np.ones(n, np.float32), icoor=np.zeros(1, np.int32), idat=np.zeros(1, np.int32),
        pdescr=np.ones(n, np.int32), pmint=np.full(n, -3.0, np.float32),
        pmaxt=np.full(n, 3.0, np.float32), ptotal=np.zeros(n, np.float32), imodel=0,
        npass=1, nseq=nseq, nbeta=nbeta, nburn=nburn, niter=niter, truth=xs)


def sgra_truth(rng) -> np.ndarray:
    return rng.uniform(SGRA9_TRUTH_LO, SGRA9_TRUTH_HI).astype(np.float32)


def _sgra9_vis_np(prm, u, v):
    """FP64 NumPy visibility of sgra_model9 (the data generator only)."""
    from scipy.special import j0, j1
    Zsp, Re, rq, ecc, fade, gax, aq, gq, th = [float(x) for x in prm]
    Re = np.radians(Re / 3600.0) * 1e3
    Ri = rq * Re
    d = ecc * (Re - Ri)
    gsy = gax * Re
    gsx = aq * gsy
    U = u * np.cos(th) + v * np.sin(th)
    V = -u * np.sin(th) + v * np.cos(th)
    h = (2.0 / np.pi) / ((Re ** 2 - Ri ** 2 * (1.0 + d / Re)) * fade
                         + (Re ** 2 - Ri ** 2 * (1.0 - d / Re)))
    h0 = fade * h
    rho = np.maximum(np.sqrt(U ** 2 + V ** 2), 1e-9)
    xe = 2 * np.pi * rho * Re
    xi = 2 * np.pi * rho * Ri
    ree = 0.5 * (h + h0) * Re * j1(xe) / rho
    # pi*R*(J0 - J2)/rho^2 - J1/rho^3 == -x J2(x) / rho^3,  J2 = 2 J1/x - J0
    j2e = np.where(xe > 1e-6, 2 * j1(xe) / np.maximum(xe, 1e-30) - j0(xe), xe ** 2 / 8)
    j2i = np.where(xi > 1e-6, 2 * j1(xi) / np.maximum(xi, 1e-30) - j0(xi), xi ** 2 / 8)
    ime = (h - h0) / (4 * np.pi) * (-xe * j2e / rho ** 3) * U
    rei = 0.5 * (h + h0 - d * (h - h0) / Re) * Ri * j1(xi) / rho
    imi = (h - h0) / (4 * np.pi) * rq * (-xi * j2i / rho ** 3) * U
    Fr = (ree + 1j * ime) - np.exp(1j * 2 * np.pi * d * U) * (rei + 1j * imi)
    gcoef = 2 * (np.pi / (2 * np.sqrt(2 * np.log(2)))) ** 2
    Fg = np.exp(-gcoef * ((U * gsx) ** 2 + (V * gsy) ** 2)) * np.exp(-1j * 2 * np.pi * (Ri - d) * U)
    F = Zsp * ((1 - gq) * Fr + gq * Fg)
    return np.abs(F), np.angle(F)


def sgra(nvis: int = 2000, ncph: int = 600, seed: int = 3, nseq: int = 64, nbeta: int = 32,
         nburn: int = 5000, niter: int = 20000, truth=None, amp_rel: float = 0.03,
         amp_floor: float = 0.002, cph_deg: float = 5.0, imodel: int = 1) -> Workload:
    """Configs 3 and 4: sgra_model9 on seeded synthetic EHT-like data.

    coor = [u0, v0, u1, v1, ...] (Glambda), dat = [amp..., cph...],
    icoor = closure triplets (i, j, k): cph = phi_i + phi_j - phi_k,
    idat = [nvis, nbeta*nseq*ndat, cpExt=0] (src/imgpu.py:818-831).
    """
    rng = np.random.default_rng(seed)
    if truth is None:
        truth = sgra_truth(rng)
    truth = np.asarray(truth, np.float32)
    r = rng.uniform(0.5, 8.0, nvis)
    pa = rng.uniform(0.0, 2 * np.pi, nvis)
    u = (r * np.cos(pa)).astype(np.float32)
    v = (r * np.sin(pa)).astype(np.float32)
    amp, pha = _sgra9_vis_np(truth, u.astype(np.float64), v.astype(np.float64))
    sig = amp_rel * amp + amp_floor
    amp_obs = amp * (1.0 + amp_rel * rng.standard_normal(nvis))
    tri = rng.integers(0, nvis, (ncph, 3)).astype(np.int32)
    bad = (tri[:, 0] == tri[:, 1]) | (tri[:, 0] == tri[:, 2]) | (tri[:, 1] == tri[:, 2])
    while bad.any():
        tri[bad] = rng.integers(0, nvis, (int(bad.sum()), 3))
        bad = (tri[:, 0] == tri[:, 1]) | (tri[:, 0] == tri[:, 2]) | (tri[:, 1] == tri[:, 2])
    cph = pha[tri[:, 0]] + pha[tri[:, 1]] - pha[tri[:, 2]]
    sig_c = np.radians(cph_deg)
    cph_obs = cph + sig_c * rng.standard_normal(ncph)
    cph_obs = np.arctan2(np.sin(cph_obs), np.cos(cph_obs))
    ndat = nvis + ncph
    coor = np.empty(2 * nvis, np.float32)
    coor[0::2] = u
    coor[1::2] = v
    dat = np.concatenate([amp_obs, cph_obs]).astype(np.float32)
    std2r = np.concatenate([1.0 / sig ** 2, np.full(ncph, 1.0 / sig_c ** 2)]).astype(np.float32)
    idat = np.array([nvis, nbeta * nseq * ndat, 0], np.int32)
    return Workload(
        name="sgra9_%dvis_%dcph" % (nvis, ncph), model="sgra", coor=coor, dat=dat,
        std2r=std2r, icoor=tri.ravel().astype(np.int32) if ncph else np.zeros(1, np.int32),
        idat=idat, pdescr=SGRA9_PDESCR.copy(), pmint=SGRA9_PMIN.copy(),
        pmaxt=SGRA9_PMAX.copy(), ptotal=np.zeros(9, np.float32), imodel=imodel,
        npass=2 if ncph else 1, nseq=nseq, nbeta=nbeta, nburn=nburn, niter=niter,
        betan=1e-4, truth=truth)


def sgra_batch(nfits: int = 1024, seed: int = 5, nseq: int = 16, nbeta: int = 16,
               nburn: int = 5000, niter: int = 20000, nvis_min: int = 500,
               nvis_max: int = 50000, cph_frac: float = 0.3) -> list:
    """Config 5: independent crescent fits with nvis ~ logU(nvis_min, nvis_max)."""
    rng = np.random.default_rng(seed)
    out = []
    for f in range(nfits):
        nvis = int(np.exp(rng.uniform(np.log(nvis_min), np.log(nvis_max))))
        ncph = int(cph_frac * nvis)
        out.append(sgra(nvis=nvis, ncph=ncph, seed=int(rng.integers(1 << 31)), nseq=nseq,
                        nbeta=nbeta, nburn=nburn, niter=niter))
    return out


def config(i: int) -> Workload:
    """The single-fit benchmark workloads by number (1-4)."""
    if i == 1:
        return rosenbrock()
    if i == 2:
        return nlsys()
    if i == 3:
        return sgra()
    if i == 4:
        return sgra(nvis=20000, ncph=6000, seed=4)
    raise ValueError("config must be 1-4 (5 is sgra_batch())")


def write_uvdata(path, nant=5, ntimes=40, t0="2009:095:02:20:00", dt_s=1200, seed=9,
                 truth=None, snr_amp=0.03, imodel=1):
    """Write a synthetic observation in the uv text format read by
    imgpu.read_uvdata (one row per baseline and time: time, u v w in
    kilolambda, baseline aa-bb, channel, (amplitude, phase in degrees),
    weight, sigma).  All baselines of nant stations are present at every time,
    so every antenna triangle gives a closure phase.  Returns the true
    parameters and the (u, v) points in gigalambda."""
    import calendar
    import time as _time
    rng = np.random.default_rng(seed)
    if truth is None:
        truth = sgra_truth(rng)
    truth = np.asarray(truth, np.float32)
    # station positions on a ~8 Glambda disk; baselines rotate with time
    pos = rng.uniform(-4.0, 4.0, (nant, 2))
    base = calendar.timegm(_time.strptime(t0, "%Y:%j:%H:%M:%S"))
    rows, uvs = [], []
    for it in range(ntimes):
        ang = 2 * np.pi * it / (4 * ntimes)
        rot = np.array([[np.cos(ang), -np.sin(ang)], [np.sin(ang), np.cos(ang)]])
        p = pos @ rot.T
        ts = _time.strftime("%Y:%j:%H:%M:%S", _time.gmtime(base + it * dt_s))
        for a in range(nant):
            for b in range(a + 1, nant):
                u, v = p[a] - p[b]
                uvs.append((u, v))
                rows.append((ts, u, v, a + 1, b + 1))
    uv = np.array(uvs)
    amp, pha = _sgra9_vis_np(truth, uv[:, 0], uv[:, 1])
    sig = snr_amp * amp + 0.002
    amp_obs = amp * (1 + snr_amp * rng.standard_normal(amp.size))
    with open(path, "w") as f:
        f.write("Scan Start (UT)  U(klam)  V(klam)  W(klam)  Baseline  Channel  "
                "Visibility (amp, phase)  Weight  Sigma\n")
        for (ts, u, v, a, b), am, ph, sg in zip(rows, amp_obs, pha, sig):
            f.write("%s.00 %13.2f %13.2f %13.2f %02d-%02d    00    ( %12.6f, %15.6f) %9.2f %.5f\n"
                    % (ts, u * 1e6, v * 1e6, 0.0, a, b, am, np.degrees(ph), 1000.0, sg))
    return truth, uv
