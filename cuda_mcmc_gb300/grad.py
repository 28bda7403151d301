"""chi^2 gradients of the Sgr A* model on the GPU, and what they drive.

* :class:`SgraChi2` -- chi^2 and d chi^2 / d p for many parameter rows at once
  through the hand-written CUDA adjoint (``cmc_grad`` in libcmc_sgra.so);
  :meth:`SgraChi2.chi2` is differentiable (a ``torch.autograd.Function`` whose
  backward is that adjoint).
* :meth:`SgraChi2.fisher_gn` -- the Gauss-Newton Fisher information of
  chi^2/2 (``cmc_fisher``: per-datum model gradients from the adjoint,
  accumulated on the GPU); always positive semi-definite;
* :func:`fisher` -- the observed Fisher information of the tempered posterior
  exp(-beta chi^2 / 2): beta/2 times the Hessian of chi^2, from central
  differences of the adjoint gradient (one batched call for all 2 k
  displacements), projected onto the positive-definite cone.
* :func:`polish` -- bounded L-BFGS descent of chi^2 from a starting point
  (e.g. the best replica at beta = 1), every step one adjoint call.

The chi^2 is the sum the sweep minimises (src/gpu_mcmc.cu:305-323 over
examples/sgra_model_fit/model.cuh): amplitude terms, plus closure-phase terms
when npass >= 2.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib

_F32, _I32 = torch.float32, torch.int32


def _dev(a, dtype, device):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype).to(device).contiguous()


class SgraChi2:
    """chi^2(p) of one Sgr A* data set for parameter rows p[n, nptot]."""

    def __init__(self, coor, dat, std2r, icoor, idat, nptot, imodel=1, npass=2,
                 device="cuda"):
        self.L = _lib.load("sgra")
        if not hasattr(self.L, "cmc_grad"):
            raise RuntimeError("libcmc_sgra.so has no cmc_grad")
        self.device = torch.device(device)
        d = self.device
        idat = np.ascontiguousarray(idat, np.int32)
        icoor = np.ascontiguousarray(icoor, np.int32)
        if icoor.size == 0:
            icoor = np.zeros(1, np.int32)
        self.nptot, self.imodel, self.npass = int(nptot), int(imodel), int(npass)
        self.t = {"coor": _dev(coor, _F32, d), "dat": _dev(dat, _F32, d),
                  "std2r": _dev(std2r, _F32, d), "icoor": _dev(icoor, _I32, d),
                  "idat": _dev(idat, _I32, d),
                  "status": torch.zeros(4, dtype=_I32, device=d)}
        j = _lib.CmcJob()
        j.ncoor, j.ndat = int(self.t["coor"].numel()), int(self.t["dat"].numel())
        j.nicoor, j.nidat = int(icoor.size), int(idat.size)
        j.nptot = j.nprm = self.nptot
        j.npass, j.imodel, j.nseq = self.npass, self.imodel, 1
        for i in range(4):
            j.hidat[i] = int(idat[i]) if i < idat.size else 0
        for k in ("coor", "dat", "std2r", "icoor", "idat", "status"):
            setattr(j, k, self.t[k].data_ptr())
        self.job = j
        self._work = None

    @classmethod
    def from_workload(cls, w, device="cuda"):
        return cls(w.coor, w.dat, w.std2r, w.icoor, w.idat, w.nptot, w.imodel, w.npass, device)

    def __call__(self, p, stream=None):
        """(chi2 [n], grad [n, nptot]) at p[n, nptot] (float32, any device)."""
        p = torch.as_tensor(p, dtype=_F32).to(self.device).contiguous()
        if p.dim() != 2 or p.shape[1] != self.nptot:
            raise ValueError("p must be [n, %d]" % self.nptot)
        n = int(p.shape[0])
        chi2 = torch.empty(n, dtype=_F32, device=self.device)
        grad = torch.empty((n, self.nptot), dtype=_F32, device=self.device)
        if n == 0:
            return chi2, grad
        j = self.job
        j.nbeta = n
        j.ndatm = 0
        j.pcur, j.chi2c, j.flag = p.data_ptr(), chi2.data_ptr(), None
        need = int(self.L.cmc_grad_work_bytes(C.byref(j)))
        if need == 0:
            raise _lib.McmcError(_lib.CMC_ERR_ARG, "cmc_grad_work_bytes: invalid job")
        if self._work is None or self._work.numel() < need:
            self._work = torch.empty(need, dtype=torch.uint8, device=self.device)
        j.work, j.work_bytes = self._work.data_ptr(), int(self._work.numel())
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        _lib.check(self.L, self.L.cmc_grad(C.byref(j), C.c_void_p(grad.data_ptr()),
                                           C.c_void_p(s.cuda_stream)))
        return chi2, grad

    def chi2(self, p):
        """Differentiable chi^2 [n] of p[n, nptot]: backward is the CUDA adjoint."""
        return _Chi2Fn.apply(p, self)

    def fisher_gn(self, p, stream=None):
        """Gauss-Newton Fisher information of chi^2/2, [n, nptot, nptot], at
        p[n, nptot] (cmc_fisher): sum over data of w * grad(model) grad(model)^T
        for the amplitudes and the closure phases."""
        p = torch.as_tensor(p, dtype=_F32).to(self.device).contiguous()
        if p.dim() != 2 or p.shape[1] != self.nptot:
            raise ValueError("p must be [n, %d]" % self.nptot)
        n = int(p.shape[0])
        out = torch.empty((n, self.nptot, self.nptot), dtype=_F32, device=self.device)
        chi2 = torch.empty(max(n, 1), dtype=_F32, device=self.device)
        if n == 0:
            return out
        j = self.job
        j.nbeta = n
        j.ndatm = 0
        j.pcur, j.chi2c, j.flag = p.data_ptr(), chi2.data_ptr(), None
        need = int(self.L.cmc_fisher_work_bytes(C.byref(j)))
        if need == 0:
            raise _lib.McmcError(_lib.CMC_ERR_ARG, "cmc_fisher_work_bytes: invalid job")
        if self._work is None or self._work.numel() < need:
            self._work = torch.empty(need, dtype=torch.uint8, device=self.device)
        j.work, j.work_bytes = self._work.data_ptr(), int(self._work.numel())
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        _lib.check(self.L, self.L.cmc_fisher(C.byref(j), C.c_void_p(out.data_ptr()),
                                             C.c_void_p(s.cuda_stream)))
        return out


class _Chi2Fn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, p, obj):
        chi2, grad = obj(p.detach())
        ctx.save_for_backward(grad)
        ctx.in_dtype, ctx.in_device = p.dtype, p.device
        return chi2.to(device=p.device, dtype=p.dtype)

    @staticmethod
    def backward(ctx, g):
        (grad,) = ctx.saved_tensors
        out = g.to(grad.device, grad.dtype)[:, None] * grad
        return out.to(device=ctx.in_device, dtype=ctx.in_dtype), None


def fisher(obj: SgraChi2, p, ivar=None, beta=1.0, rel_step=1e-3, scale=None, floor=None):
    """Observed Fisher information beta/2 * Hessian(chi^2) at p [nptot] over the
    parameters ``ivar`` (default: all), for the tempered target
    exp(-beta chi^2 / 2).  Row k is the central difference of the adjoint
    gradient along parameter ivar[k] with step rel_step * scale[k]
    (scale: e.g. the prior widths, default max(|p_k|, 1)); the result is
    symmetrised and its eigenvalues raised to ``floor`` (default 1e-9 of the
    largest), so that it inverts to a covariance.  Returns float64 [k, k]."""
    return fisher_many(obj, np.asarray(p, np.float64).reshape(1, -1), ivar, beta, rel_step,
                       scale, floor)[0]


def fisher_many(obj: SgraChi2, P, ivar=None, beta=1.0, rel_step=1e-3, scale=None, floor=None):
    """:func:`fisher` at every row of P [m, nptot] with one adjoint call
    (2 k m displaced parameter rows).  Returns float64 [m, k, k]."""
    P = np.asarray(P, np.float64)
    m, nptot = P.shape
    ivar = np.arange(nptot) if ivar is None else np.asarray(ivar, np.int64)
    k = ivar.size
    if scale is None:
        sc = np.maximum(np.abs(P[:, ivar]), 1.0)
    else:   # per parameter: [nptot] (read at ivar) or [k]
        sc = np.asarray(scale, np.float64).ravel()
        sc = np.broadcast_to(sc[ivar] if sc.size == nptot else sc, (m, k))
    h = rel_step * sc                                           # [m, k]
    Q = np.repeat(P[:, None, :], 2 * k, axis=1)                 # [m, 2k, nptot]
    a = np.arange(k)
    Q[:, 2 * a, ivar] += h
    Q[:, 2 * a + 1, ivar] -= h
    Q32 = Q.astype(np.float32)
    taken = Q32[:, 2 * a, ivar].astype(np.float64) - Q32[:, 2 * a + 1, ivar].astype(np.float64)
    _, g = obj(Q32.reshape(m * 2 * k, nptot))
    g = g.double().cpu().numpy().reshape(m, 2 * k, nptot)[:, :, ivar]
    H = (g[:, 0::2] - g[:, 1::2]) / taken[:, :, None]          # [m, k, k]
    H = 0.5 * (H + np.swapaxes(H, 1, 2)) * (0.5 * beta)
    out = np.empty_like(H)
    for i in range(m):
        w, V = np.linalg.eigh(H[i])
        fl = (1e-9 * max(float(w.max()), 0.0) if floor is None else float(floor))
        w = np.maximum(w, max(fl, np.finfo(np.float64).tiny))
        out[i] = (V * w) @ V.T
    return out


def proposal_cholesky(F, d=None):
    """Lower Cholesky factor of the Metropolis proposal covariance
    (2.38^2 / d) F^-1 for a Fisher information F [d, d] (Gelman, Roberts and
    Gilks 1996 scale for a Gaussian target)."""
    F = np.asarray(F, np.float64)
    d = F.shape[0] if d is None else d
    cov = np.linalg.inv(F) * (2.38 ** 2 / d)
    cov = 0.5 * (cov + cov.T)
    return np.linalg.cholesky(cov)


def polish(obj: SgraChi2, p0, pmin, pmax, ivar=None, maxiter=200, tol=1e-9):
    """Bounded L-BFGS (scipy's L-BFGS-B) descent of chi^2 from p0 over the
    parameters ivar (the rest fixed), within [pmin, pmax]; chi^2 and its
    gradient come from the CUDA adjoint.  Returns (p, chi2, result)."""
    from scipy.optimize import minimize
    p0 = np.asarray(p0, np.float64).ravel()
    ivar = np.arange(p0.size) if ivar is None else np.asarray(ivar, np.int64)
    lo = np.asarray(pmin, np.float64).ravel()[ivar]
    hi = np.asarray(pmax, np.float64).ravel()[ivar]
    # work in units of the prior width so that L-BFGS sees a balanced problem
    width = np.where(hi > lo, hi - lo, 1.0)

    def f(x):
        p = p0.copy()
        p[ivar] = lo + x * width
        c, g = obj(p[None, :].astype(np.float32))
        return float(c[0]), g[0].double().cpu().numpy()[ivar] * width

    x0 = np.clip((p0[ivar] - lo) / width, 0.0, 1.0)
    res = minimize(f, x0, jac=True, method="L-BFGS-B", bounds=[(0.0, 1.0)] * ivar.size,
                   options={"maxiter": maxiter, "ftol": tol, "gtol": 1e-12})
    p = p0.copy()
    p[ivar] = lo + res.x * width
    return p, float(res.fun), res
