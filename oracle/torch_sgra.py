"""PyTorch (float64) re-expression of the Sgr A* model and its chi^2.

TEST INFRASTRUCTURE ONLY: the gradient tests differentiate this function with
torch.autograd and compare the result with the CUDA adjoint; the
``cuda_mcmc_gb300`` product never imports it.

The formulas restate examples/sgra_model_fit/model.cuh (sgra_model9:
lines 322-462, sgra_model13: lines 120-315) in the form of ``oracle.c``
(or_sgra_model9 / or_sgra_model13), with J2 = 2 J1(x)/x - J0(x) in place of
jn(2, x), and the chi^2 terms of src/gpu_mcmc.cu:305-323 (closure residuals
wrapped by atan2(sin, cos)).  J0 and J1 come from scipy.special (FP64
Cephes; torch.special's versions are only good to about 4e-7 and have no
derivative) and carry their own derivatives: J0' = -J1, J1' = J0 - J1/x.
CPU tensors only.
"""
from __future__ import annotations

import math

import numpy as np
import torch


def _sp(fn, x):
    from scipy import special
    return torch.from_numpy(getattr(special, fn)(x.detach().numpy()))


class _J0(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x):
        ctx.save_for_backward(x)
        return _sp("j0", x)

    @staticmethod
    def backward(ctx, g):
        (x,) = ctx.saved_tensors
        return -g * j1(x)


class _J1(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x):
        ctx.save_for_backward(x)
        return _sp("j1", x)

    @staticmethod
    def backward(ctx, g):
        (x,) = ctx.saved_tensors
        small = x.abs() <= 1e-8
        safe = torch.where(small, torch.ones_like(x), x)
        d = j0(x) - j1(x) / safe
        return g * torch.where(small, torch.full_like(x, 0.5), d)


def j0(x):
    return _J0.apply(x)


def j1(x):
    return _J1.apply(x)


def _j2(x):
    """J2(x) = 2 J1(x)/x - J0(x), with its series x^2/8 near 0 (no 0/0, so
    that autograd stays finite at x = 0, e.g. Rin = 0)."""
    small = x.abs() < 1e-4
    xs = torch.where(small, torch.ones_like(x), x)
    return torch.where(small, x * x / 8.0, 2.0 * j1(xs) / xs - j0(xs))


def _ring(prm, U, rho, Rex, Rin, rq, d, h, h0):
    """Crescent (outer disk minus shifted inner disk), rho > 1e-7."""
    pi = math.pi
    aRex = 2.0 * pi * rho * Rex
    ree = 0.5 * (h + h0) * Rex * j1(aRex) / rho
    j2e = _j2(aRex)
    ime = (h - h0) / (4 * pi) * (pi * Rex * (j0(aRex) - j2e) / rho ** 2 - j1(aRex) / rho ** 3) * U
    aRin = 2.0 * pi * rho * Rin
    j2i = _j2(aRin)
    rei = 0.5 * (h + h0 - d * (h - h0) / Rex) * Rin * j1(aRin) / rho
    imi = (h - h0) / (4 * pi) * rq * (pi * Rin * (j0(aRin) - j2i) / rho ** 2
                                      - j1(aRin) / rho ** 3) * U
    dre, dim = torch.cos(2.0 * pi * d * U), torch.sin(2.0 * pi * d * U)
    return ree - (rei * dre - imi * dim), ime - (rei * dim + imi * dre)


def vis(prm, u, v, imodel=1):
    """Complex visibility (re, im) of parameter rows prm[n, nptot] at the uv
    points u[m], v[m] -> two [n, m] tensors.  Needs the Gaussian switched on
    (gax, aq, gq != 0, gq != 1 for sgra_model13), the region the gradient
    tests sample."""
    pi = math.pi
    P = [prm[:, k:k + 1] for k in range(prm.shape[1])]
    u, v = u[None, :], v[None, :]
    gcoef = 2.0 * (pi / (2.0 * math.sqrt(2.0 * math.log(2.0)))) ** 2
    if imodel == 1:
        Zsp, Re, rq, ecc, fade, gax, aq, gq, th = P[:9]
    else:
        Zsp, Re, rq, ecc, fade, gr, gax, aq, gq, alpha, beta, eta, th = P[:13]
    Rex = (pi / 180.0) * (Re / 3600.0) * 1e3
    Rin = rq * Rex
    d = ecc * (Rex - Rin)
    if imodel != 1:
        d = d * torch.cos(eta - th)
    h = (2.0 / pi) / ((Rex * Rex - Rin * Rin * (1.0 + d / Rex)) * fade
                      + (Rex * Rex - Rin * Rin * (1.0 - d / Rex)))
    h0 = fade * h
    U = u * torch.cos(th) + v * torch.sin(th)
    V = -u * torch.sin(th) + v * torch.cos(th)
    rho = torch.sqrt(U * U + V * V)
    fr_re, fr_im = _ring(prm, U, rho, Rex, Rin, rq, d, h, h0)
    gsy = gax * Rex
    gsx = aq * gsy
    if imodel == 1:
        gamp = torch.exp(-gcoef * ((U * gsx) ** 2 + (V * gsy) ** 2))
        gph = -2.0 * pi * (Rin - d) * U
    else:
        Ub = u * torch.cos(beta) + v * torch.sin(beta)
        Vb = -u * torch.sin(beta) + v * torch.cos(beta)
        gamp = torch.exp(-gcoef * ((Ub * gsx) ** 2 + (Vb * gsy) ** 2))
        gph = -2.0 * pi * gr * Rex * (torch.cos(alpha) * u + torch.sin(alpha) * v)
    fg_re, fg_im = gamp * torch.cos(gph), gamp * torch.sin(gph)
    return Zsp * ((1.0 - gq) * fr_re + gq * fg_re), Zsp * ((1.0 - gq) * fr_im + gq * fg_im)


def chi2(prm, coor, dat, std2r, icoor, nvis, npass=2, imodel=1):
    """chi^2 of parameter rows prm[n, nptot] (float64 tensor) for data in the
    reference's layout (cpExt = 0): amplitude terms plus, for npass >= 2,
    closure-phase terms cph = phi_i + phi_j - phi_k."""
    t = lambda a, dt=torch.float64: torch.as_tensor(np.asarray(a), dtype=dt)
    coor = t(coor)
    u, v = coor[0:2 * nvis:2], coor[1:2 * nvis:2]
    dat, std2r = t(dat), t(std2r)
    re, im = vis(prm, u, v, imodel)
    amp = torch.sqrt(re * re + im * im)
    c2 = ((dat[None, :nvis] - amp) ** 2 * std2r[None, :nvis]).sum(1)
    ncph = dat.numel() - nvis
    if npass >= 2 and ncph > 0:
        ph = torch.atan2(im, re)
        tri = t(icoor, torch.int64)[:3 * ncph].reshape(ncph, 3)
        cph = ph[:, tri[:, 0]] + ph[:, tri[:, 1]] - ph[:, tri[:, 2]]
        x = dat[None, nvis:] - cph
        dif = torch.atan2(torch.sin(x), torch.cos(x))
        c2 = c2 + (dif * dif * std2r[None, nvis:]).sum(1)
    return c2


def chi2_and_grad(prm, coor, dat, std2r, icoor, nvis, npass=2, imodel=1):
    """(chi2 [n], dchi2/dprm [n, nptot]) by autograd, in float64."""
    p = torch.as_tensor(np.asarray(prm, np.float64)).clone().requires_grad_(True)
    c = chi2(p, coor, dat, std2r, icoor, nvis, npass, imodel)
    (g,) = torch.autograd.grad(c.sum(), p)
    return c.detach().numpy(), g.numpy()


def residuals(prm, coor, dat, std2r, icoor, nvis, npass=2, imodel=1):
    """Weighted residuals r with chi^2 = sum r^2 for one parameter row prm
    [nptot]: sqrt(w) (amp_obs - |V|) for the amplitudes, then
    sqrt(w) wrap(cph_obs - cph) for the closure phases (npass >= 2)."""
    t = lambda a, dt=torch.float64: torch.as_tensor(np.asarray(a), dtype=dt)
    coor = t(coor)
    u, v = coor[0:2 * nvis:2], coor[1:2 * nvis:2]
    dat, std2r = t(dat), t(std2r)
    re, im = vis(prm[None, :], u, v, imodel)
    amp = torch.sqrt(re * re + im * im)[0]
    r = torch.sqrt(std2r[:nvis]) * (dat[:nvis] - amp)
    ncph = dat.numel() - nvis
    if npass >= 2 and ncph > 0:
        ph = torch.atan2(im, re)[0]
        tri = t(icoor, torch.int64)[:3 * ncph].reshape(ncph, 3)
        x = dat[nvis:] - (ph[tri[:, 0]] + ph[tri[:, 1]] - ph[tri[:, 2]])
        r = torch.cat([r, torch.sqrt(std2r[nvis:]) * torch.atan2(torch.sin(x), torch.cos(x))])
    return r


def fisher_gn(prm, coor, dat, std2r, icoor, nvis, npass=2, imodel=1):
    """Gauss-Newton Fisher information J^T J of chi^2/2 (J = d residuals / d prm)
    at one parameter row, float64 [nptot, nptot]."""
    p = torch.as_tensor(np.asarray(prm, np.float64))
    J = torch.autograd.functional.jacobian(
        lambda x: residuals(x, coor, dat, std2r, icoor, nvis, npass, imodel), p)
    return (J.T @ J).numpy()
