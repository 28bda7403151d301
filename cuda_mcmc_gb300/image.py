"""Model brightness images of the Sgr A* model.

:func:`vis2bri` is the reference's ``model_vis2bri_simple``
(src/obsdatafit.py:2683-2805): the model visibility on an ngrid x ngrid uv
grid spanning UVspan Gigalambda (U axis running right to left, the
astronomical convention), a cosine taper 0.5 (1 + cos(pi rho / (UVspan/2)))
cut at rho = UVspan/2, and the brightness image
ifftshift(ifft2(fftshift(V * taper))).  Here the grid visibilities come from
the library's calc_model path on the GPU (the same model kernels as the
sweep) and the FFT runs on the device (torch.fft).  The reference's
odd-ngrid branch leaves its V range undefined; here an odd grid is
symmetric about 0 in both axes.
"""
from __future__ import annotations

import numpy as np
import torch

from . import mcmc_interf as mi


def uv_grid(UVspan, ngrid):
    """(Ugrid, Vgrid) as the reference builds them (meshgrid of the U range,
    right to left, and the V range)."""
    uvext = UVspan / 2.0
    if ngrid % 2 == 0:
        urng = np.linspace(uvext - UVspan / ngrid, -uvext, ngrid)
        vrng = np.linspace(-uvext, uvext - UVspan / ngrid, ngrid)
    else:
        urng = np.linspace(uvext, -uvext, ngrid)
        vrng = np.linspace(-uvext, uvext, ngrid)
    return np.meshgrid(urng, vrng)


def grid_vis(prm, Ugrid, Vgrid, imodel=1):
    """Complex model visibility on a uv grid (float32 model on the GPU,
    returned as complex128 numpy)."""
    prm = np.ascontiguousarray(prm, np.float32).ravel()
    ul = np.asarray(Ugrid, np.float32).ravel()
    vl = np.asarray(Vgrid, np.float32).ravel()
    nvis = ul.size
    coor = np.empty(2 * nvis, np.float32)
    coor[0::2], coor[1::2] = ul, vl
    idat = np.array((nvis, 0, 0), np.int32)
    datm = np.zeros(2 * nvis, np.float32)
    mi.use_model("sgra")
    mi.calcmodel(coor, idat, datm, prm.reshape(1, 1, -1), int(imodel), coor.size, nvis,
                 idat.size, datm.size, prm.size, 1, 1)
    amp = datm[:nvis].astype(np.float64)
    pha = datm[nvis:].astype(np.float64)
    return (amp * np.exp(1j * pha)).reshape(np.shape(Ugrid))


def vis2bri(prm, UVspan, ngrid, imodel=1, device="cuda"):
    """The reference's model_vis2bri_simple for the Sgr A* model with
    parameters ``prm``.  Returns (Vi, Br, Ugrid, Vgrid, Xgrid, Ygrid, UVext,
    XYext): Vi the grid visibility, Br the complex brightness image, the X / Y
    grids in microarcseconds and the extents of both images."""
    Ugrid, Vgrid = uv_grid(UVspan, ngrid)
    uvext = UVspan / 2.0
    Vi = grid_vis(prm, Ugrid, Vgrid, imodel)
    rho = np.sqrt(Ugrid ** 2 + Vgrid ** 2)
    cwin = 0.5 * (1.0 + np.cos(np.pi * rho / uvext))
    cwin[rho > uvext] = 0.0
    t = torch.as_tensor(Vi * cwin, dtype=torch.complex128, device=device)
    Br = torch.fft.ifftshift(torch.fft.ifft2(torch.fft.fftshift(t))).cpu().numpy()
    XYspan = ngrid / UVspan                         # nanoradians
    XYspan = 3600.0 * np.degrees(XYspan) * 1e-3     # microarcseconds
    xyext = XYspan / 2.0
    if ngrid % 2 == 0:
        xrng = np.linspace(xyext - XYspan / ngrid, -xyext, ngrid)
        yrng = np.linspace(-xyext, xyext - XYspan / ngrid, ngrid)
    else:
        xrng = np.linspace(xyext, -xyext, ngrid)
        yrng = np.linspace(-xyext, xyext, ngrid)
    Xgrid, Ygrid = np.meshgrid(xrng, yrng)
    UVext = (Ugrid[0, 0], Ugrid[0, -1], Vgrid[0, 0], Vgrid[-1, 0])
    XYext = (Xgrid[0, 0], Xgrid[0, -1], Ygrid[0, 0], Ygrid[-1, 0])
    return Vi, Br, Ugrid, Vgrid, Xgrid, Ygrid, UVext, XYext
