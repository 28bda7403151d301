"""Model brightness images (cuda_mcmc_gb300.image.vis2bri, the reference's
model_vis2bri_simple): grids and extents (CPU), and on the GPU the image from
the library's calc_model against the same construction from the FP64 oracle
model with numpy's FFT."""
import numpy as np
import pytest

import oracle
from cuda_mcmc_gb300 import image, synth


def test_uv_grid_matches_the_reference_layout():
    U, V = image.uv_grid(8.0, 4)
    assert np.allclose(U[0], [2.0, 0.0, -2.0, -4.0])      # right to left
    assert np.allclose(V[:, 0], [-4.0, -2.0, 0.0, 2.0])
    U, V = image.uv_grid(8.0, 5)
    assert np.allclose(U[0], [4, 2, 0, -2, -4]) and np.allclose(V[:, 0], [-4, -2, 0, 2, 4])


@pytest.mark.gpu
@pytest.mark.parametrize("ngrid", [64, 65])
def test_image_matches_fp64_construction(ngrid):
    prm = synth.sgra(nvis=10, ncph=0, nseq=2, nbeta=4).truth
    UVspan = 16.0
    Vi, Br, U, V, X, Y, UVext, XYext = image.vis2bri(prm, UVspan, ngrid)
    amp, pha = oracle.sgra_vis(1, prm.astype(np.float64), U.ravel(), V.ravel())
    Vo = (amp * np.exp(1j * pha)).reshape(U.shape)
    tol = 1e-5 * np.abs(Vo).max() + 1e-5 * np.abs(Vo)
    assert np.all(np.abs(Vi - Vo) <= 2 * tol + 1e-6 * prm[0])
    rho = np.sqrt(U ** 2 + V ** 2)
    cwin = 0.5 * (1 + np.cos(np.pi * rho / (UVspan / 2)))
    cwin[rho > UVspan / 2] = 0
    Bo = np.fft.ifftshift(np.fft.ifft2(np.fft.fftshift(Vo * cwin)))
    assert np.abs(Br - Bo).max() <= 1e-5 * np.abs(Bo).max()
    # total flux of the tapered image = tapered zero-spacing visibility / N^2
    assert X.shape == (ngrid, ngrid) and XYext[0] > XYext[1]
