"""The chi^2 gradient of the Sgr A* model (cmc_grad, cuda_mcmc_gb300.grad).

Checks, in the order they build on each other:
* CPU: the float64 PyTorch re-expression of the model (oracle/torch_sgra.py)
  differentiated by autograd agrees with central differences of the FP64
  oracle chi^2 (oracle.chi2_d) -- this pins the re-expression;
* CPU: the Fisher / proposal host arithmetic on a quadratic with a known
  Hessian (a fake gradient object, no GPU);
* GPU: the CUDA adjoint against autograd of the re-expression at 100 seeded
  parameter points on a 20,000-visibility / 6,000-closure data set, and
  against FP64 central differences of the oracle at a subset; chi^2 against
  the FP64 oracle (relative 1e-5); the autograd.Function; flag handling; the
  Fisher matrix against the autograd Hessian; L-BFGS polish.

Gradient tolerance: float32 sums over N terms carry errors proportional to
the sum of the absolute per-term contributions, not to their (possibly
cancelling) total, so component k is compared as
|g_gpu - g_ref| <= 1e-4 (|g_ref_k| + 1e-2 max_j |g_ref_j|).
"""
import numpy as np
import pytest
import torch

import oracle
from oracle import torch_sgra
from cuda_mcmc_gb300 import synth

GRAD_RTOL = 1e-4
GRAD_FLOOR = 1e-2
CHI2_RTOL = 1e-5

M13_FROM_M9 = (0, 1, 2, 3, 4, None, 5, 6, 7, None, None, None, 8)


def _m13_truth(t9):
    extra = {5: 0.3, 9: 0.4, 10: 0.2, 11: 0.1}
    return np.array([t9[i] if i is not None else extra[k] for k, i in enumerate(M13_FROM_M9)])


def _points(w, n, imodel, seed, spread=0.15):
    """n seeded parameter rows around the truth (+-spread of the prior width),
    inside the region where every model component is on."""
    rng = np.random.default_rng(seed)
    t = w.truth.astype(np.float64)
    lo, hi = w.pmint.astype(np.float64), w.pmaxt.astype(np.float64)
    if imodel == 2:
        t = _m13_truth(t)
        lo = _m13_truth(lo)
        hi = _m13_truth(hi)
        lo[[5, 9, 10, 11]] = [0.0, -np.pi, -np.pi, -np.pi]
        hi[[5, 9, 10, 11]] = [1.0, np.pi, np.pi, np.pi]
    P = t + spread * (hi - lo) * rng.uniform(-1, 1, (n, t.size))
    P = np.clip(P, lo + 0.02 * (hi - lo), hi - 0.02 * (hi - lo))
    return P.astype(np.float32).astype(np.float64)


def _problem(w, imodel):
    nptot = 9 if imodel == 1 else 13
    return oracle.Problem("sgra", w.coor, w.dat, w.std2r, w.icoor, w.idat, nptot, imodel,
                          w.npass)


def _close(g, ref, rtol=GRAD_RTOL, floor=GRAD_FLOOR):
    ref = np.asarray(ref, np.float64)
    scale = np.abs(ref) + floor * np.abs(ref).max(axis=-1, keepdims=True)
    err = np.abs(np.asarray(g, np.float64) - ref) / scale
    return float(err.max())


# ---- CPU ---------------------------------------------------------------------

@pytest.mark.parametrize("imodel", [1, 2])
def test_torch_reexpression_matches_oracle_central_differences(imodel):
    w = synth.sgra(nvis=300, ncph=100, nseq=2, nbeta=4)
    pb = _problem(w, imodel)
    P = _points(w, 6, imodel, seed=11)
    c_t, g_t = torch_sgra.chi2_and_grad(P, w.coor, w.dat, w.std2r, w.icoor, int(w.idat[0]),
                                        w.npass, imodel)
    np.testing.assert_allclose(c_t, oracle.chi2_d(pb, P), rtol=1e-12)
    h = 1e-6 * np.maximum(np.abs(P).max(0), 1e-2)
    g_fd = oracle.chi2_grad_fd(pb, P, h)
    assert _close(g_t, g_fd, rtol=1e-5, floor=1e-3) < 1.0


class _Quadratic:
    """Fake gradient object: chi2 = (p - m)^T A (p - m), grad = 2 A (p - m)."""

    def __init__(self, A, m):
        self.A, self.m = np.asarray(A, np.float64), np.asarray(m, np.float64)

    def __call__(self, P):
        d = np.asarray(P, np.float64) - self.m
        g = 2.0 * d @ self.A
        return (torch.from_numpy(np.einsum("ni,ij,nj->n", d, self.A, d)),
                torch.from_numpy(g.astype(np.float32)))


def test_fisher_of_a_quadratic_is_beta_times_its_matrix():
    from cuda_mcmc_gb300 import grad
    rng = np.random.default_rng(2)
    B = rng.standard_normal((5, 5))
    A = B @ B.T + 5 * np.eye(5)
    q = _Quadratic(A, rng.standard_normal(5))
    F = grad.fisher(q, rng.standard_normal(5), beta=0.5, rel_step=1e-2)
    np.testing.assert_allclose(F, 0.5 * A * 0.5 * 2, rtol=1e-3, atol=1e-3 * np.abs(A).max())
    # a subset of the parameters: the matching sub-block
    F2 = grad.fisher(q, np.zeros(5), ivar=[1, 3], beta=2.0, rel_step=1e-2)
    np.testing.assert_allclose(F2, A[np.ix_([1, 3], [1, 3])] * 2.0, rtol=1e-3)


def test_fisher_projects_an_indefinite_hessian():
    from cuda_mcmc_gb300 import grad
    A = np.diag([4.0, -1.0, 2.0])
    F = grad.fisher(_Quadratic(A, np.zeros(3)), np.ones(3), rel_step=1e-2)
    w = np.linalg.eigvalsh(F)
    assert w.min() > 0
    L = grad.proposal_cholesky(F)
    np.testing.assert_allclose(L @ L.T, np.linalg.inv(F) * 2.38 ** 2 / 3, rtol=1e-10)


# ---- GPU ---------------------------------------------------------------------

@pytest.fixture(scope="module")
def big():
    """20,000 visibilities and 6,000 closure phases (the largest single-fit
    workload's sizes)."""
    return synth.sgra(nvis=20000, ncph=6000, seed=4, nseq=2, nbeta=4)


@pytest.mark.gpu
@pytest.mark.parametrize("imodel", [1, 2])
def test_grad_matches_autograd_of_the_torch_reexpression(big, imodel):
    from cuda_mcmc_gb300.grad import SgraChi2
    w = big
    nptot = 9 if imodel == 1 else 13
    obj = SgraChi2(w.coor, w.dat, w.std2r, w.icoor, w.idat, nptot, imodel, w.npass)
    P = _points(w, 100, imodel, seed=7)
    c, g = obj(P.astype(np.float32))
    c, g = c.cpu().numpy(), g.cpu().numpy()
    c_t, g_t = torch_sgra.chi2_and_grad(P, w.coor, w.dat, w.std2r, w.icoor, int(w.idat[0]),
                                        w.npass, imodel)
    np.testing.assert_allclose(c, c_t, rtol=CHI2_RTOL)
    assert _close(g, g_t) < 1.0


@pytest.mark.gpu
def test_grad_matches_fp64_central_differences_of_the_oracle(big):
    """At 100 seeded parameter points of the 20,000 + 6,000 data: the CUDA
    adjoint against FP64 central differences of the oracle's chi^2
    (h = 1e-6 x the parameter scale)."""
    from cuda_mcmc_gb300.grad import SgraChi2
    w = big
    pb = _problem(w, 1)
    obj = SgraChi2.from_workload(w)
    P = _points(w, 100, 1, seed=3)
    c, g = obj(P.astype(np.float32))
    h = 1e-6 * np.maximum(np.abs(P).max(0), 1e-2)
    g_fd = oracle.chi2_grad_fd(pb, P, h)
    assert _close(g.cpu().numpy(), g_fd) < 1.0
    _, _, _, c64 = oracle.calc_modchi2(pb, P.astype(np.float32))
    np.testing.assert_allclose(c.cpu().numpy(), c64, rtol=CHI2_RTOL)


@pytest.mark.gpu
def test_cpext_closures_and_amplitude_only_pass():
    """npass = 1 (amplitude terms only) and cpExt = 1 (each closure given by its
    triangle's corners u1, v1, u2, v2; the third is -(u1 + u2), -(v1 + v2))."""
    from cuda_mcmc_gb300.grad import SgraChi2
    w = synth.sgra(nvis=400, ncph=150, seed=8, nseq=2, nbeta=4)
    P = _points(w, 8, 1, seed=5)
    obj1 = SgraChi2(w.coor, w.dat, w.std2r, w.icoor, w.idat, 9, 1, npass=1)
    c1, g1 = obj1(P.astype(np.float32))
    c_t, g_t = torch_sgra.chi2_and_grad(P, w.coor, w.dat, w.std2r, w.icoor, int(w.idat[0]), 1, 1)
    np.testing.assert_allclose(c1.cpu().numpy(), c_t, rtol=CHI2_RTOL)
    assert _close(g1.cpu().numpy(), g_t) < 1.0
    rng = np.random.default_rng(12)
    nvis, ncph = int(w.idat[0]), 150
    corners = rng.uniform(-6, 6, (ncph, 4)).astype(np.float32)
    coor = np.concatenate([w.coor[:2 * nvis], corners.ravel()]).astype(np.float32)
    dat = np.concatenate([w.dat[:nvis], rng.uniform(-3, 3, ncph)]).astype(np.float32)
    std2r = np.concatenate([w.std2r[:nvis], np.full(ncph, 100.0)]).astype(np.float32)
    idat = np.array([nvis, 0, 1], np.int32)
    icoor = np.zeros(1, np.int32)
    obj2 = SgraChi2(coor, dat, std2r, icoor, idat, 9, 1, npass=2)
    Q = P[:3]
    c2, g2 = obj2(Q.astype(np.float32))
    pb = oracle.Problem("sgra", coor, dat, std2r, icoor, idat, 9, 1, 2)
    h = 1e-6 * np.maximum(np.abs(Q).max(0), 1e-2)
    np.testing.assert_allclose(c2.cpu().numpy(), oracle.chi2_d(pb, Q), rtol=CHI2_RTOL)
    assert _close(g2.cpu().numpy(), oracle.chi2_grad_fd(pb, Q, h)) < 1.0


@pytest.mark.gpu
def test_autograd_function_and_flags(big):
    from cuda_mcmc_gb300.grad import SgraChi2
    import ctypes as C
    from cuda_mcmc_gb300 import _lib
    w = big
    obj = SgraChi2.from_workload(w)
    P = torch.tensor(_points(w, 6, 1, seed=9), dtype=torch.float64, requires_grad=True)
    loss = (obj.chi2(P) * torch.arange(1, 7, dtype=torch.float64)).sum()
    loss.backward()
    _, g = obj(P.detach().float())
    want = g.cpu().double() * torch.arange(1, 7, dtype=torch.float64)[:, None]
    torch.testing.assert_close(P.grad, want, rtol=1e-6, atol=0)
    # flag[ist] == 0 -> zero chi2 and gradient rows (C-ABI semantics)
    p = torch.tensor(_points(w, 4, 1, seed=10), dtype=torch.float32, device="cuda")
    flag = torch.tensor([1, 0, 1, 0], dtype=torch.int32, device="cuda")
    chi2 = torch.empty(4, device="cuda")
    grad = torch.empty((4, 9), device="cuda")
    j = obj.job
    j.nbeta, j.pcur, j.chi2c, j.flag = 4, p.data_ptr(), chi2.data_ptr(), flag.data_ptr()
    work = torch.empty(int(obj.L.cmc_grad_work_bytes(C.byref(j))), dtype=torch.uint8,
                       device="cuda")
    j.work, j.work_bytes = work.data_ptr(), work.numel()
    _lib.check(obj.L, obj.L.cmc_grad(C.byref(j), C.c_void_p(grad.data_ptr()), None))
    torch.cuda.synchronize()
    j.flag = None
    c_all, g_all = obj(p)
    assert chi2[1].item() == 0 and chi2[3].item() == 0
    assert torch.all(grad[1] == 0) and torch.all(grad[3] == 0)
    torch.testing.assert_close(chi2[[0, 2]], c_all[[0, 2]], rtol=0, atol=0)
    torch.testing.assert_close(grad[[0, 2]], g_all[[0, 2]], rtol=0, atol=0)


@pytest.mark.gpu
@pytest.mark.parametrize("imodel", [1, 2])
def test_gauss_newton_fisher_matches_autograd_jacobian(imodel):
    """cmc_fisher against J^T J from torch.autograd's Jacobian of the weighted
    residuals of the FP64 re-expression, at 3 seeded points: relative
    Frobenius error 1e-4."""
    from cuda_mcmc_gb300.grad import SgraChi2
    w = synth.sgra(nvis=2000, ncph=600, seed=3, nseq=2, nbeta=4)
    nptot = 9 if imodel == 1 else 13
    obj = SgraChi2(w.coor, w.dat, w.std2r, w.icoor, w.idat, nptot, imodel, w.npass)
    P = _points(w, 3, imodel, seed=13)
    F = obj.fisher_gn(P.astype(np.float32)).double().cpu().numpy()
    for q in range(P.shape[0]):
        want = torch_sgra.fisher_gn(P[q], w.coor, w.dat, w.std2r, w.icoor, int(w.idat[0]),
                                    w.npass, imodel)
        rel = np.linalg.norm(F[q] - want) / np.linalg.norm(want)
        assert rel < 1e-4, (q, rel)


def test_torch_gauss_newton_fisher_is_jtj_of_the_chi2():
    """CPU pin of the test-side Gauss-Newton reference: sum r^2 is the chi^2."""
    w = synth.sgra(nvis=200, ncph=60, nseq=2, nbeta=4)
    P = _points(w, 2, 1, seed=4)
    for p in P:
        r = torch_sgra.residuals(torch.tensor(p), w.coor, w.dat, w.std2r, w.icoor,
                                 int(w.idat[0]), w.npass, 1)
        c = torch_sgra.chi2(torch.tensor(p)[None], w.coor, w.dat, w.std2r, w.icoor,
                            int(w.idat[0]), w.npass, 1)
        np.testing.assert_allclose(float((r * r).sum()), float(c[0]), rtol=1e-12)


@pytest.mark.gpu
def test_fisher_matches_the_autograd_hessian():
    from cuda_mcmc_gb300 import grad
    w = synth.sgra(nvis=2000, ncph=600, seed=3, nseq=2, nbeta=4)
    obj = grad.SgraChi2.from_workload(w)
    p = w.truth.astype(np.float64)
    F = grad.fisher(obj, p, beta=1.0, rel_step=1e-3, scale=w.pmaxt - w.pmint)

    def f(x):
        return torch_sgra.chi2(x[None, :], w.coor, w.dat, w.std2r, w.icoor, int(w.idat[0]),
                               w.npass, 1)[0]

    H = torch.autograd.functional.hessian(f, torch.tensor(p)).numpy()
    want = 0.5 * H
    rel = np.linalg.norm(F - want) / np.linalg.norm(want)
    assert rel < 2e-2, rel


@pytest.mark.gpu
def test_polish_descends_to_the_fit():
    from cuda_mcmc_gb300 import grad
    w = synth.sgra(nvis=2000, ncph=600, seed=3, nseq=2, nbeta=4)
    obj = grad.SgraChi2.from_workload(w)
    t = w.truth.astype(np.float64)
    p0 = np.clip(t + 0.03 * (w.pmaxt - w.pmint), w.pmint, w.pmaxt)
    c0 = float(obj(p0[None, :].astype(np.float32))[0][0])
    ct = float(obj(t[None, :].astype(np.float32))[0][0])
    p, c, res = grad.polish(obj, p0, w.pmint, w.pmaxt, maxiter=300)
    assert c < c0
    assert c <= ct * (1 + 1e-4)      # at least as good as the truth that made the data
    # FP64 refinement from the polished point gains (almost) nothing: the
    # float32 polish reached the FP64 optimum's chi^2 to 1e-5
    from scipy.optimize import minimize
    lo, hi = w.pmint.astype(np.float64), w.pmaxt.astype(np.float64)

    def f64(x):
        c64, g64 = torch_sgra.chi2_and_grad(x[None, :], w.coor, w.dat, w.std2r, w.icoor,
                                            int(w.idat[0]), w.npass, 1)
        return float(c64[0]), g64[0]

    c_at_p = f64(p)[0]
    ref = minimize(f64, p, jac=True, method="L-BFGS-B", bounds=list(zip(lo, hi)),
                   options={"maxiter": 500, "ftol": 1e-15, "gtol": 1e-10})
    assert c_at_p - ref.fun <= 1e-5 * ref.fun, (c_at_p, ref.fun)


def test_covariance_and_jittered_cholesky_of_ill_conditioned_information():
    """The Fisher schedule's host algebra: an information matrix with a 1e10
    eigenvalue spread inverts to a covariance whose Cholesky factor
    reproduces it; a singular PSD matrix factors with a tiny jitter."""
    from cuda_mcmc_gb300 import fit
    rng = np.random.default_rng(5)
    Q, _ = np.linalg.qr(rng.standard_normal((9, 9)))
    F = (Q * np.logspace(-2, 8, 9)) @ Q.T
    C = fit.covariance(F)
    np.testing.assert_allclose(C @ F, np.eye(9), atol=1e-6)
    L = fit.cholesky_psd(C)
    np.testing.assert_allclose(L @ L.T, C, rtol=1e-8, atol=1e-12 * np.abs(C).max())
    S = np.outer(np.arange(1, 4), np.arange(1, 4)).astype(np.float64)   # rank 1
    Ls = fit.cholesky_psd(S)
    np.testing.assert_allclose(Ls @ Ls.T, S, atol=1e-6 * S.max())
