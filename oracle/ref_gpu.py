"""The reference's own CUDA build on the GPU: its kernels, launched in its order.

TEST INFRASTRUCTURE ONLY (the parity tests and the ``ref_gpu`` figure of
bench.py use it; nothing in the cuda_mcmc_gb300 package does).

oracle/ref_build.py compiles the reference's src/gpu_mcmc.cu, unchanged, with
an example's model.cuh for sm_103a into ``oracle/_ref/ref_gpu_<model>.cubin``
(and ``.ptx``), and records the byte layout of its CMcmcFit job object
(``ref_gpu_layout.json``).  This module loads that code through the CUDA
driver API (libcuda, ctypes) into the current context -- the one PyTorch
uses -- and plays the role of the reference's host code:

  * CMcmcFit::CMcmcFit (src/mcmcjob.cu:552-755): the device arrays (torch
    tensors here) and the job object, built byte by byte from the recorded
    layout and copied to the device;
  * run_mcmc (src/gpu_mcmc.cu:682-763): init_rng, init_pcur,
    calc_chi2_terms x npass, calc_chi2, then per iteration and mutable
    parameter gen_proposal, calc_chi2_terms x npass, spmp_mcmc,
    adjust_steps (burn-in only), and one replica_exchange per iteration, with
    the reference's launch shapes (<<<nseq, nbeta>>> for the per-replica
    kernels, <<<nbeta*nseq*ndat/128 + 1, 128>>> for the model,
    <<<nseq, 1>>> for the exchange);
  * run_calcmodchi2 (:769-783).

Iterations can be run one at a time and the state read and overwritten in
between, which the lock-step parity tests use: the reference's generator
states (curandState, 48 bytes per replica) are plain device memory here.
"""
from __future__ import annotations

import ctypes as C
import json
import os

import numpy as np

from . import ref_build

# Itanium-mangled names of the reference's kernels (src/gpu_mcmc.cu:228-658)
KERNELS = {
    "init_rng": "_Z8init_rngP8CMcmcFit",
    "init_pcur": "_Z9init_pcurP8CMcmcFit",
    "calc_chi2_terms": "_Z15calc_chi2_termsP10CCalcModeli",
    "calc_chi2": "_Z9calc_chi2P10CCalcModel",
    "gen_proposal": "_Z12gen_proposalP8CMcmcFit",
    "spmp_mcmc": "_Z9spmp_mcmcP8CMcmcFit",
    "adjust_steps": "_Z12adjust_stepsP8CMcmcFit",
    "replica_exchange": "_Z16replica_exchangeP8CMcmcFitii",
    "calc_model": "_Z10calc_modelP10CCalcModel",
}
BLOCKSIZE = 128   # run_mcmc's model launch block size (src/gpu_mcmc.cu:686)


def available(model: str = "sgra") -> bool:
    p = ref_build.gpu_paths(model)
    return os.path.isfile(p["layout"]) and (os.path.isfile(p["cubin"]) or os.path.isfile(p["ptx"]))


_cuda = None


def _libcuda():
    global _cuda
    if _cuda is None:
        L = C.CDLL("libcuda.so.1")
        for n in ("cuInit", "cuCtxGetCurrent", "cuModuleLoadData", "cuModuleGetFunction",
                  "cuLaunchKernel", "cuGetErrorString"):
            getattr(L, n).restype = C.c_int
        _cuda = L
    return _cuda


def _check(rc, what):
    if rc != 0:
        s = C.c_char_p()
        _libcuda().cuGetErrorString(rc, C.byref(s))
        raise RuntimeError("%s failed: %s (%d)" % (what, (s.value or b"?").decode(), rc))


_draws = None


def _build_draws():
    """Compile oracle/curand_draws.cu into oracle/_build/libcurand_draws.so."""
    here = os.path.dirname(os.path.abspath(__file__))
    src = os.path.join(here, "curand_draws.cu")
    out = os.path.join(here, "_build", "libcurand_draws.so")
    if not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(src):
        import subprocess
        os.makedirs(os.path.dirname(out), exist_ok=True)
        tmp = out + ".tmp%d" % os.getpid()
        subprocess.run([ref_build._nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O2",
                        "-shared", "-Xcompiler", "-fPIC", "-o", tmp, src], check=True)
        os.replace(tmp, out)
    return out


def next_uniforms(states, per):
    """The next ``per`` uniforms of every cuRAND XORWOW state in the device
    tensor ``states`` [..., 48] (uint8), as a float32 array [n, per]; the
    states are left unchanged."""
    global _draws
    import torch
    if _draws is None:
        _draws = C.CDLL(_build_draws())
        _draws.cd_next_uniforms.restype = C.c_int
    st = states.contiguous()
    n = st.numel() // 48
    out = torch.empty((n, per), dtype=torch.float32, device=st.device)
    rc = _draws.cd_next_uniforms(C.c_void_p(st.data_ptr()), n, per, C.c_void_p(out.data_ptr()),
                                 C.c_void_p(torch.cuda.current_stream().cuda_stream))
    if rc != 0:
        raise RuntimeError("cd_next_uniforms: CUDA error %d" % rc)
    return out.cpu().numpy()


class _Module:
    """The reference's kernels of one model, loaded into the current context."""

    _cache = {}

    def __init__(self, model):
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")            # the primary context is current now
        L = _libcuda()
        _check(L.cuInit(0), "cuInit")
        ctx = C.c_void_p()
        _check(L.cuCtxGetCurrent(C.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context")
        p = ref_build.gpu_paths(model)
        path = p["cubin"] if os.path.isfile(p["cubin"]) else p["ptx"]
        with open(path, "rb") as f:
            image = f.read()
        if path.endswith(".ptx"):
            image += b"\0"
        self.image = C.create_string_buffer(image, len(image))
        self.mod = C.c_void_p()
        _check(L.cuModuleLoadData(C.byref(self.mod), self.image), "cuModuleLoadData(%s)" % path)
        self.fn = {}
        for k, name in KERNELS.items():
            f = C.c_void_p()
            _check(L.cuModuleGetFunction(C.byref(f), self.mod, name.encode()),
                   "cuModuleGetFunction(%s)" % name)
            self.fn[k] = f
        self.path = path
        with open(p["layout"]) as f:
            self.layout = json.load(f)

    @classmethod
    def get(cls, model):
        if model not in cls._cache:
            cls._cache[model] = cls(model)
        return cls._cache[model]


class RefGpuJob:
    """One CMcmcFit of the reference's CUDA build with its arrays on the GPU.

    ``state`` holds the starting sampler arrays in the reference's layouts
    (as imgpu.Mcgpu builds them: pdescr, ivar, invar, ptotal, pmint, pmaxt,
    pcur, pstp, tcur, chi2c, flag, ptent, ptentn, n_acpt, n_exch, n_cnt,
    n_hist)."""

    def __init__(self, model, coor, dat, std2r, icoor, idat, beta, state, nseq, niter,
                 seed, imodel=1, npass=2, nadj=100, nburn=0, ndatm=None):
        import torch
        self.torch = torch
        self.M = _Module.get(model)
        lay = self.M.layout
        if lay["sizeof_curandState"] != 48 or lay["sizeof_pointer"] != 8:
            raise RuntimeError("unexpected reference layout")
        beta = np.ascontiguousarray(beta, np.float32)
        self.nbeta, self.nseq = int(beta.size), int(nseq)
        nrep = self.nbeta * self.nseq
        pdescr = np.ascontiguousarray(state["pdescr"], np.int32)
        self.nptot = int(pdescr.size)
        self.nprm = int(np.count_nonzero(pdescr))
        self.ndat = int(np.asarray(dat).size)
        self.npass, self.nadj, self.niter, self.nburn = int(npass), int(nadj), int(niter), int(nburn)
        idat = np.ascontiguousarray(idat, np.int32)
        icoor = np.ascontiguousarray(icoor, np.int32)
        if icoor.size == 0:
            icoor = np.zeros(1, np.int32)
        nvis = int(idat[0]) if model == "sgra" else 0
        self.ndatm = int(ndatm) if ndatm is not None else nrep * (self.ndat + nvis)
        dev = torch.device("cuda")

        def f32(a):
            return torch.as_tensor(np.ascontiguousarray(a, np.float32)).to(dev).contiguous()

        def i32(a):
            return torch.as_tensor(np.ascontiguousarray(a, np.int32)).to(dev).contiguous()

        t = {"coor": f32(coor), "dat": f32(dat), "std2r": f32(std2r), "icoor": i32(icoor),
             "idat": i32(idat), "beta": f32(beta)}
        for k in ("pdescr", "ivar", "invar"):
            t[k] = i32(state[k])
        for k in ("ptotal", "pmint", "pmaxt", "pcur", "pstp", "chi2c", "ptent"):
            t[k] = f32(state[k])
        for k in ("tcur", "flag", "ptentn", "n_acpt", "n_exch", "n_cnt", "n_hist"):
            t[k] = i32(state[k])
        nt = max(self.niter, 1)
        t["pout"] = torch.zeros((self.nprm, self.nbeta, self.nseq, nt), dtype=torch.float32, device=dev)
        t["tout"] = torch.zeros((self.nbeta, self.nseq, nt), dtype=torch.int32, device=dev)
        t["chi2"] = torch.zeros((self.nseq, nt), dtype=torch.float32, device=dev)
        t["datm"] = torch.zeros(max(self.ndatm, 1), dtype=torch.float32, device=dev)
        t["chi2m"] = torch.zeros((self.nbeta, self.nseq, self.ndat), dtype=torch.float32, device=dev)
        t["rndst"] = torch.zeros((self.nbeta, self.nseq, 48), dtype=torch.uint8, device=dev)
        self.t = t

        # the job object, member by member (CMcmcFit::CMcmcFit, src/mcmcjob.cu:598-652)
        img = bytearray(lay["sizeof_CMcmcFit"])
        off = lay["offsets"]

        def put_i(name, v):
            img[off[name]:off[name] + 4] = np.int32(v).tobytes()

        def put_p(name, tensor):
            img[off[name]:off[name] + 8] = np.uint64(tensor.data_ptr()).tobytes()

        for name, v in (("imodel", imodel), ("ncoor", t["coor"].numel()), ("ndat", self.ndat),
                        ("nicoor", icoor.size), ("nidat", idat.size), ("ndatm", self.ndatm),
                        ("nptot", self.nptot), ("nbeta", self.nbeta), ("nseq", self.nseq),
                        ("nchi2m", nrep * self.ndat), ("nprm", self.nprm), ("nadj", self.nadj),
                        ("npass", self.npass), ("nburn", self.nburn), ("niter", self.niter),
                        ("nrndst", nrep), ("ipm", 0), ("itr", 0),
                        ("ntitr", self.nburn + self.niter)):
            put_i(name, v)
        img[off["seed"]:off["seed"] + 8] = np.uint64(seed).tobytes()
        for name in ("coor", "dat", "std2r", "icoor", "idat", "datm", "chi2m", "pcur", "flag",
                     "chi2c", "rndst", "pdescr", "ivar", "invar", "ptotal", "pmint", "pmaxt",
                     "pout", "tout", "chi2", "tcur", "n_acpt", "n_exch", "n_cnt", "n_hist",
                     "pstp", "beta", "ptent", "ptentn"):
            put_p(name, t[name])
        self.mc = torch.tensor(np.frombuffer(bytes(img), np.uint8).copy(), device=dev)
        self._mcp = C.c_uint64(self.mc.data_ptr())
        self.nblocks = nrep * self.ndat // BLOCKSIZE + 1
        self.launches = 0

    # ---- launching -----------------------------------------------------------
    def _launch(self, name, grid, block, *ints):
        args = [C.pointer(self._mcp)] + [C.pointer(C.c_int(v)) for v in ints]
        params = (C.c_void_p * len(args))(*[C.cast(a, C.c_void_p) for a in args])
        stream = self.torch.cuda.current_stream().cuda_stream
        _check(_libcuda().cuLaunchKernel(self.M.fn[name], grid, 1, 1, block, 1, 1, 0,
                                         C.c_void_p(stream), params, None), name)
        self.launches += 1

    def _chi2_terms(self):
        for ipass in range(self.npass):
            self._launch("calc_chi2_terms", self.nblocks, BLOCKSIZE, ipass)

    def init(self):
        """init_rng, init_pcur and the first chi^2 (src/gpu_mcmc.cu:714-719)."""
        self._launch("init_rng", self.nseq, self.nbeta)
        self._launch("init_pcur", self.nseq, self.nbeta)
        self._chi2_terms()
        self._launch("calc_chi2", self.nseq, self.nbeta)

    def iteration(self, burn, itr):
        """One burn-in (burn=True) or main iteration recorded at column itr
        (src/gpu_mcmc.cu:727-757)."""
        for _ in range(self.nprm):
            self._launch("gen_proposal", self.nseq, self.nbeta)
            self._chi2_terms()
            self._launch("spmp_mcmc", self.nseq, self.nbeta)
            if burn:
                self._launch("adjust_steps", self.nseq, self.nbeta)
        self._launch("replica_exchange", self.nseq, 1, 1 if burn else 0, int(itr))

    def iteration_trace(self, burn, itr, chi2_rtol=1e-5, floor=1e-3):
        """iteration() launched kernel by kernel, reading the decision inputs
        in between: for each Metropolis decision of spmp_mcmc
        (src/gpu_mcmc.cu:426-474) its acceptance probability alpha from the
        chi2m row the reference just computed and the uniform u its
        generator gives next, and likewise for every exchange attempt of
        replica_exchange (:533-626).  A decision compares u with
        alpha = min(1, e^x), x = -beta/2 (chi2_new - chi2_cur) (exchange:
        -(beta_k+1 - beta_k)/2 (chi2_k - chi2_k+1)); chi^2 values that differ
        by a relative ``chi2_rtol`` move x by up to
        w = |beta|/2 chi2_rtol (|chi2_new| + |chi2_cur|).  Returns per
        sequence the smallest |ln u - x| / max(w, floor) over its decisions
        (inf where none was taken): below 1, float32 chi^2 rounding within
        the tolerance may flip that decision."""
        torch = self.torch
        nb, ns = self.nbeta, self.nseq
        old_err = np.seterr(over="ignore")
        beta = self.t["beta"].cpu().numpy()
        best = np.full(ns, np.inf)
        for _ in range(self.nprm):
            self._launch("gen_proposal", ns, nb)
            self._chi2_terms()
            torch.cuda.synchronize()
            flag = self.t["flag"].cpu().numpy()
            c2c = self.t["chi2c"].cpu().numpy()
            rows = self.t["chi2m"].cpu().numpy()
            c2 = np.cumsum(rows, axis=-1, dtype=np.float32)[..., -1]   # the serial float sum
            u = next_uniforms(self.t["rndst"], 1).reshape(nb, ns).astype(np.float64)
            x = -0.5 * beta[:, None].astype(np.float64) * (c2.astype(np.float64) - c2c)
            wdt = 0.5 * beta[:, None] * chi2_rtol * (np.abs(c2) + np.abs(c2c))
            m = np.abs(np.log(u) - x) / np.maximum(wdt, floor)
            m = np.where(flag != 0, m, np.inf)
            best = np.minimum(best, m.min(axis=0))
            self._launch("spmp_mcmc", ns, nb)
            if burn:
                self._launch("adjust_steps", ns, nb)
        torch.cuda.synchronize()
        c2c = self.t["chi2c"].cpu().numpy()
        extra = 8
        us = next_uniforms(self.t["rndst"][0], 2 * nb + extra)        # replica ibeta = 0
        for q in range(ns):
            chi = c2c[:, q].copy()
            pos = 0
            for _ in range(nb):
                while True:
                    k = int(np.float32(nb - 1) * us[q, pos])
                    pos += 1
                    if k < nb - 1 or pos >= us.shape[1] - 1:
                        break
                db = float(beta[k + 1]) - float(beta[k])
                x = -0.5 * db * (float(chi[k]) - float(chi[k + 1]))
                a = np.float32(np.exp(np.float32(-0.5) * (beta[k + 1] - beta[k]) * (chi[k] - chi[k + 1])))
                alpha = min(a, np.float32(1.0))
                u = us[q, pos]
                pos += 1
                wdt = 0.5 * abs(db) * chi2_rtol * (abs(float(chi[k])) + abs(float(chi[k + 1])))
                best[q] = min(best[q], abs(np.log(float(u)) - x) / max(wdt, floor))
                if u <= alpha:
                    chi[k], chi[k + 1] = chi[k + 1], chi[k]
        self._launch("replica_exchange", ns, 1, 1 if burn else 0, int(itr))
        np.seterr(**old_err)
        return best

    def run(self, nburn, niter):
        """run_mcmc: init, nburn burn-in and niter main iterations."""
        self.init()
        for itr in range(nburn):
            self.iteration(True, itr)
        for itr in range(niter):
            self.iteration(False, itr)

    def calc_modchi2(self):
        """run_calcmodchi2 (src/gpu_mcmc.cu:769-783) on the current pcur / flag."""
        self._launch("calc_chi2_terms", self.nblocks, BLOCKSIZE, 0)
        self._launch("calc_chi2_terms", self.nblocks, BLOCKSIZE, 1)
        self._launch("calc_chi2", self.nseq, self.nbeta)

    # ---- state access --------------------------------------------------------------
    def to_numpy(self, fields=None):
        self.torch.cuda.synchronize()
        keys = fields or [k for k in self.t if k not in ("coor", "dat", "std2r", "icoor", "idat")]
        return {k: self.t[k].cpu().numpy() for k in keys}

    def set_state(self, **arrays):
        for k, v in arrays.items():
            dst = self.t[k]
            src = self.torch.as_tensor(np.ascontiguousarray(v)).to(dtype=dst.dtype)
            dst.copy_(src.reshape(dst.shape).to(dst.device))
