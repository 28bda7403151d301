"""Device-resident sampler jobs: the C-ABI's ``cmc_run`` / ``cmc_eval`` on
arrays that stay in GPU memory (PyTorch tensors used as plain device buffers).

A :class:`DeviceJob` holds one problem (data + parameter description) and
the full sampler state in the reference's layouts.  ``run()`` launches the
fused sweep for any number of burn-in / main iterations and can resume from
the current state, so long runs can be split into chunks (and captured in
CUDA graphs) without changing the chain: a run split into chunks walks the
same chain as one launch over all iterations.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib

_F32, _I32, _U8 = torch.float32, torch.int32, torch.uint8

# state arrays copied back by to_numpy(), in the reference's shapes
STATE_FIELDS = ("pcur", "chi2c", "flag", "ptent", "ptentn", "pstp", "n_acpt", "n_exch",
                "n_cnt", "n_hist", "tcur", "rndst", "pout", "tout", "chi2", "datm", "chi2m")


def sampler_defaults(pdescr, pmint, pmaxt, nbeta, nseq, nadj=100, ptotal=None, pstp=None):
    """Initial state as imgpu.Mcgpu builds it (src/imgpu.py:320-424): ivar /
    invar maps, pcur at the prior centres (ptotal for frozen parameters),
    pstp = (pmax - pmin)/50 unless given, tcur = 0..nbeta-1 per sequence,
    n_cnt = 1 and zeroed counters."""
    pdescr = np.ascontiguousarray(pdescr, np.int32)
    nptot = pdescr.size
    pmint = np.ascontiguousarray(pmint, np.float32)
    pmaxt = np.ascontiguousarray(pmaxt, np.float32)
    ivar = np.where(pdescr != 0)[0].astype(np.int32)
    nprm = ivar.size
    invar = np.full(nptot, -1, np.int32)
    invar[ivar] = np.arange(nprm, dtype=np.int32)
    ptotal = np.zeros(nptot, np.float32) if ptotal is None else np.asarray(ptotal, np.float32)
    pcur = np.empty((nbeta, nseq, nptot), np.float32)
    pcur[:] = ptotal
    pcur[:, :, ivar] = pmint[ivar] + (pmaxt[ivar] - pmint[ivar]) / np.float32(2.0)
    st = np.empty((nprm, nbeta, nseq), np.float32)
    if pstp is None:
        st[:] = ((pmaxt[ivar] - pmint[ivar]) / 50.0).astype(np.float32)[:, None, None]
    else:
        p = np.asarray(pstp, np.float32)
        st[:] = p.reshape(nprm, 1, 1) if p.size == nprm else p.reshape(nprm, nbeta, nseq)
    tcur = np.empty((nbeta, nseq), np.int32)
    tcur[:] = np.arange(nbeta, dtype=np.int32)[:, None]
    return dict(pdescr=pdescr, ivar=ivar, invar=invar, ptotal=ptotal, pmint=pmint, pmaxt=pmaxt,
                pcur=pcur, pstp=st, tcur=tcur,
                chi2c=np.zeros((nbeta, nseq), np.float32),
                flag=np.zeros((nbeta, nseq), np.int32),
                ptent=np.zeros((nbeta, nseq), np.float32),
                ptentn=np.zeros((nbeta, nseq), np.int32),
                n_acpt=np.zeros((nprm, nbeta, nseq), np.int32),
                n_exch=np.zeros((nbeta, nseq), np.int32),
                n_cnt=np.ones((nprm, nbeta, nseq), np.int32),
                n_hist=np.zeros((nadj, nprm, nbeta, nseq), np.int32))


def _dev(a, dtype, device):
    return torch.as_tensor(np.ascontiguousarray(a)).to(device=device, dtype=dtype).contiguous()


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None and t.numel() > 0 else C.c_void_p(0)


class DeviceJob:
    """One MCMC-RE problem with all arrays resident on ``device``.

    rng = "curand" uses the reference's generator (curand_init(seed, ist, 0));
    rng = "injected" reads uniforms / normals from ``streams = (u, n)``,
    float32 arrays [nbeta*nseq, L] consumed in the reference's draw order.
    """

    def __init__(self, model, coor, dat, std2r, icoor, idat, pdescr, pmint, pmaxt, beta,
                 nseq, niter_total, imodel=1, npass=1, nadj=100, ptotal=None, pstp=None,
                 seed=1234, rng="curand", streams=None, ndatm=None, device="cuda",
                 lib=None, seq_offset=0, nseq_total=0):
        self.L = lib if lib is not None else _lib.load(model)
        self.device = torch.device(device)
        d = self.device
        beta = np.ascontiguousarray(beta, np.float32)
        self.nbeta, self.nseq = int(beta.size), int(nseq)
        nrep = self.nbeta * self.nseq
        s = sampler_defaults(pdescr, pmint, pmaxt, self.nbeta, self.nseq, nadj, ptotal, pstp)
        self.nptot, self.nprm, self.nadj = int(s["pdescr"].size), int(s["ivar"].size), int(nadj)
        self.ndat = int(np.asarray(dat).size)
        idat = np.ascontiguousarray(idat, np.int32)
        nvis = int(idat[0]) if model == "sgra" else 0
        self.nvis = nvis
        self.ndatm = int(ndatm) if ndatm is not None else nrep * (self.ndat + nvis)
        self.niter_total = int(niter_total)
        icoor = np.ascontiguousarray(icoor, np.int32)
        if icoor.size == 0:
            icoor = np.zeros(1, np.int32)
        t = {}
        t["coor"] = _dev(coor, _F32, d)
        t["dat"] = _dev(dat, _F32, d)
        t["std2r"] = _dev(std2r, _F32, d)
        t["icoor"] = _dev(icoor, _I32, d)
        t["idat"] = _dev(idat, _I32, d)
        for k in ("pdescr", "ivar", "invar"):
            t[k] = _dev(s[k], _I32, d)
        for k in ("pmint", "pmaxt"):
            t[k] = _dev(s[k], _F32, d)
        t["beta"] = _dev(beta, _F32, d)
        for k in ("pcur", "chi2c", "ptent", "pstp"):
            t[k] = _dev(s[k], _F32, d)
        for k in ("flag", "ptentn", "n_acpt", "n_exch", "n_cnt", "n_hist", "tcur"):
            t[k] = _dev(s[k], _I32, d)
        t["rndst"] = torch.zeros((self.nbeta, self.nseq, 48), dtype=_U8, device=d)
        nt = max(self.niter_total, 1)
        t["pout"] = torch.zeros((self.nprm, self.nbeta, self.nseq, nt), dtype=_F32, device=d)
        t["tout"] = torch.zeros((self.nbeta, self.nseq, nt), dtype=_I32, device=d)
        t["chi2"] = torch.zeros((self.nseq, nt), dtype=_F32, device=d)
        t["datm"] = torch.zeros(max(self.ndatm, 1), dtype=_F32, device=d)
        t["chi2m"] = torch.zeros((self.nbeta, self.nseq, self.ndat), dtype=_F32, device=d)
        t["status"] = torch.zeros(4, dtype=_I32, device=d)
        self.rng = rng
        if rng == "injected":
            if streams is None:
                raise ValueError("rng='injected' needs streams=(u, n)")
            u, n = streams
            t["inj_u"] = _dev(u, _F32, d)
            t["inj_n"] = _dev(n, _F32, d)
            t["inj_cur"] = torch.zeros((nrep, 2), dtype=_I32, device=d)
        elif rng != "curand":
            raise ValueError("rng must be 'curand' or 'injected'")
        self.t = t
        j = _lib.CmcJob()
        j.ncoor, j.ndat, j.nicoor, j.nidat = int(t["coor"].numel()), self.ndat, \
            int(icoor.size), int(idat.size)
        j.ndatm, j.nptot, j.nprm, j.nadj = self.ndatm, self.nptot, self.nprm, self.nadj
        j.npass, j.nbeta, j.nseq, j.imodel = int(npass), self.nbeta, self.nseq, int(imodel)
        j.niter_total = self.niter_total
        j.rng_mode = _lib.CMC_RNG_INJECTED if rng == "injected" else _lib.CMC_RNG_CURAND
        j.seed = int(np.uint64(seed))
        # a shard of sequences [seq_offset, seq_offset + nseq) of an
        # nseq_total-sequence run (see cmc_job.h); 0 = unsharded
        if nseq_total and not (0 <= seq_offset and seq_offset + self.nseq <= nseq_total):
            raise ValueError("shard [%d, %d) outside 0..%d" % (seq_offset, seq_offset + self.nseq,
                                                               nseq_total))
        j.seq_offset, j.nseq_total = int(seq_offset), int(nseq_total)
        self.seq_offset, self.nseq_total = int(seq_offset), int(nseq_total)
        for i in range(4):
            j.hidat[i] = int(idat[i]) if i < idat.size else 0
        for k in ("coor", "dat", "std2r", "icoor", "idat", "pdescr", "ivar", "invar", "pmint",
                  "pmaxt", "beta", "pcur", "chi2c", "flag", "ptent", "ptentn", "pstp", "n_acpt",
                  "n_exch", "n_cnt", "n_hist", "tcur", "rndst", "pout", "tout", "chi2", "datm",
                  "chi2m", "status"):
            setattr(j, k, _ptr(t[k]))
        if rng == "injected":
            j.inj_u, j.inj_n, j.inj_cur = _ptr(t["inj_u"]), _ptr(t["inj_n"]), _ptr(t["inj_cur"])
            j.inj_lu, j.inj_ln = int(t["inj_u"].shape[1]), int(t["inj_n"].shape[1])
        wb = int(self.L.cmc_work_bytes(C.byref(j), 0))
        t["work"] = torch.zeros(max(wb, 16), dtype=_U8, device=d)
        j.work, j.work_bytes = _ptr(t["work"]), wb
        self.job = j
        self.itr_done = 0
        self.shape = None          # forced launch shape {R, T, phasor[, layout]} (autotune.py)

    @classmethod
    def from_workload(cls, w, niter_total=None, seed=1234, rng="curand", streams=None,
                      device="cuda", lib=None, seqs=None):
        """``seqs`` = (s0, s1): only sequences s0..s1-1 of the workload's nseq
        (a shard; its chains are those sequences of the unsharded run)."""
        nseq, off, tot = w.nseq, 0, 0
        if seqs is not None:
            off, tot = int(seqs[0]), w.nseq
            nseq = int(seqs[1]) - off
        return cls(w.model, w.coor, w.dat, w.std2r, w.icoor, w.idat, w.pdescr, w.pmint, w.pmaxt,
                   w.beta(), nseq, w.niter if niter_total is None else niter_total,
                   imodel=w.imodel, npass=w.npass, ptotal=w.ptotal, pstp=w.pstp0, seed=seed,
                   rng=rng, streams=streams, device=device, lib=lib, seq_offset=off,
                   nseq_total=tot)

    # ---- launching -----------------------------------------------------------
    def run(self, nburn=0, niter=0, do_init=False, itr0=None, stream=None):
        """Launch the fused sweep on ``stream`` (torch's current stream by
        default).  Main iterations are recorded from column ``itr0`` (default:
        after the previously recorded ones).  Asynchronous: call
        :meth:`check` to synchronise and read the device status."""
        j = self.job
        j.do_init = 1 if do_init else 0
        j.nburn, j.niter = int(nburn), int(niter)
        j.itr0 = self.itr_done if itr0 is None else int(itr0)
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        self._force_shape()
        try:
            _lib.check(self.L, self.L.cmc_run(C.byref(j), C.c_void_p(s.cuda_stream)))
        finally:
            self._release_shape()
        self.itr_done = j.itr0 + j.niter

    def graph_schedule(self, nburn, niter, chunk=256, itr0=0):
        """Capture a sweep schedule of this job as ONE CUDA graph: nburn
        burn-in iterations, then niter recorded ones (columns itr0 ..), as
        launches of at most ``chunk`` iterations.  Replaying the graph once
        runs the schedule from the job's current state (the launch shape and
        the packed data are fixed at capture)."""
        g = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.graph(g, stream=side):
            done = 0
            while done < nburn:
                n = min(chunk, nburn - done)
                self.run(n, 0, itr0=itr0, stream=side)
                done += n
            done = 0
            while done < niter:
                n = min(chunk, niter - done)
                self.run(0, n, itr0=itr0 + done, stream=side)
                done += n
        self.itr_done = itr0 + niter
        return g

    def autotune(self, **kw):
        """Time every feasible launch shape on this job and keep the fastest."""
        from . import autotune
        return autotune.tune(self, **kw)

    def eval(self, mode=_lib.MODE_MODCHI2, stream=None):
        """calc_modchi2 (mode 1) / calc_model (mode 2) on the current pcur."""
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        _lib.check(self.L, self.L.cmc_eval(C.byref(self.job), int(mode),
                                           C.c_void_p(s.cuda_stream)))

    def check(self):
        torch.cuda.synchronize(self.device)
        st = int(self.t["status"][0].item())
        if st:
            raise _lib.McmcError(st, "device status %d (see cmc_status in cmc_job.h)" % st)

    def clear_status(self):
        """Reset the device status word (after an error or a batch cancel was
        read), so that the job can run again."""
        self.t["status"].zero_()

    def _force_shape(self):
        if self.shape:
            self.L.cmc_set_config(self.shape["R"], self.shape["T"], self.shape["phasor"])
            self.L.cmc_set_layout(int(self.shape.get("layout", 0)))
            self.L.cmc_set_spread(int(self.shape.get("groups", 0)),
                                  int(self.shape.get("blocks", 0)))

    def _release_shape(self):
        if self.shape:
            self.L.cmc_set_config(0, 0, -1)
            self.L.cmc_set_layout(0)
            self.L.cmc_set_spread(0, 0)

    def config(self):
        """Launch shape used for this job: R, G, T, phasor, smem, clusters/wave
        and the layout ("cluster", or "spread" with G = 0, `blocks` CTAs and
        `groups` sequence groups)."""
        R, G, T, P, W, NB, NG = (C.c_int() for _ in range(7))
        sm = C.c_size_t()
        self._force_shape()
        try:
            _lib.check(self.L, self.L.cmc_query_config(C.byref(self.job), C.byref(R), C.byref(G),
                                                       C.byref(T), C.byref(P), C.byref(sm),
                                                       C.byref(W)))
            _lib.check(self.L, self.L.cmc_query_spread(C.byref(self.job), C.byref(NB),
                                                       C.byref(NG)))
        finally:
            self._release_shape()
        out = dict(R=R.value, G=G.value, T=T.value, phasor=P.value, smem=sm.value,
                   clusters_per_wave=W.value, layout="cluster" if G.value else "spread")
        if not G.value:
            out["blocks"] = NB.value
            out["groups"] = NG.value
        return out

    # ---- state access ----------------------------------------------------------
    def to_numpy(self, fields=STATE_FIELDS):
        torch.cuda.synchronize(self.device)
        out = {k: self.t[k].cpu().numpy() for k in fields}
        if self.rng == "injected":
            out["inj_cur"] = self.t["inj_cur"].cpu().numpy()
        return out

    def set_state(self, **arrays):
        """Overwrite device state arrays from host arrays of the same shapes."""
        for k, v in arrays.items():
            dst = self.t[k]
            src = torch.as_tensor(np.ascontiguousarray(v)).to(dtype=dst.dtype).reshape(dst.shape)
            dst.copy_(src.to(self.device))

    # ---- proposals ---------------------------------------------------------------
    def set_block_proposals(self, chol, scale=None):
        """Switch to block proposals p += pstp[0] * L z for all nprm parameters
        at once.  ``chol`` [nseq, nprm, nprm] (or [nprm, nprm] for every
        sequence): lower Cholesky factors of the beta = 1 proposal covariance
        in ivar order.  ``scale`` [nbeta, nseq] (default 1/sqrt(beta), the
        tempered target's width) becomes pstp[0], the per-replica step that
        burn-in keeps adapting.  The acceptance counters of slot 0 restart."""
        chol = np.asarray(chol, np.float32)
        if chol.ndim == 2:
            chol = np.broadcast_to(chol, (self.nseq,) + chol.shape)
        if chol.shape != (self.nseq, self.nprm, self.nprm):
            raise ValueError("chol must be [nseq, nprm, nprm] = [%d, %d, %d]"
                             % (self.nseq, self.nprm, self.nprm))
        self.t["prop_chol"] = _dev(np.tril(chol), _F32, self.device)
        beta = self.t["beta"].double()
        if scale is None:
            scale = (1.0 / torch.sqrt(beta))[:, None].expand(self.nbeta, self.nseq)
        scale = torch.as_tensor(np.asarray(scale, np.float32) if not torch.is_tensor(scale)
                                else scale).to(self.device, _F32).reshape(self.nbeta, self.nseq)
        self.t["pstp"][0].copy_(scale)
        self.t["n_cnt"][0].fill_(1)
        self.t["n_acpt"][0].zero_()
        self.t["n_hist"][:, 0].zero_()
        self.job.prop_chol = _ptr(self.t["prop_chol"])
        self.job.prop_mode = _lib.CMC_PROP_BLOCK

    def set_single_proposals(self, pstp0=None):
        """Back to the reference's one-parameter proposals; ``pstp0`` [nbeta,
        nseq] restores parameter 0's step (block mode used pstp[0] as its
        scale)."""
        self.job.prop_mode = _lib.CMC_PROP_SINGLE
        self.job.prop_chol = None
        if pstp0 is not None:
            self.t["pstp"][0].copy_(torch.as_tensor(np.asarray(pstp0, np.float32)).to(self.device)
                                    .reshape(self.nbeta, self.nseq))


class BatchJob:
    """Many independent fits of one model (DeviceJobs with the same nbeta) run
    by persistent work-list launches: the (fit, sequence) items are split into
    size classes, each class one launch whose clusters take items from an
    atomic counter, largest first.  ``run()`` only launches (the descriptors
    and work lists are built once here), so a chunk loop can be captured in a
    CUDA graph."""

    def __init__(self, jobs, stream=None):
        if not jobs:
            raise ValueError("BatchJob needs at least one DeviceJob")
        self.jobs = list(jobs)
        self.L = self.jobs[0].L
        self.device = self.jobs[0].device
        if any(j.L is not self.L for j in self.jobs):
            raise ValueError("all jobs of a batch must use the same model library")
        n = len(self.jobs)
        arr = (_lib.CmcJob * n)(*[j.job for j in self.jobs])
        wb = int(self.L.cmc_batch_work_bytes(arr, n))
        self.work = torch.zeros(max(wb, 16), dtype=_U8, device=self.device)
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        plan = self.L.cmc_batch_prepare(arr, n, C.c_void_p(self.work.data_ptr()), wb,
                                        C.c_void_p(s.cuda_stream))
        if not plan:
            raise _lib.McmcError(_lib.CMC_ERR_ARG, self.L.cmc_last_error().decode())
        self.plan = C.c_void_p(plan)
        self.itr_done = 0

    def run(self, nburn=0, niter=0, do_init=False, itr0=None, stream=None):
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        i0 = self.itr_done if itr0 is None else int(itr0)
        _lib.check(self.L, self.L.cmc_batch_run(self.plan, 1 if do_init else 0, int(nburn),
                                                int(niter), i0, C.c_void_p(s.cuda_stream)))
        self.itr_done = i0 + int(niter)

    def cancel(self):
        """Stop the running batch launches (callable from another host thread
        while they run): no cluster takes a further (fit, sequence) item, a
        running one stops after its current iteration's exchange with its
        state and records written back, and every job's status becomes
        CMC_ERR_CANCELLED (its check() raises; the jobs are left at different
        iterations).  The next run() clears the cancel flags; clear_status()
        resets the status words."""
        _lib.check(self.L, self.L.cmc_batch_cancel(self.plan))

    def graph(self, nburn=0, niter=0, itr0=0):
        """Capture one chunk (memsets + one persistent launch per size class)
        as a CUDA graph; replaying it runs the chunk again (recording main
        iterations at column itr0 each time)."""
        g = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.graph(g, stream=side):
            self.run(nburn, niter, itr0=itr0, stream=side)
        return g

    def graph_schedule(self, nburn, niter, chunk=256, itr0=0):
        """Capture a whole sweep schedule as ONE CUDA graph: nburn burn-in
        iterations, then niter recorded ones (columns itr0 ..), each phase as
        launches of at most ``chunk`` iterations (so a replay can be followed
        chunk by chunk with events, and no launch runs for long).  Replaying
        the graph once runs the schedule from the jobs' current state."""
        g = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.graph(g, stream=side):
            done = 0
            while done < nburn:
                n = min(chunk, nburn - done)
                self.run(n, 0, itr0=itr0, stream=side)
                done += n
            done = 0
            while done < niter:
                n = min(chunk, niter - done)
                self.run(0, n, itr0=itr0 + done, stream=side)
                done += n
        self.itr_done = itr0 + niter
        return g

    def run_class(self, cls, nburn=0, niter=0, itr0=0, stream=None):
        """Launch size class ``cls`` alone (burn-in / recorded iterations)."""
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        _lib.check(self.L, self.L.cmc_batch_run_class(self.plan, int(cls), 0, int(nburn),
                                                      int(niter), int(itr0),
                                                      C.c_void_p(s.cuda_stream)))

    def set_class(self, cls, R, T, phasor, stream=None):
        """Give class ``cls`` the shape (R, T, phasor); raises McmcError if a
        job of the class does not fit it."""
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        _lib.check(self.L, self.L.cmc_batch_set_class(self.plan, int(cls), int(R), int(T),
                                                      int(phasor), C.c_void_p(s.cuda_stream)))

    def autotune(self, iters=2, R_values=(1, 2, 4, 8, 16, 32), T_values=(64, 128, 256),
                 verbose=False):
        """Time every feasible shape of every size class on the batch itself
        (``iters`` burn-in iterations of the class, from a saved state that is
        restored after each trial) and keep the fastest per class.  Returns
        the chosen shapes."""
        saved_fields = ("pcur", "chi2c", "flag", "ptent", "ptentn", "pstp", "n_acpt", "n_exch",
                        "n_cnt", "n_hist", "tcur", "rndst", "datm", "chi2m", "status")
        saved = [{k: j.t[k].clone() for k in saved_fields} for j in self.jobs]

        def restore():
            for j, sv in zip(self.jobs, saved):
                for k, v in sv.items():
                    j.t[k].copy_(v)

        chosen = []
        try:
            for c, cur in enumerate(self.classes()):
                best, best_t = (cur["R"], cur["T"], cur["phasor"]), float("inf")
                for R in R_values:
                    for T in T_values:
                        for ph in (1, 0, 2):
                            try:
                                self.set_class(c, R, T, ph)
                            except _lib.McmcError:
                                continue
                            times = []
                            for _ in range(2):          # the first run loads the instance
                                e0 = torch.cuda.Event(enable_timing=True)
                                e1 = torch.cuda.Event(enable_timing=True)
                                e0.record()
                                self.run_class(c, nburn=iters)
                                e1.record()
                                e1.synchronize()
                                times.append(e0.elapsed_time(e1))
                                restore()
                            if verbose:
                                print("class %d R=%d T=%d phasor=%d: %.3f ms" % (c, R, T, ph,
                                                                                times[-1]))
                            if times[-1] < best_t:
                                best_t, best = times[-1], (R, T, ph)
                self.set_class(c, *best)
                chosen.append(dict(zip(("R", "T", "phasor"), best), ms=best_t))
        finally:
            restore()
            torch.cuda.synchronize(self.device)
        self.check()
        return chosen

    def classes(self):
        out = []
        n = self.L.cmc_batch_info(self.plan, -1, None, None, None, None, None, None, None)
        for c in range(n):
            v = [C.c_int() for _ in range(6)]
            sm = C.c_size_t()
            self.L.cmc_batch_info(self.plan, c, *[C.byref(x) for x in v], C.byref(sm))
            out.append(dict(R=v[0].value, G=v[1].value, T=v[2].value, phasor=v[3].value,
                            items=v[4].value, clusters=v[5].value, smem=sm.value))
        return out

    def check(self):
        for j in self.jobs:
            j.check()

    def clear_status(self):
        """Reset every job's status word (after cancel())."""
        for j in self.jobs:
            j.clear_status()

    def __del__(self):
        plan = getattr(self, "plan", None)
        if plan is not None and plan.value:
            self.L.cmc_batch_free(plan)
            self.plan = None
