"""Launch-shape autotuner for the fused sweep.

The sweep kernel has three shape knobs: replicas per CTA R (so the cluster
size is G = nbeta/R), threads per CTA T, and the closure-phase storage (unit
phasors or phases).  The C-ABI picks a shape by a measured heuristic; this
module measures instead: it times a short chunk of the job itself under every
feasible shape (on a copy of the job's state, which it restores) and keeps the
fastest.  Results are cached per problem signature (model, sizes, GPU) in
memory and in ``_lib/autotune.json``.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import time

import torch

from . import _build, _lib

_CACHE = {}
_FILE = os.path.join(_build.LIB_DIR, "autotune.json")

R_VALUES = (1, 2, 4, 8, 16, 32)   # shapes a library lacks are skipped
T_VALUES = (64, 128, 256)

# DeviceJob tensors that a trial run modifies
_STATE = ("pcur", "chi2c", "flag", "ptent", "ptentn", "pstp", "n_acpt", "n_exch", "n_cnt",
          "n_hist", "tcur", "rndst", "pout", "tout", "chi2", "datm", "chi2m", "status",
          "inj_cur")


def _build_stamp(lib_file: str) -> str:
    """The source digest the library was built from (shapes timed on other
    kernels are not reused)."""
    try:
        with open(lib_file + ".stamp") as f:
            return f.read().strip()
    except OSError:
        return ""


def signature(job) -> str:
    j = job.job
    dev = torch.cuda.get_device_name(job.device)
    return "|".join(str(x) for x in (
        os.path.basename(job.L._name), _build_stamp(job.L._name), dev, j.nbeta, j.nseq, j.ndat,
        j.hidat[0], j.hidat[2], j.nptot, j.nprm, j.npass, j.imodel, j.nadj))


def _load_file():
    if not _CACHE and os.path.exists(_FILE):
        try:
            _CACHE.update(json.load(open(_FILE)))
        except (OSError, ValueError):
            pass


def _save_file():
    try:
        os.makedirs(os.path.dirname(_FILE), exist_ok=True)
        tmp = _FILE + ".tmp%d" % os.getpid()
        with open(tmp, "w") as f:
            json.dump(_CACHE, f, indent=1, sort_keys=True)
        os.replace(tmp, _FILE)
    except OSError:
        pass


def candidates(job):
    """Feasible (R, T, phasor) shapes for this job, with the library's view
    (clusters per wave, shared memory)."""
    L, out = job.L, []
    try:
        for R in R_VALUES:
            if job.nbeta % R or job.nbeta // R > 16:
                continue
            for T in T_VALUES:
                if T < 32 * ((R + 31) // 32):
                    continue
                for ph in (1, 0, 2):        # 2: phases in global memory (large data)
                    L.cmc_set_config(R, T, ph)
                    L.cmc_set_layout(1)
                    try:
                        cfg = job.config()
                    except _lib.McmcError:
                        continue
                    out.append(cfg)
        # the spread layout (any R up to the model's largest; models without
        # it report no shape)
        for R in range(1, 9):
            if R > job.nbeta:
                continue
            for T in T_VALUES:
                if T < 32 * ((R + 31) // 32):
                    continue
                for ph in (1, 0, 2):
                    L.cmc_set_config(R, T, ph)
                    L.cmc_set_layout(2)
                    try:
                        cfg = job.config()
                    except _lib.McmcError:
                        continue
                    out.append(cfg)
    finally:
        L.cmc_set_config(0, 0, -1)
        L.cmc_set_layout(0)
    return out


_LAYOUTS = {"cluster": 1, "spread": 2}


def _key(cfg):
    return (cfg["R"], cfg["T"], cfg["phasor"], _LAYOUTS.get(cfg.get("layout"), 1))


# a measured shape replaces the library's own pick only when it is faster
# by more than this fraction (shapes within timing noise keep the pick, so
# that repeated tunings agree)
MARGIN = 0.01


def tune(job, iters=8, repeats=2, use_cache=True, verbose=False):
    """Return the fastest shape {R, T, phasor} for ``job`` (a DeviceJob) and
    store it on the job (``job.shape``), which then applies it to every run.
    The library's own pick is kept unless a shape beats it by MARGIN."""
    _load_file()
    job.shape = None
    key = signature(job)
    if use_cache and key in _CACHE:
        job.shape = dict(_CACHE[key])
        return job.shape
    saved = {k: job.t[k].clone() for k in _STATE if k in job.t}
    itr_done = job.itr_done
    best, best_t = None, float("inf")
    try:
        own = _key(job.config())
    except _lib.McmcError:
        own = None
    own_t = float("inf")
    L = job.L
    try:
        for cfg in candidates(job):
            L.cmc_set_config(cfg["R"], cfg["T"], cfg["phasor"])
            L.cmc_set_layout(_key(cfg)[3])
            try:
                job.run(0, 0, do_init=True)          # start every trial from the same state
                job.check()
                times = []
                for _ in range(repeats):
                    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    s.record()
                    job.run(iters, 0)
                    e.record()
                    e.synchronize()
                    times.append(s.elapsed_time(e))
                job.check()
            except _lib.McmcError:
                continue
            t = min(times)
            if verbose:
                print("autotune R=%d T=%d phasor=%d layout=%s: %.3f ms" % (
                    cfg["R"], cfg["T"], cfg["phasor"], cfg.get("layout"), t))
            if _key(cfg) == own:
                own_t = t
            if t < best_t:
                best_t, best = t, {"R": cfg["R"], "T": cfg["T"], "phasor": cfg["phasor"],
                                   "layout": _key(cfg)[3]}
    finally:
        L.cmc_set_config(0, 0, -1)
        L.cmc_set_layout(0)
        for k, v in saved.items():
            job.t[k].copy_(v)
        job.itr_done = itr_done
        torch.cuda.synchronize(job.device)
    if best is None:
        raise _lib.McmcError(_lib.CMC_ERR_UNSUPPORTED, "autotune: no launch shape ran")
    if own is not None and own_t < float("inf") and best_t > (1.0 - MARGIN) * own_t:
        best = {"R": own[0], "T": own[1], "phasor": own[2], "layout": own[3]}
    _CACHE[key] = best
    _save_file()
    job.shape = dict(best)
    return job.shape
