"""Benchmark: chi^2 model evaluations per second of the MCMC-RE sweep.

Workload (default): the Sgr A* crescent + Gaussian fit, sgra_model9 on
seeded synthetic data with 2000 visibility amplitudes + 600 closure phases,
64 sequences x 32 temperatures (2048 replicas), 9 mutable parameters.  One
"step" is one sweep chunk of 500 iterations (100 burn-in + 400 main, the
1:4 ratio of the full 5000 + 20000 run) over all replicas:
500 * 9 * 2048 = 9,216,000 chi^2 evaluations, each over all 2600 data.

  value  -- device-resident inputs, the fused sweep via cmc_run (resumed
            chunk after chunk, as a long run is split);
  e2e    -- the reference-facing call mcmc_cuda (host buffers, H2D + D2H
            copies inside the timed region) per step;
  cpu_baseline -- the CPU port of the reference's sweep on a bounded sample,
            all host threads;
  roofline -- the sweep kernel's achieved FP32 rate from the algorithmic
            FLOP count per evaluation against a measured FP32 (SGEMM) peak;
  configs -- the other workloads, each measured in the same run on the same
            GPU: the 20000 + 6000 Sgr A* fit, 1024 batched fits (persistent
            work-list launches from a CUDA graph) beside one cmc_run per fit,
            the Rosenbrock and nonlinear-system plugin models, and the
            effective samples per second of the fused (Fisher-adapted,
            graph-captured) schedule against the plain per-fit schedule on
            the 20000 + 6000 data at matched posterior accuracy.

Run: python bench.py [--gpus N --steps K --warmup W] [--impl reference]
     [--no-extras] [--workload sgra|batch|ess|ess-batch|rosenbrock|nlsys]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Algorithmic work per chi^2 evaluation of sgra_model9 (frozen op-count
# convention: FADD/FMUL = 1, FFMA = 2 FLOP; Bessel J0/J1 as degree-5/5
# rationals): 180 FLOP per amplitude term, 25 FLOP per closure term.
FLOP_PER_AMP, FLOP_PER_CPH = 180.0, 25.0
L2_BYTES = 129 * 1024 * 1024

# ESS comparison on the 20000 + 6000 data: (burn-in, recorded) iterations of
# the plain per-fit arm, the fused arm and the long fused run both are
# compared with.  The plain arm gets the budget it needs to match the long
# run's posterior within 3 Monte-Carlo standard errors.
ESS_PLAIN = (4000, 8000)
ESS_FUSED = (1000, 2000)
ESS_LONG = (1000, 8000)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="mine", choices=["mine", "reference"])
    ap.add_argument("--burn-per-step", type=int, default=100)
    ap.add_argument("--main-per-step", type=int, default=400)
    ap.add_argument("--nvis", type=int, default=2000)
    ap.add_argument("--ncph", type=int, default=600)
    ap.add_argument("--nseq", type=int, default=64)
    ap.add_argument("--nbeta", type=int, default=32)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="use the library's heuristic shape")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the other workloads' records in the default line")
    ap.add_argument("--cpu-iters", type=int, default=20,
                    help="iterations of the CPU baseline sample")
    ap.add_argument("--workload", default="sgra",
                    choices=["sgra", "batch", "ess", "ess-batch", "rosenbrock", "nlsys"],
                    help="sgra: one 64x32 Sgr A* fit; batch: many independent fits; "
                         "ess: ESS/sec of Fisher block proposals vs the reference's proposals; "
                         "ess-batch: the same over many fits, batched vs one fit per launch; "
                         "rosenbrock / nlsys: the plugin-model configurations, one full run "
                         "per step")
    ap.add_argument("--nfits", type=int, default=1024)
    ap.add_argument("--ess-nseq", type=int, default=32)
    ap.add_argument("--ess-burn", type=int, default=2000)
    ap.add_argument("--ess-iter", type=int, default=4000)
    return ap.parse_args()


def dist_setup(args):
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64,
                     device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload(args, rank=0):
    from cuda_mcmc_gb300 import synth
    return synth.sgra(nvis=args.nvis, ncph=args.ncph, seed=3, nseq=args.nseq, nbeta=args.nbeta,
                      nburn=args.burn_per_step, niter=args.main_per_step)


def evals_per_step(w, args):
    return (args.burn_per_step + args.main_per_step) * w.nprm * w.nbeta * w.nseq


# DRAM bytes of one sweep launch of the 2000 vis + 600 closure, 64 x 32 workload:
# ncu dram__bytes_read.sum + dram__bytes_write.sum of a 16-iteration launch of
# the library's shape (spread layout, R=7, T=256; 4 burn-in + 12 recorded;
# 26.7 + 28.0 MB) = a fixed part (state, model data per CTA, final datm /
# chi2m rows) plus the records of each main iteration (pout + tout + chi2,
# 9*32*64*4 + 32*64*4 + 64*4 bytes).
TRAFFIC_SOURCE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of a 16-iteration launch "
                  "(54.7 MB) scaled to this launch: fixed part + the records of each main "
                  "iteration; only for the 2000 vis + 600 closure 64 x 32 workload")
_TRAFFIC_CAPTURE = 54.7e6
_TRAFFIC_REC_PER_ITER = 9 * 32 * 64 * 4 + 32 * 64 * 4 + 64 * 4


def sweep_traffic(w, args):
    """DRAM bytes per sweep launch (the timed step is one launch), or None when
    the workload is not the profiled one."""
    if (w.nvis, w.ndat - w.nvis, w.nseq, w.nbeta) != (2000, 600, 64, 32):
        return None
    fixed = _TRAFFIC_CAPTURE - 12 * _TRAFFIC_REC_PER_ITER
    return fixed + args.main_per_step * _TRAFFIC_REC_PER_ITER


def flop_per_eval(w):
    return w.nvis * FLOP_PER_AMP + (w.ndat - w.nvis) * FLOP_PER_CPH


class Clocks:
    """nvidia-smi samples (200 ms) during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                self.out = ""

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


def fp32_peak_tflops():
    """Measured FP32 SIMT peak: cuBLAS SGEMM (TF32 off), best of 5."""
    import torch
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    n = 8192
    a = torch.randn(n, n, device="cuda")
    b = torch.randn(n, n, device="cuda")
    torch.matmul(a, b)
    best = 1e30
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        torch.matmul(a, b)
        e.record()
        e.synchronize()
        best = min(best, s.elapsed_time(e) / 1e3)
    torch.backends.cuda.matmul.allow_tf32 = prev
    del a, b
    return 2.0 * n ** 3 / best / 1e12


# ---------------------------------------------------------------------------
# CPU: the oracle port of the sweep, parallel over sequences
# ---------------------------------------------------------------------------

class CpuSweep:
    """The CPU port of the reference's sweep (oracle.c's or_sweep) on all
    w.nseq sequences, split over `threads` host threads: sequences are
    independent (the replica exchange stays inside a sequence), so each
    thread owns a group of them; ctypes releases the GIL, so the threads run
    in parallel.  The Sgr A* model (sgra_model9) is evaluated in float32 with
    float Bessel functions and the chi^2 row summed serially in float, as the
    reference's kernels compute it (oracle.c, OR_ARITH_F32); the plugin models
    in FP64.  On one core of the build host this port ran at 1.43e3 evals/s
    against 0.95e3 for the reference's own kernels compiled for the CPU
    (oracle/_ref/libref_sgra.so, 2000 + 600 data), so it is the faster of
    the two baselines."""

    ARITH = "float32 (as the reference's kernels)"

    def __init__(self, w, threads, max_iters, seed=1):
        import oracle
        self.oracle = oracle
        self.w = w
        self.pb = oracle.Problem(w.model, w.coor, w.dat, w.std2r, w.icoor, w.idat, w.nptot,
                                 w.imodel, w.npass, arith=1)
        self.jobs = []
        for i, g in enumerate([list(range(i, w.nseq, threads))
                               for i in range(min(threads, w.nseq))]):
            ns = len(g)
            st = oracle.new_state(w.pdescr, w.pmint, w.pmaxt, w.beta(), ns, 1, ptotal=w.ptotal,
                                  ndat=w.ndat)
            rs = oracle.make_streams(ns * w.nbeta,
                                     w.nprm * (3 * max_iters + 2) + 3 * w.nbeta * max_iters + 64,
                                     w.nprm * max_iters + 8, seed + i)
            self.jobs.append((st, rs, ns))
        self._parallel(1, 0)                      # init_pcur + first chi^2

    def _parallel(self, do_init, iters):
        ths = [threading.Thread(target=self.oracle.sweep,
                                args=(self.pb, st, rs, do_init, iters, 0))
               for (st, rs, _) in self.jobs]
        for t in ths:
            t.start()
        for t in ths:
            t.join()

    def step(self, iters):
        t0 = time.perf_counter()
        self._parallel(0, iters)
        dt = time.perf_counter() - t0
        return iters * self.w.nprm * self.w.nbeta * self.w.nseq, dt


def run_reference(args, rank, world):
    if rank != 0:
        return
    w = workload(args)
    threads = os.cpu_count() or 1
    cpu = CpuSweep(w, threads, args.warmup + args.steps, seed=100)
    rates = []
    for i in range(args.warmup + args.steps):
        ev, dt = cpu.step(1)
        if i >= args.warmup:
            rates.append((ev, dt))
    tot_ev = sum(x[0] for x in rates)
    tot_t = sum(x[1] for x in rates)
    val = tot_ev / tot_t
    line = {
        "impl": "reference", "metric": "chi2 model evals/sec", "value": val,
        "unit": "chi2 evals/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * tot_t / len(rates), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "sgra9 %dvis+%dcph, %dx%d replicas" % (
            w.nvis, w.ndat - w.nvis, w.nseq, w.nbeta),
            "step": "1 MCMC-RE iteration (9 proposals + exchange) of all replicas",
            "parallelism": "replicas only"},
        "cpu_baseline": {"value": val, "unit": "chi2 evals/s", "cores": threads, "kind": "port",
                         "sample": "%d iterations x %d replicas, CPU port of the reference's "
                                   "sweep (float32 model as its kernels), sequences split over "
                                   "%d threads" % (args.steps, w.nseq * w.nbeta, threads)},
        "e2e": {"value": val, "unit": "chi2 evals/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    line["ref_gpu"] = ref_gpu_rate(w)
    print(json.dumps(line))


def ref_gpu_rate(w, warm=2, iters=10):
    """The reference's own CUDA build (src/gpu_mcmc.cu with the Sgr A*
    model.cuh, compiled for sm_103a in the build container) on this GPU:
    run_mcmc's kernel sequence, launched per iteration as the reference does
    (gen_proposal, calc_chi2_terms x npass, spmp_mcmc per mutable parameter,
    replica_exchange), timed with CUDA events over ``iters`` main iterations
    after init and ``warm`` untimed ones."""
    try:
        import torch
        if not torch.cuda.is_available():
            return {"unavailable": "no CUDA device"}
        from oracle import ref_gpu
        if not ref_gpu.available("sgra"):
            return {"unavailable": "the reference's CUDA build (oracle/_ref/ref_gpu_sgra.cubin) "
                                   "was not built in the build container"}
        from cuda_mcmc_gb300.device import sampler_defaults
        st = sampler_defaults(w.pdescr, w.pmint, w.pmaxt, w.nbeta, w.nseq, ptotal=w.ptotal,
                              pstp=w.pstp0)
        job = ref_gpu.RefGpuJob("sgra", w.coor, w.dat, w.std2r, w.icoor, w.idat, w.beta(), st,
                                w.nseq, iters, 1234, imodel=w.imodel, npass=w.npass)
        job.init()
        for i in range(warm):
            job.iteration(False, i % iters)
        stream = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        n0 = job.launches
        e0.record(stream)
        for i in range(iters):
            job.iteration(False, i)
        e1.record(stream)
        torch.cuda.synchronize()
        dt = e0.elapsed_time(e1) / 1e3
        ev = iters * w.nprm * w.nbeta * w.nseq
        return {"value": ev / dt, "unit": "chi2 evals/s", "s_per_iteration": dt / iters,
                "launches_per_iteration": (job.launches - n0) / iters,
                "sample": "%d main iterations x %d replicas after init + %d" % (
                    iters, w.nbeta * w.nseq, warm),
                "form": "the reference's gpu_mcmc.cu kernels unchanged (nvcc -arch=sm_103a), "
                        "run_mcmc's launch sequence and shapes"}
    except Exception as e:      # a missing piece is reported, not fatal to the CPU line
        return {"unavailable": "%s: %s" % (type(e).__name__, e)}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def e2e_rate(w, args, steps, warmup):
    """mcmc_cuda with host numpy buffers, one full call per step."""
    import torch
    from cuda_mcmc_gb300 import mcmc_interf
    from cuda_mcmc_gb300.device import sampler_defaults
    mcmc_interf.use_model("sgra")
    nrep, nprm = w.nbeta * w.nseq, w.nprm
    nb, ni = args.burn_per_step, args.main_per_step
    s0 = sampler_defaults(w.pdescr, w.pmint, w.pmaxt, w.nbeta, w.nseq)
    beta = w.beta()

    # host buffers in pinned (page-locked) memory, allocated once: every step
    # copies its inputs from them and its results back into them
    tdt = {np.dtype(np.float32): torch.float32, np.dtype(np.int32): torch.int32,
           np.dtype(np.uint8): torch.uint8}

    def pinned(shape, dtype):
        return torch.empty(shape, dtype=tdt[np.dtype(dtype)], pin_memory=True).numpy()

    sp = {k: pinned(v.shape, v.dtype) for k, v in s0.items()}
    pout = pinned((nprm, w.nbeta, w.nseq, ni), np.float32)
    tout = pinned((w.nbeta, w.nseq, ni), np.int32)
    chi2 = pinned((w.nseq, ni), np.float32)
    datm = pinned((nrep * (w.ndat + w.nvis),), np.float32)
    chi2m = pinned((w.nbeta, w.nseq, w.ndat), np.float32)
    rndst = pinned((w.nbeta, w.nseq, 48), np.uint8)

    def call(seed):
        for k, v in s0.items():        # the step's starting state
            sp[k][...] = v
        s = sp
        mcmc_interf.mcmcuda(w.coor, w.dat, w.std2r, w.icoor, w.idat, datm, chi2m, s["pdescr"],
                            s["ivar"], s["invar"], s["ptotal"], s["pmint"], s["pmaxt"], pout,
                            tout, chi2, s["chi2c"], s["tcur"], s["flag"], s["n_acpt"],
                            s["n_exch"], s["n_cnt"], s["n_hist"], beta, s["pstp"], s["ptent"],
                            s["ptentn"], s["pcur"], rndst, np.uint64(seed), w.imodel,
                            w.coor.size, w.ndat, w.icoor.size, w.idat.size, datm.size, w.nptot,
                            nprm, 100, w.npass, w.nbeta, w.nseq, nb, ni)
        return s, pout, tout, chi2, datm, chi2m, rndst

    for i in range(warmup):
        call(1000 + i)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(steps):
        out = call(2000 + i)
    dt = time.perf_counter() - t0
    s = out[0]
    h2d = sum(a.nbytes for a in (w.coor, w.dat, w.std2r, w.icoor, w.idat, s["pdescr"], s["ivar"],
                                 s["invar"], s["pmint"], s["pmaxt"], s["tcur"], s["flag"],
                                 s["chi2c"], s["n_acpt"], s["n_exch"], s["n_cnt"], s["n_hist"],
                                 beta, s["pstp"], s["ptent"], s["ptentn"], s["pcur"],
                                 out[6]))   # rndst goes in as well (src/mcmcjob.cu:724)
    d2h = sum(a.nbytes for a in out[1:]) + sum(
        s[k].nbytes for k in ("tcur", "n_acpt", "n_cnt", "n_exch", "n_hist", "pstp", "ptent",
                              "ptentn", "pcur", "flag", "chi2c"))
    return evals_per_step(w, args) * steps / dt, dt / steps, h2d, d2h


def run_mine(args, rank, world, local):
    import torch
    from cuda_mcmc_gb300 import _lib
    from cuda_mcmc_gb300.device import DeviceJob
    _lib.load("sgra")
    w = workload(args, rank)
    if world > 1:
        # one run of world*nseq sequences, rank r holding sequences
        # [r*nseq, (r+1)*nseq): the shards together walk the unsharded chains
        from cuda_mcmc_gb300 import synth
        wt = synth.sgra(nvis=args.nvis, ncph=args.ncph, seed=3, nseq=args.nseq * world,
                        nbeta=args.nbeta, nburn=args.burn_per_step, niter=args.main_per_step)
        job = DeviceJob.from_workload(wt, niter_total=args.main_per_step, seed=1234,
                                      seqs=(rank * args.nseq, (rank + 1) * args.nseq))
    else:
        job = DeviceJob.from_workload(w, niter_total=args.main_per_step, seed=1234)
    if not args.no_tune:
        job.autotune()
    cfg = job.config()
    stream = torch.cuda.current_stream()
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    job.run(0, 0, do_init=True)
    job.check()
    for _ in range(args.warmup):
        job.run(args.burn_per_step, args.main_per_step, itr0=0)
        flush.zero_()
    job.check()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    with Clocks(local) as clk:
        barrier(world)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(args.steps):
            evs[i][0].record(stream)
            job.run(args.burn_per_step, args.main_per_step, itr0=0, stream=stream)
            evs[i][1].record(stream)
            flush.zero_()
        torch.cuda.synchronize()
        barrier(world)
        dt = time.perf_counter() - t0
    job.check()
    dt = max_over_ranks(dt, world)
    kern_s = [a.elapsed_time(b) / 1e3 for a, b in evs]
    n_ev = evals_per_step(w, args)
    value = n_ev * args.steps * world / dt
    if rank != 0:
        return
    clocks = clk.summary()
    avg_launch = float(np.mean(kern_s))
    peak = fp32_peak_tflops()
    achieved = n_ev * flop_per_eval(w) / avg_launch / 1e12
    line = {
        "metric": "chi2 model evals/sec", "value": value, "unit": "chi2 evals/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {
            "workload": "sgra9 %dvis+%dcph, %dx%d replicas" % (w.nvis, w.ndat - w.nvis, w.nseq,
                                                                w.nbeta),
            "step": "%d burn-in + %d main iterations (9 proposals + exchange each) of all "
                    "replicas = %d chi2 evals" % (args.burn_per_step, args.main_per_step, n_ev),
            "parallelism": "replicas only: sequences sharded across ranks (seq_offset/"
                           "nseq_total), no collective in the sweep",
            "l2": "2x L2 buffer written between timed steps",
            "launch": cfg},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": sweep_traffic(w, args),
                     "traffic_source": TRAFFIC_SOURCE,
                     "peak_source": "measured cuBLAS SGEMM (TF32 off) in this run",
                     "flop_per_eval": flop_per_eval(w)},
        "clocks": clocks,
        # per step (one cmc_run): the packing kernels (points, closure-corner
        # marks when there are closures, rank, scatter) and the sweep kernel
        "gpu_launches": args.steps * (4 + (1 if w.ndat > w.nvis else 0)),
    }
    if not args.no_e2e and world == 1:
        e2e, e2e_step, h2d, d2h = e2e_rate(w, args, steps=args.steps, warmup=1)
        line["e2e"] = {"value": e2e, "unit": "chi2 evals/s", "h2d_bytes_per_step": h2d,
                       "d2h_bytes_per_step": d2h, "s_per_step": e2e_step,
                       "call": "mcmc_cuda (host buffers, one call per step incl. init)"}
    if not args.no_cpu and world == 1:
        line["cpu_baseline"] = cpu_baseline(w, args.cpu_iters)
    if not args.no_extras and world == 1:
        line["configs"] = extras(args, local, peak)
    print(json.dumps(line))


def cpu_baseline(w, iters):
    """The CPU port of the reference's sweep on the host cores: ``iters``
    iterations of all replicas, sequences split over every host thread, and
    the same on one core (4 sequences)."""
    import copy
    threads = os.cpu_count() or 1
    cpu = CpuSweep(w, threads, iters)
    cev, cdt = cpu.step(iters)
    w1 = copy.copy(w)
    w1.nseq = 4
    n1 = max(1, iters // 4)
    c1, d1 = CpuSweep(w1, 1, n1).step(n1)
    return {"value": cev / cdt, "unit": "chi2 evals/s", "cores": threads, "kind": "port",
            "sample": "%d iterations x %d replicas (%d evals, %.1f s), CPU port of the sweep "
                      "with %s model arithmetic, sequences over %d threads" % (
                          iters, w.nseq * w.nbeta, cev, cdt, CpuSweep.ARITH, threads),
            "one_core": {"value": c1 / d1, "cores": 1,
                         "sample": "%d iterations x %d replicas (%d evals)" % (
                             n1, w1.nseq * w1.nbeta, c1)}}


def extras(args, local, peak):
    """The other workloads of the benchmark definition, measured in the same
    run on the same GPU (device-resident inputs, CUDA-event or synchronised
    wall timing, clocks sampled per record)."""
    import torch
    from cuda_mcmc_gb300 import synth
    from cuda_mcmc_gb300.device import DeviceJob
    out = {}
    # config 4: the 20000 + 6000 Sgr A* fit, 64 x 32, chunks of 10 + 40
    w4 = synth.sgra(nvis=20000, ncph=6000, seed=4, nseq=64, nbeta=32)
    job = DeviceJob.from_workload(w4, niter_total=40, seed=4321)
    nb4, ni4, st4 = 10, 40, 5
    job.run(0, 0, do_init=True)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        job.run(nb4, ni4, itr0=0)
    job.check()
    stream = torch.cuda.current_stream()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(st4)]
    with Clocks(local) as clk:
        torch.cuda.synchronize()
        for i in range(st4):
            evs[i][0].record(stream)
            job.run(nb4, ni4, itr0=0, stream=stream)
            evs[i][1].record(stream)
            flush.zero_()
        torch.cuda.synchronize()
    job.check()
    ks = float(np.mean([a.elapsed_time(b) / 1e3 for a, b in evs]))
    n4 = (nb4 + ni4) * w4.nprm * w4.nbeta * w4.nseq
    a4 = n4 * flop_per_eval(w4) / ks / 1e12
    out["config4_sgra9_20000vis_64x32"] = {
        "value": n4 / ks, "unit": "chi2 evals/s", "steps": st4, "warmup": args.warmup,
        "ms_per_step": 1e3 * ks,
        "step": "%d burn-in + %d main iterations of all replicas = %d chi2 evals" % (nb4, ni4, n4),
        "launch": job.config(), "l2": "2x L2 buffer written between timed steps",
        "roofline": {"bound": "fp32", "achieved": a4, "peak": peak, "unit": "TFLOP/s",
                     "frac": a4 / peak, "flop_per_eval": flop_per_eval(w4)},
        "clocks": clk.summary(), "gpu_launches": st4 * 5}
    del job, flush
    torch.cuda.empty_cache()
    # config 5: 1024 batched fits
    out["config5_batch_1024fits"] = measure_batch(args.nfits, 3, args.warmup, False, local,
                                                  nb=2, ni=8)
    torch.cuda.empty_cache()
    # configs 1 and 2: the plugin models
    out["config1_rosenbrock4_16x32"] = measure_plugin("rosenbrock", 2, 1, local, cpu=False)
    out["config2_nlsys8_64x32"] = measure_plugin("nlsys", 2, 1, local, cpu=False)
    # ESS/sec, fused vs plain, on the config-4 data at matched accuracy
    out["ess_config4_data"] = measure_ess(20000, 6000, 4, args.ess_nseq, 32, ESS_PLAIN, ESS_FUSED,
                                          ESS_LONG, False, local)
    return out


def measure_batch(nfits, steps, warmup, tune, local=0, rank=0, world=1, nb=1, ni=3):
    """Many independent Sgr A* fits (nvis ~ logU(500, 50000), ncph = 0.3 nvis,
    16 x 16 replicas each): persistent work-list launches replayed from a CUDA
    graph, against a loop of one plain cmc_run launch per fit.  A step is nb
    burn-in + ni main iterations of every fit."""
    import torch
    from cuda_mcmc_gb300 import synth
    from cuda_mcmc_gb300.device import BatchJob, DeviceJob
    t_setup = time.perf_counter()
    fits = synth.sgra_batch(nfits=nfits, seed=5 + rank, nseq=16, nbeta=16, nburn=nb, niter=ni)
    jobs = [DeviceJob.from_workload(w, niter_total=ni, seed=77 + i) for i, w in enumerate(fits)]
    batch = BatchJob(jobs)
    batch.run(0, 0, do_init=True)
    batch.check()
    heuristic = batch.classes()
    tune_s = None
    if tune:
        t0 = time.perf_counter()
        batch.autotune(iters=1)
        tune_s = time.perf_counter() - t0
    g = batch.graph(nb, ni, itr0=0)
    for _ in range(warmup):
        g.replay()
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t_setup
    terms = sum(w.ndat for w in fits)
    evals = (nb + ni) * sum(w.nprm * w.nbeta * w.nseq for w in fits)
    with Clocks(local) as clk:
        barrier(world)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            g.replay()
        torch.cuda.synchronize()
        barrier(world)
        dt = time.perf_counter() - t0
    batch.check()
    dt = max_over_ranks(dt, world)
    # plain: one cmc_run per fit per chunk, heuristic shape, no graph
    for j in jobs[: min(8, len(jobs))]:
        j.run(nb, ni, itr0=0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for j in jobs:
        j.run(nb, ni, itr0=0)
    torch.cuda.synchronize()
    plain_dt = time.perf_counter() - t0
    for j in jobs:
        j.check()
    fl = sum(w.nprm * w.nbeta * w.nseq * flop_per_eval(w) for w in fits) * (nb + ni)
    return {
        "value": evals * steps * world / dt, "unit": "chi2 evals/s", "steps": steps,
        "warmup": warmup, "ms_per_step": 1e3 * dt / steps,
        "workload": "%d independent sgra9 fits, nvis logU(500,50000), ncph 0.3 nvis, 16x16 "
                    "replicas each (%d data in total)" % (len(fits), terms),
        "step": "%d burn-in + %d main iterations of every fit (%d chi2 evals), one CUDA graph "
                "replay" % (nb, ni, evals),
        "classes": batch.classes(), "heuristic_classes": heuristic, "autotune_s": tune_s,
        "l2": "inputs larger than L2 in total",
        "achieved_tflops": fl * steps / dt / 1e12,
        "plain_per_fit_loop": {"value": evals / plain_dt, "unit": "chi2 evals/s",
                               "s_per_step": plain_dt,
                               "form": "one cmc_run per fit, heuristic shape, no graph"},
        "speedup_vs_plain_loop": (evals * steps / dt) / (evals / plain_dt),
        "per_fit_ms_per_iteration": 1e3 * dt / steps / (nb + ni) / len(fits),
        "setup_s": setup_s, "clocks": clk.summary(),
        "gpu_launches": steps * len(batch.classes()),
    }


def run_batch(args, rank, world, local):
    r = measure_batch(args.nfits, args.steps, args.warmup, not args.no_tune, local, rank, world)
    if rank != 0:
        return
    peak = fp32_peak_tflops()
    line = {
        "metric": "chi2 model evals/sec", "value": r["value"], "unit": "chi2 evals/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": r["workload"], "step": r["step"], "parallelism": "replicas only",
                   "classes": r["classes"], "heuristic_classes": r["heuristic_classes"],
                   "autotune_s": r["autotune_s"], "l2": r["l2"]},
        "roofline": {"bound": "fp32", "achieved": r["achieved_tflops"], "peak": peak,
                     "unit": "TFLOP/s", "frac": r["achieved_tflops"] / peak,
                     "traffic": None, "peak_source": "measured cuBLAS SGEMM (TF32 off)"},
        "plain_per_fit_loop": r["plain_per_fit_loop"],
        "per_fit_ms_per_iteration": r["per_fit_ms_per_iteration"],
        "clocks": r["clocks"], "gpu_launches": r["gpu_launches"],
    }
    print(json.dumps(line))


def measure_ess(nvis, ncph, data_seed, nseq, nbeta, plain_budget, fused_budget, long_budget,
                tune, local=0):
    """Effective samples per second at the T = 1 slot (min over parameters,
    pooled sequences, Geyer initial monotone sequence; wall time of the whole
    schedule, burn-in and Fisher set-up included): the plain per-fit form
    (the reference's one-parameter proposals, run_mcmc's schedule) against the
    fused form (fit.run_fisher: a quarter of the burn-in with the reference's
    proposals, L-BFGS polish of the best replica on the CUDA adjoint, Fisher
    information there, restart around it, block proposals; the rest of the
    schedule captured as one CUDA graph).  Posterior accuracy is matched as
    the benchmark definition states: both arms' posterior means within 3
    Monte-Carlo standard errors of a long fused run (other seed), and their
    68 % widths compared with it.  Budgets are (burn-in, recorded)
    iterations; the plain arm gets as many as it needs to pass."""
    import torch
    from cuda_mcmc_gb300 import fit, synth
    from cuda_mcmc_gb300.device import DeviceJob
    from cuda_mcmc_gb300.ess import ess_per_param
    from cuda_mcmc_gb300.grad import SgraChi2
    w = synth.sgra(nvis=nvis, ncph=ncph, seed=data_seed, nseq=nseq, nbeta=nbeta)
    obj = SgraChi2.from_workload(w)

    def one(kind, seed, nburn, niter):
        job = DeviceJob.from_workload(w, niter_total=niter, seed=seed)
        if tune:
            job.autotune()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if kind == "plain":
            fit.run_plain(job, nburn, niter)
        else:
            fit.run_fisher(job, obj, nburn, niter, graph=True)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        job.check()
        return dt, job.t["pout"].cpu().numpy()

    one("plain", 5, 20, 20)            # warm-up: library load, autotune cache, graph path
    one("fisher", 5, 20, 20)
    with Clocks(local) as clk:
        tp, pp = one("plain", 11, *plain_budget)
        tf, pf = one("fisher", 11, *fused_budget)
    _, pl = one("fisher", 99, *long_budget)
    sp, sf, sl = (fit.posterior_summary(x) for x in (pp, pf, pl))
    ess_p, ess_f = ess_per_param(pp), ess_per_param(pf)
    zp = np.abs(sp["mean"] - sl["mean"]) / np.sqrt(sp["mcse"] ** 2 + sl["mcse"] ** 2)
    zf = np.abs(sf["mean"] - sl["mean"]) / np.sqrt(sf["mcse"] ** 2 + sl["mcse"] ** 2)
    q = lambda x: np.percentile(x[:, 0], [16, 84], axis=(1, 2)).T    # 68 % interval per param
    qp, qf, ql = q(pp), q(pf), q(pl)
    wp = (qp[:, 1] - qp[:, 0]) / (ql[:, 1] - ql[:, 0])
    wf = (qf[:, 1] - qf[:, 0]) / (ql[:, 1] - ql[:, 0])
    vp, vf = float(ess_p.min() / tp), float(ess_f.min() / tf)
    return {
        "workload": "sgra9 %dvis+%dcph (data seed %d), %dx%d replicas" % (
            w.nvis, w.ndat - w.nvis, data_seed, nseq, nbeta),
        "metric": "ESS/sec (min over parameters, T=1 slot, pooled sequences)",
        "unit": "ESS/s",
        "plain": {"value": vp, "s": tp, "budget": "%d burn-in + %d recorded" % plain_budget,
                  "ess": ess_p.tolist(),
                  "form": "the reference's one-parameter proposals and schedule, one fit"},
        "fused": {"value": vf, "s": tf, "budget": "%d burn-in + %d recorded" % fused_budget,
                  "ess": ess_f.tolist(),
                  "form": "Fisher schedule (adjoint polish, Gauss-Newton Fisher, restart, "
                          "block proposals), post-setup schedule as one CUDA graph"},
        "speedup": vf / vp,
        "accuracy": {"z_mean_plain_vs_long": zp.tolist(), "z_mean_fused_vs_long": zf.tolist(),
                     "z_max_plain": float(zp.max()), "z_max_fused": float(zf.max()),
                     "width68_ratio_plain": wp.tolist(), "width68_ratio_fused": wf.tolist(),
                     "matched": bool(zp.max() <= 3.0 and zf.max() <= 3.0),
                     "criterion": "|mean - long mean| <= 3 MC s.e. for every parameter, both "
                                  "arms",
                     "long_run": "fused schedule, %d burn-in + %d recorded, seed 99" % long_budget},
        "clocks": clk.summary(),
    }


def run_ess(args, rank, world, local):
    r = measure_ess(args.nvis, args.ncph, 3, args.nseq // 2, args.nbeta,
                    (args.ess_burn, args.ess_iter), (args.ess_burn, args.ess_iter),
                    (args.ess_burn, 4 * args.ess_iter), not args.no_tune, local)
    if rank != 0:
        return
    line = {
        "metric": r["metric"], "value": r["fused"]["value"], "unit": "ESS/s", "n_gpus": world,
        "steps": 1, "warmup": 1, "ms_per_step": 1e3 * r["fused"]["s"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": {"workload": r["workload"]},
        "plain": r["plain"], "fisher": r["fused"], "speedup": r["speedup"],
        "accuracy": r["accuracy"], "clocks": r["clocks"],
    }
    print(json.dumps(line))


def run_ess_batch(args, rank, world, local):
    """ESS per second over many independent fits: the plain per-fit form (one
    cmc_run per fit, the reference's proposals) against the fused form (all
    fits in persistent work-list launches; after a quarter of the burn-in,
    polish + Fisher information + restart + block proposals, and the rest of
    the sweep replayed as one captured CUDA graph), same fits, replicas and
    iteration budget."""
    import torch
    from cuda_mcmc_gb300 import fit, synth
    from cuda_mcmc_gb300.device import BatchJob, DeviceJob
    from cuda_mcmc_gb300.grad import SgraChi2
    nb, ni = args.ess_burn, args.ess_iter
    fits = synth.sgra_batch(nfits=args.nfits, seed=5 + rank, nseq=16, nbeta=16,
                            nvis_min=500, nvis_max=20000)
    objs = [SgraChi2.from_workload(w) for w in fits]

    def jobs_for(seed):
        return [DeviceJob.from_workload(w, niter_total=ni, seed=seed + i) for i, w in enumerate(fits)]

    def plain(jobs):
        for j in jobs:
            j.run(nb, 0, do_init=True)
        for j in jobs:
            j.run(0, ni, itr0=0)

    def fused(jobs):
        n1 = nb // 4
        b = BatchJob(jobs)
        b.run(n1, 0, do_init=True)
        torch.cuda.synchronize()
        for j, o in zip(jobs, objs):
            fit.fisher_setup(j, o)
        b = BatchJob(jobs)            # descriptors now carry the block proposals
        g = b.graph_schedule(nb - n1, ni, chunk=250)   # the rest of the sweep: one graph
        g.replay()

    def timed(fn, jobs):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn(jobs)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        for j in jobs:
            j.check()
        return dt, [fit.posterior_summary(j.t["pout"].cpu().numpy()) for j in jobs]

    saved = (nb, ni)
    nb, ni = 10, 10                   # warm-up: library loads, allocator
    timed(plain, jobs_for(1))
    timed(fused, jobs_for(1))
    nb, ni = saved
    with Clocks(local) as clk:
        tp, ep = timed(plain, jobs_for(100))
        tf, ef = timed(fused, jobs_for(100))
    # reference posteriors: the fused schedule with 4x the recorded iterations
    ni = 4 * ni
    _, el = timed(fused, jobs_for(500))
    ni = saved[1]
    if rank != 0:
        return

    def zmax(x, y):
        return [float(np.max(np.abs(a["mean"] - b["mean"]) / np.sqrt(a["mcse"] ** 2 + b["mcse"] ** 2)))
                for a, b in zip(x, y)]

    def sdr(x, y):
        return [float(np.max(np.abs(np.log(a["sd"] / b["sd"])))) for a, b in zip(x, y)]

    acc = {"z_mean_max_plain_vs_long": zmax(ep, el), "z_mean_max_fused_vs_long": zmax(ef, el),
           "abs_log_sd_ratio_max_plain_vs_long": sdr(ep, el),
           "abs_log_sd_ratio_max_fused_vs_long": sdr(ef, el),
           "long_run": "fused schedule, %d recorded iterations, other seeds" % (4 * ni)}
    ep = [float(x["ess"].min()) for x in ep]
    ef = [float(x["ess"].min()) for x in ef]
    vp, vf = float(np.sum(ep) / tp), float(np.sum(ef) / tf)
    line = {
        "metric": "ESS/sec over fits (sum over fits of min-over-parameter ESS, T=1 slot)",
        "value": vf, "unit": "ESS/s", "n_gpus": world, "steps": 1, "warmup": 1,
        "ms_per_step": 1e3 * tf, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "%d independent sgra9 fits, nvis logU(500,20000), ncph 0.3 nvis, "
                               "16x16 replicas each" % len(fits),
                   "budget": "%d burn-in + %d recorded iterations" % (nb, ni)},
        "plain_per_fit": {"value": vp, "s": tp, "min_ess_per_fit": [float(x) for x in ep]},
        "fused": {"value": vf, "s": tf, "min_ess_per_fit": [float(x) for x in ef]},
        "speedup": vf / vp,
        "accuracy": acc,
        "clocks": clk.summary(),
    }
    print(json.dumps(line))


def measure_plugin(name, steps, warmup, local=0, rank=0, world=1, cpu=True):
    """The plugin-model configurations (Rosenbrock N=4: 16 x 32, 1000 + 5000
    iterations; the 8-unknown nonlinear system: 64 x 32, 2000 + 10000), a step
    being one complete run (init + burn-in + recorded iterations) of the
    config, beside the CPU port of the same sweep on the host cores."""
    import torch
    from cuda_mcmc_gb300 import synth
    from cuda_mcmc_gb300.device import DeviceJob
    w = synth.rosenbrock() if name == "rosenbrock" else synth.nlsys()
    job = DeviceJob.from_workload(w, niter_total=w.niter, seed=1234 + rank)
    evals = (w.nburn + w.niter) * w.nprm * w.nbeta * w.nseq
    for _ in range(warmup):
        job.run(w.nburn, w.niter, do_init=True, itr0=0)
    job.check()
    stream = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        barrier(world)
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(steps):
            job.run(w.nburn, w.niter, do_init=True, itr0=0)
        ev1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
    job.check()
    dt = max_over_ranks(ev0.elapsed_time(ev1) / 1e3, world)
    out = {"value": evals * steps * world / dt, "unit": "chi2 evals/s", "steps": steps,
           "warmup": warmup, "ms_per_step": 1e3 * dt / steps,
           "workload": "%s, %dx%d replicas, %d + %d iterations" % (
               w.name, w.nseq, w.nbeta, w.nburn, w.niter),
           "launch": job.config(), "step": "one complete run (%d chi2 evals)" % evals,
           "bound": "latency (ndat = %d terms per evaluation)" % w.ndat,
           "clocks": clk.summary(), "gpu_launches": steps}
    if cpu and rank == 0:
        threads = os.cpu_count() or 1
        cev, cdt = CpuSweep(w, threads, 20).step(20)
        out["cpu_baseline"] = {"value": cev / cdt, "unit": "chi2 evals/s", "cores": threads,
                               "kind": "port",
                               "sample": "20 iterations of all replicas (%d evals)" % cev}
    return out


def run_plugin(args, rank, world, local):
    r = measure_plugin(args.workload, args.steps, args.warmup, local, rank, world)
    if rank != 0:
        return
    line = {
        "metric": "chi2 model evals/sec", "value": r["value"], "unit": "chi2 evals/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": r["workload"], "launch": r["launch"], "step": r["step"]},
        "cpu_baseline": r.get("cpu_baseline"), "clocks": r["clocks"],
        "gpu_launches": r["gpu_launches"],
    }
    print(json.dumps(line))


def main():
    args = parse()
    rank, world, local = dist_setup(args)
    if args.impl == "mine" and args.workload == "batch":
        run_batch(args, rank, world, local)
    elif args.impl == "mine" and args.workload == "ess":
        run_ess(args, rank, world, local)
    elif args.impl == "mine" and args.workload == "ess-batch":
        run_ess_batch(args, rank, world, local)
    elif args.impl == "mine" and args.workload in ("rosenbrock", "nlsys"):
        run_plugin(args, rank, world, local)
    elif args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_mine(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
