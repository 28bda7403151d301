/*
 * cuda_mcmc.h -- C-ABI of the GB300 MCMC-RE sweep libraries.
 *
 * Every model library (libcmc_sgra.so for the built-in Sgr A* model,
 * libcmc_<name>.so for a model.cuh plugin) exports exactly these symbols.
 * All arguments are plain pointers and sizes.
 *
 * Entry points that replace the reference's (MITHaystack/cuda_mcmc,
 * src/mcmc.h:7-32, implemented in src/mcmcjob.cu:227-298 and :475-545):
 * identical signatures, argument meaning, array layouts and in-place output
 * semantics.  The arrays are caller-owned HOST buffers; the call copies them
 * to the device, runs, and writes every output back into the same buffers.
 * Where the reference reports a CUDA error by printing and calling exit(1)
 * (src/mcmcjob.cu:212-219), these print to stderr and return; the _v2
 * variants return the status instead (see cmc_last_error()).
 */
#ifndef CUDA_MCMC_H
#define CUDA_MCMC_H

#include <stddef.h>

#include "cmc_job.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Replaces mcmc_cuda, src/mcmc.h:7-20 / src/mcmcjob.cu:475-545: the full
 * burn-in + main-stage MCMC-RE run (run_mcmc, src/gpu_mcmc.cu:682-763).
 * Inputs: coor, dat, std2r, icoor, idat, pdescr, ivar, invar, ptotal, pmint,
 * pmaxt, beta and the starting tcur, flag, n_acpt, n_exch, n_cnt, n_hist, pstp,
 * ptent, ptentn, pcur (mutable parameters are re-drawn from the prior, as
 * init_pcur does).  Outputs (in place): pout [nprm][nbeta][nseq][niter],
 * tout [nbeta][nseq][niter], chi2 [nseq][niter], the final sampler state
 * (pcur, chi2c, flag, tcur, pstp, ptent, ptentn, n_acpt, n_exch, n_cnt,
 * n_hist, rndst = cuRAND XORWOW states, 48 bytes per replica) and the model
 * rows datm / chi2m of each replica's last evaluation. */
void mcmc_cuda(float *coor, float *dat, float *std2r, int *icoor, int *idat, float *datm,
               float *chi2m, int *pdescr, int *ivar, int *invar, float *ptotal, float *pmint,
               float *pmaxt, float *pout, int *tout, float *chi2, float *chi2c, int *tcur,
               int *flag, int *n_acpt, int *n_exch, int *n_cnt, int *n_hist, float *beta,
               float *pstp, float *ptent, int *ptentn, float *pcur, unsigned char *rndst,
               unsigned long long seed, int imodel, int ncoor, int ndat, int nicoor, int nidat,
               int ndatm, int nptot, int nprm, int nadj, int npass, int nbeta, int nseq,
               int nburn, int niter);

/* Replaces calc_modchi2, src/mcmc.h:23-27 / src/mcmcjob.cu:227-254 (the
 * header names the 17th int nprm, the definition nptot; it is nptot): model
 * values datm, chi^2 terms chi2m and chi2c = sum of each chi2m row for the
 * nbeta*nseq parameter sets in pcur whose flag is non-zero (two passes, as
 * run_calcmodchi2, src/gpu_mcmc.cu:769-783). */
void calc_modchi2(float *coor, float *dat, float *std2r, int *icoor, int *idat, float *datm,
                  float *chi2m, float *pcur, float *chi2c, int *flag, int imodel, int ncoor,
                  int ndat, int nicoor, int nidat, int ndatm, int nptot, int nbeta, int nseq);

/* Replaces calc_model, src/mcmc.h:30-32 / src/mcmcjob.cu:257-298: model
 * values only (pass 0, run_calcmodel, src/gpu_mcmc.cu:790-802) for every
 * parameter set in pcur (the reference leaves its flag array uninitialised;
 * here every set is evaluated). */
void calc_model(float *coor, int *idat, float *datm, float *pcur, int imodel, int ncoor,
                int ndat, int nidat, int ndatm, int nptot, int nbeta, int nseq);

/* Same arguments as the three above; return a cmc_status (0 = success).
 * Reference counterparts: mcmc_cuda / calc_modchi2 / calc_model, whose
 * failure path is CUDA_CALL -> cudaAssert -> exit(1) (src/mcmcjob.cuh:6). */
int mcmc_cuda_v2(float *coor, float *dat, float *std2r, int *icoor, int *idat, float *datm,
                 float *chi2m, int *pdescr, int *ivar, int *invar, float *ptotal, float *pmint,
                 float *pmaxt, float *pout, int *tout, float *chi2, float *chi2c, int *tcur,
                 int *flag, int *n_acpt, int *n_exch, int *n_cnt, int *n_hist, float *beta,
                 float *pstp, float *ptent, int *ptentn, float *pcur, unsigned char *rndst,
                 unsigned long long seed, int imodel, int ncoor, int ndat, int nicoor, int nidat,
                 int ndatm, int nptot, int nprm, int nadj, int npass, int nbeta, int nseq,
                 int nburn, int niter);
int calc_modchi2_v2(float *coor, float *dat, float *std2r, int *icoor, int *idat, float *datm,
                    float *chi2m, float *pcur, float *chi2c, int *flag, int imodel, int ncoor,
                    int ndat, int nicoor, int nidat, int ndatm, int nptot, int nbeta, int nseq);
int calc_model_v2(float *coor, int *idat, float *datm, float *pcur, int imodel, int ncoor,
                  int ndat, int nidat, int ndatm, int nptot, int nbeta, int nseq);

/* Message of the last failed call on this thread ("" after a success).
 * The reference prints "Cuda error in file ..." (src/mcmcjob.cu:212-219). */
const char *cmc_last_error(void);

/* Replaces reset_gpu, src/mcmc_interf.pyx:342-343 (cudaDeviceReset): waits
 * for the device instead of destroying the context other libraries share.
 * Returns a cmc_status. */
int cmc_reset_gpu(void);

/* ---- device-pointer API: the same sweep on arrays already in GPU memory ----
 * Reference counterpart: CMcmcFit::do_mcmc_on_gpu -> run_mcmc
 * (src/mcmcjob.cu:835-848, src/gpu_mcmc.cu:682-763) on the device copies that
 * the CMcmcFit constructor made (src/mcmcjob.cu:552-755); here the caller owns
 * the device arrays (see cmc_job in cmc_job.h).  A job can run in chunks:
 * do_init = 0 resumes from the state arrays (including the generator states),
 * and main iteration m of a launch is recorded at column itr0 + m.  Launches
 * are asynchronous on `stream` (a cudaStream_t; NULL = legacy default stream);
 * the kernels report device-side failures in job->status. */
int cmc_run(const cmc_job *job, void *stream);

/* libcmc_sgra.so only.  No counterpart in the reference.  cmc_run for callers
 * that cannot allocate device memory at run time (their memory is reserved
 * up front by another allocator, or a cudaMalloc / cudaFree would synchronise
 * a latency-critical pipeline): job->work is ignored and the scratch comes
 * from a fixed 4 MiB array inside the library instead.  Limits: the packed
 * data (52 bytes per point + 32 per closure: at most about 80,000 points,
 * else CMC_ERR_ARG), and the closure phases of all replicas either beside it
 * in the array ((nbeta*nseq + 8)*points*4 bytes, from 2048 points on) or else in
 * shared memory (R*points*4 bytes per CTA with R >= nbeta/16: up to about
 * 27,000 points at 32 temperatures), else CMC_ERR_UNSUPPORTED.  A large job
 * whose phases cmc_run would keep in a full job->work may therefore run here
 * with its phases in shared memory, at another launch shape and speed.  The
 * array's address is resolved by the first call on each device, which should
 * come before any stream capture, and cached for the life of the process (it
 * is stale after a cudaDeviceReset); all calls share the array, so calls that
 * overlap on the GPU race. */
int cmc_run_noalloc(const cmc_job *job, void *stream);

/* Reference counterpart: run_calcmodchi2 / run_calcmodel
 * (src/gpu_mcmc.cu:769-802) on device arrays: mode 1 = calc_modchi2,
 * mode 2 = calc_model.  Asynchronous on `stream`. */
int cmc_eval(const cmc_job *job, int mode, void *stream);

/* ---- chi^2 gradient (Sgr A* model; libcmc_sgra.so only) ---------------------
 * No counterpart in the reference (its sampler uses no derivatives).
 * cmc_grad writes chi2c[ist] and d chi2 / d p into grad[ist*nptot + k] at
 * p = pcur[ist*nptot ..] for every replica ist < nbeta*nseq (zeros where flag
 * is non-NULL and flag[ist] == 0).  chi2 is the sum the sweep minimises:
 * amplitude terms, plus closure-phase terms when npass >= 2
 * (src/gpu_mcmc.cu:305-323 over examples/sgra_model_fit/model.cuh).  Needs
 * coor, dat, std2r, icoor, idat, pcur, chi2c, status and job->work of at least
 * cmc_grad_work_bytes(job) bytes; nptot <= 16.  Asynchronous on `stream`. */
size_t cmc_grad_work_bytes(const cmc_job *job);
int cmc_grad(const cmc_job *job, float *grad, void *stream);

/* Gauss-Newton Fisher information of chi^2/2 (libcmc_sgra.so only; no
 * counterpart in the reference):
 *   fisher[ist][a][b] = sum_i w_i dA_i/dp_a dA_i/dp_b
 *                     + sum_c w_c dphi_c/dp_a dphi_c/dp_b
 * over the amplitude terms i and (npass >= 2) the closure-phase terms c of
 * the chi^2 above, at p = pcur[ist] for every replica (zeros where flag[ist]
 * == 0).  Same inputs as cmc_grad; job->work of at least
 * cmc_fisher_work_bytes(job) bytes.  Asynchronous on `stream`. */
size_t cmc_fisher_work_bytes(const cmc_job *job);
int cmc_fisher(const cmc_job *job, float *fisher, void *stream);

/* ---- batches of independent jobs (fits) ------------------------------------
 * No counterpart in the reference (it runs one fit per mcmc_cuda call).
 * Every job is a complete cmc_job (device arrays, own sizes; all with the same
 * nbeta).  cmc_batch_prepare validates the jobs, packs their data (each job's
 * own job->work), splits the (job, sequence) items into size classes and
 * uploads the descriptors and work lists into `work` (cmc_batch_work_bytes
 * bytes, caller-owned device memory); it returns an opaque plan (NULL on
 * error, see cmc_last_error).  cmc_batch_run then only launches: one
 * persistent kernel per size class whose clusters take items, largest first,
 * from an atomic counter, with this launch's iteration window (do_init, nburn,
 * niter, itr0) applied to every job; it can be captured in a CUDA graph.
 * cmc_batch_info reports class `cls`'s launch shape (returns the number of
 * classes); cmc_batch_free releases the host-side plan.
 * cmc_batch_set_class gives class `cls` another launch shape (R replicas per
 * CTA, T threads, phase mode 0/1/2) when every job of the class fits it, and
 * re-uploads the descriptors (synchronising `stream`); cmc_batch_run_class
 * launches that class alone.  Together they let a caller time the shapes of
 * each class (cuda_mcmc_gb300.device.BatchJob.autotune). */
size_t cmc_batch_work_bytes(const cmc_job *jobs, int njobs);
void *cmc_batch_prepare(const cmc_job *jobs, int njobs, void *work, size_t work_bytes,
                        void *stream);
int cmc_batch_run(void *plan, int do_init, int nburn, int niter, int itr0, void *stream);
int cmc_batch_info(void *plan, int cls, int *R, int *G, int *T, int *phasor, int *nitems,
                   int *nclusters, size_t *smem);
int cmc_batch_run_class(void *plan, int cls, int do_init, int nburn, int niter, int itr0,
                        void *stream);
int cmc_batch_set_class(void *plan, int cls, int R, int T, int phasor, void *stream);
/* Cancel the plan's running batch launches: callable from any host thread
 * while cmc_batch_run's launches run on their stream (a cancel that lands
 * before the run's first memset has executed is cleared by it).  A cluster takes no further (fit, sequence)
 * item, and one in the middle of an item stops after the exchange of its
 * current iteration with its state and records written back; every job of
 * the plan gets CMC_ERR_CANCELLED in its status word (the jobs are left at
 * different iterations).  The next cmc_batch_run clears the cancel flags;
 * the status words stay until the caller resets them.  No reference
 * counterpart (the reference has no batches). */
int cmc_batch_cancel(void *plan);
void cmc_batch_free(void *plan);

/* Bytes of library scratch (packed data of the built-in fast models) that
 * job->work must provide for cmc_run (mode 0) or cmc_eval (mode 1, 2).  The
 * reference allocates its device buffers itself (src/mcmcjob.cu:689-718). */
size_t cmc_work_bytes(const cmc_job *job, int mode);

/* Launch shape the library picks for a cmc_run of this job: replicas per
 * CTA R, cluster size G = nbeta/R, threads per CTA T, closure storage
 * (1 = unit phasors, 0 = phases in shared memory, 2 = phases in global
 * memory, which needs job->work of cmc_work_bytes(job, 0) bytes), dynamic
 * shared memory and resident clusters per wave.  In the spread layout (see
 * cmc_set_layout) G is 0 and *clusters_per_wave is the number of CTAs.  The reference always launches <<<nseq, nbeta>>> per
 * step kernel and <<<nbeta*nseq*ndat/128+1, 128>>> for the model
 * (src/gpu_mcmc.cu:686-687). */
int cmc_query_config(const cmc_job *job, int *R, int *G, int *T, int *phasor, size_t *smem,
                     int *clusters_per_wave);

/* Force a launch shape (0 / -1 = automatic), e.g. from the autotuner.  No
 * reference counterpart (the reference's shape is fixed). */
void cmc_set_config(int R, int T, int phasor);

/* Force the replica layout of cmc_run's sweep (0 = automatic).  1: one
 * thread-block cluster per sequence, its nbeta/R CTAs holding R temperatures
 * each, the exchange over distributed shared memory.  2 (built-in Sgr A*
 * model, nbeta <= 32, job->work of cmc_work_bytes(job, 0) bytes): one
 * cooperative launch whose CTAs share the nbeta*nseq replicas evenly (R or
 * R - 1 each, sequence-major), each sequence's exchange run by the CTA
 * holding its ibeta = 0 replica through job->work; the automatic choice
 * takes it where it leaves fewer replicas on the busiest SM.  Same chains
 * either way.  No reference counterpart. */
void cmc_set_layout(int layout);

/* Spread layout only: force the number of sequence groups and of CTAs
 * (0 = automatic).  A spread launch runs its sequences in `groups` groups
 * (nseq / groups each, the first nseq % groups one more) one after the
 * other on all of its CTAs, so that with phases in global memory only one
 * group's phase regions are in use (the automatic choice: the fewest groups
 * whose corner phases fit in L2).  `blocks` must lie between the fewest CTAs
 * that hold the largest group at R replicas each and the smallest group's
 * replica count.  Same chains whatever the grouping.  No reference
 * counterpart. */
void cmc_set_spread(int groups, int blocks);

/* The spread layout's CTAs and sequence groups for this job (both 0 in the
 * cluster layout); returns a cmc_status.  No reference counterpart. */
int cmc_query_spread(const cmc_job *job, int *blocks, int *groups);

/* libcmc_module.so only; no reference counterpart.  That library is the
 * plugin C-ABI without a model compiled in: its launches take the kernels
 * from a CUDA module file (a cubin or PTX built from a model.cuh with
 * cuda_mcmc_gb300/csrc/module_plugin.cu), loaded at the first launch from
 * `path` (or, without a call, from the environment variable
 * CMC_PLUGIN_MODULE).  Call before the first launch (afterwards only the
 * same path is accepted); returns a cmc_status. */
int cmc_module_set(const char *path);

/* Library identification; no reference counterpart. */
const char *cmc_model_name(void);
int cmc_abi_version(void);
int cmc_sizeof_job(void);

#ifdef __cplusplus
}
#endif

#endif /* CUDA_MCMC_H */
