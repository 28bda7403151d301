// cmc_host.cuh -- host side of the C-ABI, shared by every model library.
//
// A model library is one translation unit that includes this header with
// CMC_MODEL set to a model policy (SgraModel, PluginModel) and
// CMC_MODEL_NAME to its name; it then exports the reference's entry points
// (src/mcmc.h:7-32) plus the status-returning and device-pointer variants
// declared in include/cuda_mcmc.h.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "cmc_common.cuh"
#include "cmc_job.h"
#include "cmc_launch.cuh"

namespace cmc {

inline std::string &last_error()
{
  static thread_local std::string e;
  return e;
}

// Defined once per library (non-inline): the kernel-instance objects call it.
int fail(int code, const std::string &msg)
{
  last_error() = msg;
  return code;
}

inline int cuda_fail(cudaError_t e, const char *what)
{
  return fail(CMC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CMC_CUDA(call)                                   \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);  \
  } while (0)

// Launch-shape override set by cmc_set_config / cmc_set_layout /
// cmc_set_spread (the autotuner, tests) or, where those are unset, by the
// environment variables CUDA_MCMC_R, CUDA_MCMC_THREADS, CUDA_MCMC_PHASOR,
// CUDA_MCMC_LAYOUT, CUDA_MCMC_GROUPS and CUDA_MCMC_BLOCKS; 0 (phase mode -1)
// = automatic.
struct Override {
  int R = 0, T = 0, phasor = -1;
  int layout = 0;   // 0 = automatic, 1 = cluster layout, 2 = spread layout
  int groups = 0, blocks = 0;   // spread layout: sequence groups and CTAs (0 = automatic)
};
inline Override &override_cfg()
{
  static Override o;
  return o;
}

inline int env_int(const char *name, int dflt)
{
  const char *v = std::getenv(name);
  return (v && *v) ? std::atoi(v) : dflt;
}

// Calls f(std::integral_constant<int, R>) for the instantiated R values of
// the model (R <= Model::kMaxR).
template <class Model, class F>
inline int dispatch_R(int R, F &&f)
{
  switch (R) {
    case 1: return f(std::integral_constant<int, 1>{});
    case 2: return f(std::integral_constant<int, 2>{});
    case 4: return f(std::integral_constant<int, 4>{});
    case 8: return f(std::integral_constant<int, 8>{});
    case 16:
      if constexpr (Model::kMaxR >= 16) return f(std::integral_constant<int, 16>{});
      break;
    case 32:
      if constexpr (Model::kMaxR >= 32) return f(std::integral_constant<int, 32>{});
      break;
    default: break;
  }
  return fail(CMC_ERR_UNSUPPORTED, "no kernel instance for this replicas-per-CTA count");
}

// Calls f(std::integral_constant<int, R>) for the spread-layout kernel
// instances (R = 1..Model::kMaxR of a model with Model::kSpread).
template <class Model, class F>
inline int dispatch_spread_R(int R, F &&f)
{
  if constexpr (Model::kSpread) {
    static_assert(Model::kMaxR <= 8, "spread instances cover R = 1..8");
    switch (R) {
      case 1: return f(std::integral_constant<int, 1>{});
      case 2: return f(std::integral_constant<int, 2>{});
      case 3: return f(std::integral_constant<int, 3>{});
      case 4: return f(std::integral_constant<int, 4>{});
      case 5: return f(std::integral_constant<int, 5>{});
      case 6: return f(std::integral_constant<int, 6>{});
      case 7: return f(std::integral_constant<int, 7>{});
      case 8: return f(std::integral_constant<int, 8>{});
      default: break;
    }
  }
  return fail(CMC_ERR_UNSUPPORTED, "no spread-layout kernel instance for this replicas-per-CTA count");
}

inline int smem_optin()
{
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return v;
}

inline int sm_count()
{
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
  return v > 0 ? v : 1;
}

inline long long l2_bytes()
{
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrL2CacheSize, dev);
  return v;
}

template <class Model>
size_t plan_bytes(const cmc_job &j, const typename Model::Packed &pk, int R, int T, int sweep)
{
  if (sweep)
    return make_plan(R, T, j.nptot, j.nprm, j.nbeta, j.nadj, sizeof(typename Model::Consts),
                     Model::scratch_bytes(pk, R)).total;
  return make_plan(R, T, j.nptot, 1, 1, 1, sizeof(typename Model::Consts),
                   Model::scratch_bytes(pk, R)).total;
}

// Phase mode 2 (global memory) is available: the model supports it and the
// job's work holds the regions (Model::host_dims set the pointer).
template <class Model>
inline bool global_phases_ok(const typename Model::Packed &pk)
{
  if constexpr (Model::kGlobalPhases) return pk.gph != nullptr;
  else return false;
}

// Data terms per replica evaluation up to which a sweep is latency-bound (the
// launch-shape ranking below then minimises the work per CTA).
constexpr int kFewPoints = 64;

// The spread layout's exchange area sits in job.work after the model's
// scratch (packed data and, when allocated, global phase regions).
template <class Model>
inline size_t spread_offset(const typename Model::Packed &pk)
{
  return align256(Model::host_work_bytes(pk));
}

// The spread layout can run this job: the model has it, every sequence's
// exchange fits one warp (nbeta <= 32) and job.work holds the exchange area
// (after the phase regions, of which the model allocates nrep + kMaxR).
template <class Model>
inline bool spread_ok(const cmc_job &j, const typename Model::Packed &pk)
{
  if constexpr (!Model::kSpread) {
    return false;
  } else {
    if (j.nbeta > 32 || j.work == nullptr) return false;
    return j.work_bytes >= spread_offset<Model>(pk) + spread_ctl_bytes(j.nseq, j.nbeta, j.nptot);
  }
}

// Pick replicas-per-CTA R (cluster size G = nbeta/R <= 16), threads T and the
// phase storage mode by the ranking below (autotune.py measures instead).
template <class Model>
int pick_sweep_config(const cmc_job &j, typename Model::Packed &pk, LaunchCfg &out)
{
  out = LaunchCfg{};
  const Override &ov = override_cfg();
  const int Rfix = ov.R ? ov.R : env_int("CUDA_MCMC_R", 0);
  const int Tfix = ov.T ? ov.T : env_int("CUDA_MCMC_THREADS", 0);
  const int Pfix = ov.phasor >= 0 ? ov.phasor : env_int("CUDA_MCMC_PHASOR", -1);
  const int Lfix = ov.layout ? ov.layout : env_int("CUDA_MCMC_LAYOUT", 0);
  const int lim = smem_optin();
  const double l2_budget = 0.75 * (double)l2_bytes();
  double best = 1e300;
  bool found = false;
  const int Rs[] = {1, 2, 4, 8, 16, 32};
  for (int R : Rs) {
    if (Lfix == 2) break;   // spread layout only
    if (R > Model::kMaxR) continue;
    if (Rfix && R != Rfix) continue;
    if (j.nbeta % R != 0) continue;
    const int G = j.nbeta / R;
    if (G > 16) continue;
    const int Ts[] = {64, 128, 256};
    for (int T : Ts) {
      if (Tfix && T != Tfix) continue;
      if (!Tfix && T == 64 && R > 4) continue;
      for (int ph = 2; ph >= 0; --ph) {
        if (Pfix >= 0 && ph != Pfix) continue;
        if (ph == 2 && !global_phases_ok<Model>(pk)) continue;
        typename Model::Packed q = pk;
        q.phasor = ph;
        const size_t smem = plan_bytes<Model>(j, q, R, T, 1);
        if ((long long)smem > lim) continue;
        const int n = dispatch_R<Model>(R, [&](auto rc) {
          return sweep_capacity<Model, decltype(rc)::value>(G, T, smem, j.nseq);
        });
        if (n <= 0) continue;
        const int waves = (j.nseq + n - 1) / n;
        // Measured on GB300, lexicographic, lower is better.  With phases in
        // global memory, first whether the resident replicas' phases fit in
        // three quarters of L2 -- phases are kept for closure corners only,
        // at most 3 per closure (20000 visibilities + 6000 closures: 36 or 40
        // resident clusters of 32 replicas in two waves beat 64 clusters in
        // one by 7 %: the larger set spills to DRAM).  Then fewest
        // waves of resident clusters.  Then, with a few data terms per replica
        // (the plugin models: ndat 1-8), the per-proposal serial work of a
        // CTA's R replicas is the time: fewest replicas per CTA, then fewest
        // threads (Rosenbrock, 16 x 32: R=2 T=64 4.3 ms, R=8 T=256 6.9 ms).
        // Otherwise (Sgr A*, 2000-20000 visibilities) about 32 threads per
        // replica (16 or 64 cost ~10 %); then the phase storage (phasors,
        // phases in shared memory, phases in global memory: an L2 round trip
        // per closure gather); then more replicas per CTA (more independent
        // work per thread), except with phases in global memory, where the
        // point data stream from L2 (loaded two points ahead up to R = 4)
        // and 2, then 4, replicas per CTA do best (20000 + 6000, 10
        // iterations: R=2 T=128 21.7 ms, R=4 T=256 22.8 ms, R=4 T=128 23.0
        // ms; R=8 T=256 12.7 ms against R=4 T=128 11.1 ms per 4 iterations).
        double phase_set = 0.0;
        if constexpr (Model::kGlobalPhases) {
          if (ph == 2) {
            const int corners = (q.ncph > 0 && q.npass >= 2) ? std::min(q.npts, 3 * q.ncph) : 0;
            phase_set = (double)std::min(n, j.nseq) * j.nbeta * (double)corners * 4.0;
          }
        }
        const int spill = (ph == 2 && l2_budget > 0.0 && phase_set > l2_budget) ? 1 : 0;
        double score = spill * 100000.0;
        if (Model::points(q) <= kFewPoints) {
          score += waves * 1000.0 + R * 10.0 + T / 64;
        } else {
          // A job whose replicas at 64 threads each fill at most half of the
          // GPU's thread slots (few sequences) runs faster with 64 threads
          // per replica (2000 + 600 data, 8 x 32: R=4 T=256 2.8e7 evals/s,
          // R=8 T=256 1.7e7; 2 x 32: 6.9e6 and 4.3e6); otherwise about 32.
          const bool small = (double)j.nseq * j.nbeta * 64.0 <= (double)sm_count() * 1024.0;
          const int tpr = T / R;
          const int shape_rank =
              small ? ((tpr == 64) ? 0 : (tpr == 32 || tpr == 128) ? 1 : 2)
                    : ((tpr == 32) ? 0 : (tpr == 64 || tpr == 16) ? 1 : 2);
          const int store_rank = (ph == 1) ? 0 : (ph == 0) ? 1 : 2;
          const double r_rank =
              (ph == 2) ? ((R == 2) ? 0.0 : (R == 4) ? 1.0 : 2.0 + std::abs(R - 4)) : -(double)R;
          score += waves * 1000.0 + shape_rank * 100.0 + store_rank * 10.0 + r_rank;
        }
        if (score < best - 1e-9) {
          best = score;
          out.R = R; out.G = G; out.T = T; out.phasor = ph; out.smem = smem;
          out.clusters_per_wave = n;
          found = true;
        }
      }
    }
  }
  // Spread layout (cmc_sweep.cuh): the replicas shared evenly by N
  // co-resident CTAs.  Chosen by itself where the cluster layout's pick puts
  // two or more CTAs on the busiest SM and the spread layout, at that pick's
  // threads and phase storage, holds fewer replicas there (2000 + 600 data,
  // 64 x 32 on 152 SMs: 293 CTAs of 6-7 replicas, at most 14 per SM, against
  // 256 CTAs of 8 with up to 16; one CTA alone on an SM runs at about 0.73 of
  // the pair's rate, so one-CTA placements are left alone).  With the layout
  // forced (cmc_set_layout 2, the autotuner): the least-loaded spread shape
  // in the cluster ranking's order.
  const int sms = sm_count();
  const int nrep = j.nbeta * j.nseq;
  const int Gfix = ov.groups ? ov.groups : env_int("CUDA_MCMC_GROUPS", 0);
  const int Nfix = ov.blocks ? ov.blocks : env_int("CUDA_MCMC_BLOCKS", 0);
  int per_sm_c = 0, load_c = 1 << 30;
  if (found) {
    const int wave = std::min(j.nseq, out.clusters_per_wave);
    per_sm_c = (out.G * wave + sms - 1) / sms;
    load_c = out.R * per_sm_c * ((j.nseq + out.clusters_per_wave - 1) / out.clusters_per_wave);
  }
  const bool spread_auto = found && Lfix == 0 && out.phasor != 2 && !Rfix && !Tfix &&
                           Model::points(pk) > kFewPoints && per_sm_c >= 2;
  if (Lfix == 2 || spread_auto) {
    double best_s = 1e300;
    LaunchCfg bs;
    bool found_s = false;
    for (int R = 1; R <= std::min(Model::kMaxR, j.nbeta); ++R) {
      if (Rfix && R != Rfix) continue;
      const int Ts[] = {64, 128, 256};
      for (int T : Ts) {
        if (Tfix && T != Tfix) continue;
        if (spread_auto && T != out.T) continue;
        if (T < 32 * ((R + 31) / 32)) continue;
        for (int ph = 2; ph >= 0; --ph) {
          if (Pfix >= 0 && ph != Pfix) continue;
          if (spread_auto && ph != out.phasor) continue;
          if (ph == 2 && !global_phases_ok<Model>(pk)) continue;
          typename Model::Packed q = pk;
          q.phasor = ph;
          if (!spread_ok<Model>(j, q)) continue;
          const size_t smem = plan_bytes<Model>(j, q, R, T, 1);
          if ((long long)smem > lim) continue;
          const int cap = dispatch_spread_R<Model>(R, [&](auto rc) {
            return spread_capacity<Model, decltype(rc)::value>(T, smem);
          });
          if (cap <= 0) continue;
          // Sequence groups, run one after the other by the same CTAs: the
          // fewest whose largest group fits the resident CTAs at R replicas
          // each and, with phases in global memory, whose largest group's
          // corner phases fit the L2 budget.
          double per_seq = 0.0;
          if constexpr (Model::kGlobalPhases) {
            if (ph == 2) {
              const int corners =
                  (q.ncph > 0 && q.npass >= 2) ? std::min(q.npts, 3 * q.ncph) : 0;
              per_seq = (double)j.nbeta * corners * 4.0;
            }
          }
          auto fits = [&](int g) {
            const int smax = (j.nseq + g - 1) / g;
            return (j.nbeta * smax + R - 1) / R <= cap && (double)smax * per_seq <= l2_budget;
          };
          int ng = Gfix ? std::min(Gfix, j.nseq) : 1;
          while (!Gfix && ng < j.nseq && !fits(ng)) ++ng;
          // CTAs: the fewest that hold the largest group at R per CTA (every
          // slot is evaluated, used or not), at most one per replica of the
          // smallest group
          const int rep_max = j.nbeta * ((j.nseq + ng - 1) / ng);
          const int rep_min = j.nbeta * (j.nseq / ng);
          const int Nlo = (rep_max + R - 1) / R;
          const int N = Nfix ? Nfix : Nlo;
          if (N < Nlo || N > std::min(cap, rep_min)) continue;
          if (ph == 2 && N * R > nrep + Model::kMaxR) continue;
          const int per_sm = (N + sms - 1) / sms;
          const int load = ng * R * per_sm;
          if (spread_auto && (load >= load_c || per_sm < per_sm_c)) continue;
          const int tpr = T / R;
          const int shape_rank = (tpr >= 32 && tpr < 64) ? 0 : (tpr >= 16 && tpr < 128) ? 1 : 2;
          const int store_rank = (ph == 1) ? 0 : (ph == 0) ? 1 : 2;
          const double score = load * 1000.0 + shape_rank * 100.0 + store_rank * 10.0 - R;
          if (score < best_s - 1e-9) {
            best_s = score;
            bs = LaunchCfg{};
            bs.R = R; bs.G = 0; bs.T = T; bs.phasor = ph; bs.smem = smem;
            bs.clusters_per_wave = N;
            bs.spread = 1;
            bs.nblocks = N;
            bs.groups = ng;
            found_s = true;
          }
        }
      }
    }
    if (found_s) {
      out = bs;
      found = true;
    } else if (Lfix == 2) {
      return fail(CMC_ERR_UNSUPPORTED,
                  "no spread-layout launch shape fits: it needs the built-in Sgr A* model, "
                  "nbeta <= 32, job.work of cmc_work_bytes() bytes and at most as many CTAs "
                  "as are resident at once");
    }
  }
  if (!found)
    return fail(CMC_ERR_UNSUPPORTED,
                "no sweep launch shape fits: nbeta must be a multiple of a power of two "
                "<= 32 with nbeta/R <= 16, and a CTA's replicas must fit in shared memory");
  pk.phasor = out.phasor;
  return CMC_OK;
}

inline int validate_common(const cmc_job &j, int mode)
{
  if (j.nbeta < 1 || j.nseq < 1 || j.nptot < 1 || j.ndat < 1)
    return fail(CMC_ERR_ARG, "nbeta, nseq, nptot and ndat must be >= 1");
  if ((long long)j.nbeta * j.nseq * (long long)std::max(j.ndat, j.nptot) > 0x7fffffffLL)
    return fail(CMC_ERR_ARG, "nbeta*nseq*ndat exceeds the 32-bit index range");
  if (!j.coor || !j.idat || !j.pcur || !j.status)
    return fail(CMC_ERR_ARG, "coor, idat, pcur and status must be device pointers");
  if (mode != 2 && (!j.dat || !j.std2r || !j.chi2c))
    return fail(CMC_ERR_ARG, "dat, std2r and chi2c must be device pointers");
  if (mode == 0) {
    if (j.nbeta < 2)
      return fail(CMC_ERR_ARG, "nbeta must be >= 2 (the replica exchange picks adjacent pairs)");
    if (j.nprm < 1 || j.nprm > j.nptot)
      return fail(CMC_ERR_ARG, "nprm must be in [1, nptot]");
    if (j.nadj < 1) return fail(CMC_ERR_ARG, "nadj must be >= 1");
    if (j.npass < 1) return fail(CMC_ERR_ARG, "npass must be >= 1");
    if (j.nburn < 0 || j.niter < 0 || j.itr0 < 0 || j.itr0 + j.niter > j.niter_total)
      return fail(CMC_ERR_ARG, "need nburn, niter >= 0 and itr0 + niter <= niter_total");
    if (!j.pdescr || !j.ivar || !j.pmint || !j.pmaxt || !j.beta || !j.flag || !j.ptent ||
        !j.ptentn || !j.pstp || !j.n_acpt || !j.n_exch || !j.n_cnt || !j.n_hist || !j.tcur)
      return fail(CMC_ERR_ARG, "a sampler state array is missing");
    if (j.niter > 0 && (!j.pout || !j.tout || !j.chi2))
      return fail(CMC_ERR_ARG, "pout, tout and chi2 are required when niter > 0");
    if (j.rng_mode == CMC_RNG_CURAND && !j.rndst)
      return fail(CMC_ERR_ARG, "rndst is required for the cuRAND generator");
    if (j.rng_mode == CMC_RNG_INJECTED && (!j.inj_u || !j.inj_n || !j.inj_cur))
      return fail(CMC_ERR_ARG, "injected streams need inj_u, inj_n and inj_cur");
    if (j.prop_mode != CMC_PROP_SINGLE && j.prop_mode != CMC_PROP_BLOCK)
      return fail(CMC_ERR_ARG, "prop_mode must be CMC_PROP_SINGLE (0) or CMC_PROP_BLOCK (1)");
    if (j.prop_mode == CMC_PROP_BLOCK && !j.prop_chol)
      return fail(CMC_ERR_ARG, "block proposals need prop_chol [nseq][nprm][nprm]");
    if (j.nseq_total < 0 ||
        (j.nseq_total > 0 && (j.seq_offset < 0 || j.seq_offset + j.nseq > j.nseq_total)))
      return fail(CMC_ERR_ARG, "sharding: need 0 <= seq_offset and seq_offset + nseq <= nseq_total");
  }
  return CMC_OK;
}

template <class Model>
int run_sweep(const cmc_job &j, cudaStream_t s, LaunchCfg *used = nullptr)
{
  int rc = validate_common(j, 0);
  if (rc) return rc;
  typename Model::Packed pk;
  const char *err = nullptr;
  rc = Model::host_dims(j, 0, pk, &err);
  if (rc) return fail(rc, err);
  if (Model::host_work_bytes_min(pk) > 0 &&
      (j.work == nullptr || j.work_bytes < Model::host_work_bytes_min(pk)))
    return fail(CMC_ERR_ARG, "job.work is smaller than the packed data (cmc_work_bytes())");
  LaunchCfg c;
  rc = pick_sweep_config<Model>(j, pk, c);
  if (rc) return rc;
  rc = Model::host_pack(j, pk, j.work, s);
  if (rc) return fail(rc, "packing the model data failed");
  if (c.spread) {
    void *ctl = static_cast<unsigned char *>(j.work) + spread_offset<Model>(pk);
    rc = dispatch_spread_R<Model>(c.R, [&](auto rcnst) {
      return launch_spread<Model, decltype(rcnst)::value>(j, pk, c, ctl, s);
    });
  } else {
    rc = dispatch_R<Model>(c.R, [&](auto rcnst) {
      return launch_sweep<Model, decltype(rcnst)::value>(j, pk, c, s);
    });
  }
  if (used) *used = c;
  return rc;
}

template <class Model>
int run_eval(const cmc_job &j, int mode, cudaStream_t s)
{
  int rc = validate_common(j, mode);
  if (rc) return rc;
  typename Model::Packed pk;
  const char *err = nullptr;
  rc = Model::host_dims(j, mode, pk, &err);
  if (rc) return fail(rc, err);
  if (Model::host_work_bytes_min(pk) > 0 &&
      (j.work == nullptr || j.work_bytes < Model::host_work_bytes_min(pk)))
    return fail(CMC_ERR_ARG, "job.work is smaller than the packed data (cmc_work_bytes())");
  pk.phasor = 0;
  const int lim = smem_optin();
  const int T = 128;
  int R = 0;
  size_t smem = 0;
  const int Rs[] = {4, 2, 1};
  for (int r : Rs) {
    if (r > Model::kMaxR) continue;
    smem = plan_bytes<Model>(j, pk, r, T, 0);
    if ((long long)smem <= lim) { R = r; break; }
  }
  if (!R && global_phases_ok<Model>(pk)) {   // phases in global memory
    pk.phasor = 2;
    for (int r : Rs) {
      if (r > Model::kMaxR) continue;
      smem = plan_bytes<Model>(j, pk, r, T, 0);
      if ((long long)smem <= lim) { R = r; break; }
    }
  }
  if (!R)
    return fail(CMC_ERR_UNSUPPORTED, "one replica's model rows do not fit in shared memory "
                                     "(give job.work cmc_work_bytes() bytes for larger data)");
  rc = Model::host_pack(j, pk, j.work, s);
  if (rc) return fail(rc, "packing the model data failed");
  // A count whose kernel a loaded module lacks (libcmc_module.so) reports
  // CMC_ERR_UNSUPPORTED before launching anything: fall back to fewer
  // replicas per CTA (the plan of R replicas also fits R/2).
  for (; R >= 1; R /= 2) {
    smem = plan_bytes<Model>(j, pk, R, T, 0);
    rc = dispatch_R<Model>(R, [&](auto rcnst) {
      return launch_eval<Model, decltype(rcnst)::value>(j, pk, mode == 2 ? 1 : 0, T, smem, s);
    });
    if (rc != CMC_ERR_UNSUPPORTED) return rc;
  }
  return rc;
}

template <class Model>
size_t work_bytes(const cmc_job &j, int mode)
{
  typename Model::Packed pk;
  const char *err = nullptr;
  if (Model::host_dims(j, mode, pk, &err)) return 0;
  if constexpr (Model::kSpread) {
    // a sweep's spread-layout exchange area after the model's scratch
    if (mode == 0 && j.nbeta <= 32)
      return spread_offset<Model>(pk) + spread_ctl_bytes(j.nseq, j.nbeta, j.nptot);
  }
  return Model::host_work_bytes(pk);
}

// The smallest job.work a launch accepts: the packed data alone (no global
// phase regions).
template <class Model>
size_t work_bytes_min(const cmc_job &j, int mode)
{
  typename Model::Packed pk;
  const char *err = nullptr;
  if (Model::host_dims(j, mode, pk, &err)) return 0;
  return Model::host_work_bytes_min(pk);
}

// ---- batches of independent jobs (fits) ------------------------------------

// One size class of a batch: one persistent batch-kernel launch whose work
// list holds the (job, sequence) items of the class's jobs.
struct BatchClass {
  int R = 0, G = 0, T = 0, phasor = 0, item0 = 0, nitems = 0, nclusters = 0;
  size_t smem = 0;
};

struct BatchPlan {
  int njobs = 0, min_niter_total = 0;
  std::vector<BatchClass> classes;
  cmc_job *jobs_dev = nullptr;
  void *pks_dev = nullptr;
  int2 *items_dev = nullptr;
  int *counters_dev = nullptr;      // [class][2]: work-list counter, cancel flag
  int *cancel_src = nullptr;        // pinned host values the cancel copies from (a copy
                                    // from pinned memory runs beside running launches)
  std::vector<cmc_job> jobs;        // host copies (kept for the uploads)
  std::vector<unsigned char> pks;   // host copies of the packed descriptors
  std::vector<int2> items;
  ~BatchPlan()
  {
    if (cancel_src) cudaFreeHost(cancel_src);
  }
};

constexpr int kBatchMaxClasses = 4;
constexpr int kBatchClassLimit[kBatchMaxClasses] = {2048, 8192, 32768, 1 << 30};

template <class Model>
size_t batch_work_bytes(const cmc_job *jobs, int n)
{
  size_t items = 0;
  for (int i = 0; i < n; ++i) items += (size_t)std::max(jobs[i].nseq, 0);
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  return al(sizeof(cmc_job) * n) + al(sizeof(typename Model::Packed) * n) + al(8 * items) +
         al(8 * kBatchMaxClasses);
}

template <class Model>
int batch_prepare(const cmc_job *jobs, int n, void *work, size_t bytes, cudaStream_t s,
                  BatchPlan **out)
{
  using Packed = typename Model::Packed;
  *out = nullptr;
  if (!jobs || n < 1) return fail(CMC_ERR_ARG, "batch: need at least one job");
  if (!work || bytes < batch_work_bytes<Model>(jobs, n))
    return fail(CMC_ERR_ARG, "batch: work is smaller than cmc_batch_work_bytes()");
  BatchPlan *P = new BatchPlan();
  P->njobs = n;
  P->jobs.assign(jobs, jobs + n);
  P->pks.resize(sizeof(Packed) * n);
  Packed *pk = reinterpret_cast<Packed *>(P->pks.data());
  std::vector<int> npts(n);
  P->min_niter_total = 1 << 30;
  int rc = CMC_OK;
  for (int i = 0; i < n; ++i) {
    cmc_job v = jobs[i];
    v.nburn = 0;
    v.itr0 = 0;
    v.niter = std::min(1, v.niter_total);
    if ((rc = validate_common(v, 0)) != CMC_OK) break;
    if (v.nbeta != jobs[0].nbeta) {
      rc = fail(CMC_ERR_ARG, "batch: every job must have the same nbeta");
      break;
    }
    const char *err = nullptr;
    if ((rc = Model::host_dims(v, 0, pk[i], &err)) != CMC_OK) {
      fail(rc, err);
      break;
    }
    const size_t wb = Model::host_work_bytes_min(pk[i]);
    if (wb > 0 && (v.work == nullptr || v.work_bytes < wb)) {
      rc = fail(CMC_ERR_ARG, "batch: a job's work is smaller than cmc_work_bytes()");
      break;
    }
    if ((rc = Model::host_pack(v, pk[i], v.work, s)) != CMC_OK) {
      fail(rc, "batch: packing a job's data failed");
      break;
    }
    npts[i] = Model::scratch_bytes(pk[i], 1);   // per-replica scratch: the size key
    P->min_niter_total = std::min(P->min_niter_total, v.niter_total);
  }
  if (rc != CMC_OK) {
    delete P;
    return rc;
  }
  // size classes, each a work list sorted by decreasing cost (LPT)
  const int lim = smem_optin();
  const int nbeta = jobs[0].nbeta;
  for (int c = 0; c < kBatchMaxClasses; ++c) {
    const int lo = c ? kBatchClassLimit[c - 1] : -1, hi = kBatchClassLimit[c];
    std::vector<int> mem;
    for (int i = 0; i < n; ++i) {
      const int key = (int)(npts[i] / 4);
      if (key > lo && key <= hi) mem.push_back(i);
    }
    if (mem.empty()) continue;
    const int size_rank = (int)P->classes.size();   // 0 for the smallest non-empty class
    std::stable_sort(mem.begin(), mem.end(), [&](int a, int b) {
      return (double)npts[a] * (double)jobs[a].nseq > (double)npts[b] * (double)jobs[b].nseq;
    });
    int big = mem[0];
    for (int i : mem)
      if (npts[i] > npts[big]) big = i;
    BatchClass bc;
    double best = -1.0;
    long long reps = 0;
    for (int i : mem) reps += (long long)jobs[i].nseq * nbeta;
    bool gl_all = true;   // every job of the class can keep its phases in global memory
    for (int i : mem) gl_all = gl_all && global_phases_ok<Model>(pk[i]);
    const int Rs[] = {1, 2, 4, 8, 16, 32};
    for (int R : Rs) {
      if (R > Model::kMaxR || nbeta % R || nbeta / R > 16) continue;
      const int G = nbeta / R;
      // Threads per replica grow with the class's data (32, 64, then 128)
      // with 4 replicas per CTA, 2 from the third class on: the shapes
      // BatchJob.autotune measured best on GB300 over 1024 fits of
      // 500-50000 visibilities (R=4 T=128 phases in shared memory; R=4
      // T=256 and R=2 T=256, phases in global memory; 1.86e7 evals/s
      // against 1.54e7 for the most resident replicas).  The larger a
      // class's items, the more its time is the tail of its last items,
      // which more threads per replica shorten.  Other shapes rank by
      // resident replicas, after these.
      const int tpr = 32 << std::min(size_rank, 2);
      const int want = tpr * R;
      if (want > 256 && R > 1) continue;
      const int T = want <= 64 ? 64 : want <= 128 ? 128 : 256;
      const bool preferred = (R == (size_rank < 2 ? 4 : 2));
      for (int ph = 2; ph >= 0; --ph) {
        if (ph == 2 && !gl_all) continue;
        Packed q = pk[big];
        q.phasor = ph;
        const size_t smem = plan_bytes<Model>(jobs[big], q, R, T, 1);
        if ((long long)smem > lim) continue;
        const int cap = dispatch_R<Model>(R, [&](auto rcn) {
          return batch_capacity<Model, decltype(rcn)::value>(G, T, smem);
        });
        if (cap <= 0) continue;
        const double resident = std::min((double)cap * nbeta, (double)reps);
        // the first class keeps its phases in shared memory, the larger ones
        // in global memory (measured), then phasors
        const double phase_pref = (size_rank == 0) ? (ph == 0 ? 1.05 : ph == 1 ? 1.0 : 0.95)
                                                   : (ph == 2 ? 1.05 : ph == 0 ? 1.0 : 0.95);
        const double score = (preferred ? 1e9 : 0.0) + resident * phase_pref;
        if (score > best + 1e-9) {
          best = score;
          bc.R = R; bc.G = G; bc.T = T; bc.phasor = ph; bc.smem = smem; bc.nclusters = cap;
        }
      }
    }
    if (best < 0) {
      delete P;
      return fail(CMC_ERR_UNSUPPORTED, "batch: a job's data does not fit any launch shape "
                                       "(too many points for shared memory)");
    }
    for (int i : mem) pk[i].phasor = bc.phasor;
    bc.item0 = (int)P->items.size();
    for (int i : mem)
      for (int q = 0; q < jobs[i].nseq; ++q) P->items.push_back(make_int2(i, q));
    bc.nitems = (int)P->items.size() - bc.item0;
    bc.nclusters = std::min(bc.nclusters, bc.nitems);
    // the descriptors' per-job smem must fit the class's launch
    for (int i : mem) {
      if (plan_bytes<Model>(jobs[i], pk[i], bc.R, bc.T, 1) > bc.smem) {
        delete P;
        return fail(CMC_ERR_UNSUPPORTED, "batch: inconsistent class shared-memory plan");
      }
    }
    P->classes.push_back(bc);
  }
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  unsigned char *w = (unsigned char *)work;
  size_t o = 0;
  P->jobs_dev = (cmc_job *)(w + o);   o += al(sizeof(cmc_job) * n);
  P->pks_dev = (void *)(w + o);       o += al(sizeof(Packed) * n);
  P->items_dev = (int2 *)(w + o);     o += al(8 * P->items.size());
  P->counters_dev = (int *)(w + o);
  cudaError_t e = cudaHostAlloc(&P->cancel_src, 2 * sizeof(int), cudaHostAllocDefault);
  if (e == cudaSuccess) {
    P->cancel_src[0] = 1;                    // a set cancel flag
    P->cancel_src[1] = CMC_ERR_CANCELLED;    // the jobs' status
    e = cudaMemsetAsync(P->counters_dev, 0, 8 * kBatchMaxClasses, s);
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(P->jobs_dev, P->jobs.data(), sizeof(cmc_job) * n,
                                  cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(P->pks_dev, P->pks.data(), sizeof(Packed) * n, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(P->items_dev, P->items.data(), 8 * P->items.size(),
                        cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    delete P;
    return cuda_fail(e, "batch: uploading the work lists");
  }
  *out = P;
  return CMC_OK;
}

// Launches only (device-side state and work lists are ready): one memset of
// the counters and cancel flags, then one persistent kernel per size class,
// all on `s`.
template <class Model>
int batch_run(BatchPlan *P, int do_init, int nburn, int niter, int itr0, cudaStream_t s)
{
  using Packed = typename Model::Packed;
  if (!P) return fail(CMC_ERR_ARG, "batch: plan is NULL");
  if (nburn < 0 || niter < 0 || itr0 < 0 || itr0 + niter > P->min_niter_total)
    return fail(CMC_ERR_ARG, "batch: need nburn, niter >= 0 and itr0 + niter <= niter_total");
  // every class's work-list counter and cancel flag, once before the first
  // launch: a cancel that lands while one class runs stops the later ones too
  CMC_CUDA(cudaMemsetAsync(P->counters_dev, 0, 8 * kBatchMaxClasses, s));
  for (size_t c = 0; c < P->classes.size(); ++c) {
    const BatchClass &bc = P->classes[c];
    const int rc = dispatch_R<Model>(bc.R, [&](auto rcn) {
      return launch_batch<Model, decltype(rcn)::value>(
          P->jobs_dev, reinterpret_cast<const Packed *>(P->pks_dev), P->items_dev + bc.item0,
          bc.nitems, P->counters_dev + 2 * c, bc.G, bc.T, bc.smem, bc.nclusters, do_init, nburn,
          niter, itr0, s);
    });
    if (rc) return rc;
  }
  return CMC_OK;
}

// Launches of one class only (the autotuner times classes one by one).
template <class Model>
int batch_run_class(BatchPlan *P, int cls, int do_init, int nburn, int niter, int itr0,
                    cudaStream_t s)
{
  using Packed = typename Model::Packed;
  if (!P) return fail(CMC_ERR_ARG, "batch: plan is NULL");
  if (cls < 0 || cls >= (int)P->classes.size()) return fail(CMC_ERR_ARG, "batch: no such class");
  if (nburn < 0 || niter < 0 || itr0 < 0 || itr0 + niter > P->min_niter_total)
    return fail(CMC_ERR_ARG, "batch: need nburn, niter >= 0 and itr0 + niter <= niter_total");
  const BatchClass &bc = P->classes[cls];
  CMC_CUDA(cudaMemsetAsync(P->counters_dev + 2 * cls, 0, 2 * sizeof(int), s));
  return dispatch_R<Model>(bc.R, [&](auto rcn) {
    return launch_batch<Model, decltype(rcn)::value>(
        P->jobs_dev, reinterpret_cast<const Packed *>(P->pks_dev), P->items_dev + bc.item0,
        bc.nitems, P->counters_dev + 2 * cls, bc.G, bc.T, bc.smem, bc.nclusters, do_init, nburn,
        niter, itr0, s);
  });
}

// Cancel the plan's running batch launches: sets every class's cancel flag
// from a stream of its own, while the launches run (a cancel that lands
// before the run's first memset is cleared by it), and CMC_ERR_CANCELLED in
// every job's status word.
// A cluster then takes no further (fit, sequence) item, and one in the
// middle of an item stops after the exchange of its current iteration with
// its state written back (records of the iterations done included); the
// jobs are left at different iterations.  The next cmc_batch_run clears the
// flags (the status words stay until the caller resets them).
template <class Model>
int batch_cancel(BatchPlan *P)
{
  if (!P || !P->cancel_src) return fail(CMC_ERR_ARG, "batch: plan is NULL");
  cudaStream_t cs = nullptr;
  CMC_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaError_t e = cudaSuccess;
  for (size_t c = 0; c < P->classes.size() && e == cudaSuccess; ++c)
    e = cudaMemcpyAsync(P->counters_dev + 2 * c + 1, P->cancel_src, sizeof(int),
                        cudaMemcpyHostToDevice, cs);
  for (int i = 0; i < P->njobs && e == cudaSuccess; ++i)
    if (P->jobs[i].status)
      e = cudaMemcpyAsync(P->jobs[i].status, P->cancel_src + 1, sizeof(int),
                          cudaMemcpyHostToDevice, cs);
  if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
  cudaStreamDestroy(cs);
  if (e != cudaSuccess) return cuda_fail(e, "batch: setting the cancel flags");
  return CMC_OK;
}

// Give class `cls` the launch shape (R, T, phase mode) if every job of the
// class fits it; the jobs' descriptors are re-uploaded on `s` (synchronised).
template <class Model>
int batch_set_class(BatchPlan *P, int cls, int R, int T, int phasor, cudaStream_t s)
{
  using Packed = typename Model::Packed;
  if (!P) return fail(CMC_ERR_ARG, "batch: plan is NULL");
  if (cls < 0 || cls >= (int)P->classes.size()) return fail(CMC_ERR_ARG, "batch: no such class");
  const int nbeta = P->jobs[0].nbeta;
  if (R < 1 || R > Model::kMaxR || nbeta % R != 0 || nbeta / R > 16)
    return fail(CMC_ERR_UNSUPPORTED, "batch: R must divide nbeta with nbeta/R <= 16");
  if ((T != 64 && T != 128 && T != 256) || T < 32 * ((R + 31) / 32))
    return fail(CMC_ERR_UNSUPPORTED, "batch: T must be 64, 128 or 256 and >= 32 per 32 replicas");
  if (phasor < 0 || phasor > 2) return fail(CMC_ERR_ARG, "batch: phase mode must be 0, 1 or 2");
  BatchClass &bc = P->classes[cls];
  Packed *pk = reinterpret_cast<Packed *>(P->pks.data());
  std::vector<int> mem;
  for (int it = bc.item0; it < bc.item0 + bc.nitems; ++it) {
    const int j = P->items[it].x;
    if (mem.empty() || mem.back() != j) mem.push_back(j);
  }
  size_t smem = 0;
  for (int i : mem) {
    if (phasor == 2 && !global_phases_ok<Model>(pk[i]))
      return fail(CMC_ERR_UNSUPPORTED, "batch: a job of the class has no global phase regions");
    Packed q = pk[i];
    q.phasor = phasor;
    smem = std::max(smem, plan_bytes<Model>(P->jobs[i], q, R, T, 1));
  }
  if ((long long)smem > smem_optin())
    return fail(CMC_ERR_UNSUPPORTED, "batch: the class's shared memory does not fit this shape");
  const int G = nbeta / R;
  const int cap = dispatch_R<Model>(R, [&](auto rcn) {
    return batch_capacity<Model, decltype(rcn)::value>(G, T, smem);
  });
  if (cap <= 0) return fail(CMC_ERR_UNSUPPORTED, "batch: no cluster of this shape is resident");
  bc.R = R; bc.G = G; bc.T = T; bc.phasor = phasor; bc.smem = smem;
  bc.nclusters = std::min(cap, bc.nitems);
  for (int i : mem) pk[i].phasor = phasor;
  CMC_CUDA(cudaMemcpyAsync(P->pks_dev, P->pks.data(), P->pks.size(), cudaMemcpyHostToDevice, s));
  CMC_CUDA(cudaStreamSynchronize(s));
  return CMC_OK;
}

// ---- the reference's host-pointer entry points ------------------------------

// One device allocation carved into 256-byte aligned pieces.
struct Arena {
  size_t off = 0;
  unsigned char *base = nullptr;
  size_t take(size_t bytes)
  {
    size_t o = off;
    off += (bytes + 255) & ~(size_t)255;
    return o;
  }
  template <class T>
  T *at(size_t o) const { return reinterpret_cast<T *>(base + o); }
};

template <class T>
inline int h2d(T *dst, const T *src, size_t n, cudaStream_t s)
{
  if (n == 0 || src == nullptr) return CMC_OK;
  CMC_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyHostToDevice, s));
  return CMC_OK;
}

template <class T>
inline int d2h(T *dst, const T *src, size_t n, cudaStream_t s)
{
  if (n == 0 || dst == nullptr) return CMC_OK;
  CMC_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyDeviceToHost, s));
  return CMC_OK;
}

struct DevBuf {
  void *p = nullptr;
  cudaStream_t s = nullptr;
  ~DevBuf()
  {
    if (p) cudaFreeAsync(p, s);
  }
};

// The device memory pool of the host-buffer entry points (mcmc_cuda and co.):
// one per device, created by the first call on it, whose freed blocks stay
// reserved for the next call (release threshold unlimited), so that repeated
// calls do not map and unmap their device arrays each time.  The pool keeps
// the largest call's footprint until the process exits.
inline int host_api_pool(cudaMemPool_t *out)
{
  constexpr int kMaxDev = 64;
  static std::mutex mu;
  static cudaMemPool_t pools[kMaxDev] = {};
  int dev = 0;
  CMC_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDev) return fail(CMC_ERR_ARG, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(mu);
  if (!pools[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t p = nullptr;
    CMC_CUDA(cudaMemPoolCreate(&p, &props));
    unsigned long long keep = ~0ull;   // the attribute's value type is a 64-bit unsigned
    CMC_CUDA(cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep));
    pools[dev] = p;
  }
  *out = pools[dev];
  return CMC_OK;
}

inline cudaError_t host_api_alloc(void **p, size_t bytes, cudaStream_t s)
{
  cudaMemPool_t pool = nullptr;
  if (host_api_pool(&pool) != CMC_OK) return cudaErrorMemoryAllocation;
  return cudaMallocFromPoolAsync(p, bytes, pool, s);
}

inline int read_status(const int *dstatus, cudaStream_t s, int *out)
{
  CMC_CUDA(cudaMemcpyAsync(out, dstatus, sizeof(int), cudaMemcpyDeviceToHost, s));
  CMC_CUDA(cudaStreamSynchronize(s));
  return CMC_OK;
}

inline const char *status_text(int st)
{
  switch (st) {
    case CMC_ERR_ARG: return "invalid input detected on the device (e.g. a closure index out of range)";
    case CMC_ERR_STREAM: return "an injected random stream ran out";
    case CMC_ERR_MODEL: return "the model reported an error";
    default: return "device error";
  }
}

template <class Model>
int host_mcmc(float *coor, float *dat, float *std2r, int *icoor, int *idat, float *datm,
              float *chi2m, int *pdescr, int *ivar, int *invar, float *ptotal, float *pmint,
              float *pmaxt, float *pout, int *tout, float *chi2, float *chi2c, int *tcur,
              int *flag, int *n_acpt, int *n_exch, int *n_cnt, int *n_hist, float *beta,
              float *pstp, float *ptent, int *ptentn, float *pcur, unsigned char *rndst,
              unsigned long long seed, int imodel, int ncoor, int ndat, int nicoor, int nidat,
              int ndatm, int nptot, int nprm, int nadj, int npass, int nbeta, int nseq,
              int nburn, int niter)
{
  (void)ptotal;
  if (!coor || !dat || !std2r || !idat || !datm || !chi2m || !pdescr || !ivar || !invar ||
      !pmint || !pmaxt || !chi2c || !tcur || !flag || !n_acpt || !n_exch || !n_cnt ||
      !n_hist || !beta || !pstp || !ptent || !ptentn || !pcur || !rndst)
    return fail(CMC_ERR_ARG, "mcmc_cuda: a required array pointer is NULL");
  if (niter > 0 && (!pout || !tout || !chi2))
    return fail(CMC_ERR_ARG, "mcmc_cuda: pout, tout and chi2 are required when niter > 0");
  if (nptot < 1 || nprm < 1 || nprm > nptot || nbeta < 2 || nseq < 1 || ndat < 1 ||
      nadj < 1 || npass < 1 || nburn < 0 || niter < 0 || nidat < 1 || ncoor < 0 || nicoor < 0)
    return fail(CMC_ERR_ARG, "mcmc_cuda: invalid sizes");
  for (int k = 0; k < nprm; ++k) {
    if (ivar[k] < 0 || ivar[k] >= nptot || invar[ivar[k]] != k)
      return fail(CMC_ERR_ARG, "mcmc_cuda: ivar/invar are not inverse maps of the mutable "
                               "parameters (ivar[k] in [0,nptot), invar[ivar[k]] == k)");
  }
  const size_t nrep = (size_t)nbeta * nseq;
  cudaStream_t s = cudaStreamPerThread;

  cmc_job j;
  std::memset(&j, 0, sizeof(j));
  j.ncoor = ncoor; j.ndat = ndat; j.nicoor = nicoor; j.nidat = nidat; j.ndatm = ndatm;
  j.nptot = nptot; j.nprm = nprm; j.nadj = nadj; j.npass = npass; j.nbeta = nbeta;
  j.nseq = nseq; j.imodel = imodel;
  j.do_init = 1; j.nburn = nburn; j.niter = niter; j.itr0 = 0; j.niter_total = niter;
  j.rng_mode = CMC_RNG_CURAND; j.seed = seed;
  for (int i = 0; i < 4; ++i) j.hidat[i] = i < nidat ? idat[i] : 0;

  Arena a;
  const size_t o_coor = a.take(4 * (size_t)ncoor), o_dat = a.take(4 * (size_t)ndat),
               o_std = a.take(4 * (size_t)ndat), o_icoor = a.take(4 * (size_t)std::max(nicoor, 1)),
               o_idat = a.take(4 * (size_t)nidat), o_datm = a.take(4 * (size_t)ndatm),
               o_chi2m = a.take(4 * nrep * ndat), o_pdescr = a.take(4 * (size_t)nptot),
               o_ivar = a.take(4 * (size_t)nprm), o_invar = a.take(4 * (size_t)nptot),
               o_pmin = a.take(4 * (size_t)nptot), o_pmax = a.take(4 * (size_t)nptot),
               o_pout = a.take(4 * (size_t)nprm * nrep * niter), o_tout = a.take(4 * nrep * niter),
               o_chi2 = a.take(4 * (size_t)nseq * niter), o_chi2c = a.take(4 * nrep),
               o_tcur = a.take(4 * nrep), o_flag = a.take(4 * nrep),
               o_nacpt = a.take(4 * nprm * nrep), o_nexch = a.take(4 * nrep),
               o_ncnt = a.take(4 * nprm * nrep), o_nhist = a.take(4 * (size_t)nadj * nprm * nrep),
               o_beta = a.take(4 * (size_t)nbeta), o_pstp = a.take(4 * nprm * nrep),
               o_ptent = a.take(4 * nrep), o_ptentn = a.take(4 * nrep),
               o_pcur = a.take(4 * nrep * nptot), o_rndst = a.take(48 * nrep),
               o_status = a.take(16);
  // model scratch, sized with the final device pointers unknown yet: dims only
  {
    cmc_job probe = j;
    probe.datm = reinterpret_cast<float *>(16);
    probe.chi2m = reinterpret_cast<float *>(16);
    j.work_bytes = work_bytes<Model>(probe, 0);
  }
  const size_t o_work = a.take(j.work_bytes);

  DevBuf buf;
  buf.s = s;
  {
    cudaError_t e = host_api_alloc(&buf.p, a.off, s);
    if (e != cudaSuccess) {
      buf.p = nullptr;
      return fail(CMC_ERR_NOMEM, std::string("mcmc_cuda: device allocation failed: ") +
                                     cudaGetErrorString(e));
    }
  }
  a.base = (unsigned char *)buf.p;
  j.coor = a.at<float>(o_coor); j.dat = a.at<float>(o_dat); j.std2r = a.at<float>(o_std);
  j.icoor = a.at<int>(o_icoor); j.idat = a.at<int>(o_idat);
  j.datm = a.at<float>(o_datm); j.chi2m = a.at<float>(o_chi2m);
  j.pdescr = a.at<int>(o_pdescr); j.ivar = a.at<int>(o_ivar); j.invar = a.at<int>(o_invar);
  j.pmint = a.at<float>(o_pmin); j.pmaxt = a.at<float>(o_pmax);
  j.pout = a.at<float>(o_pout); j.tout = a.at<int>(o_tout); j.chi2 = a.at<float>(o_chi2);
  j.chi2c = a.at<float>(o_chi2c); j.tcur = a.at<int>(o_tcur); j.flag = a.at<int>(o_flag);
  j.n_acpt = a.at<int>(o_nacpt); j.n_exch = a.at<int>(o_nexch); j.n_cnt = a.at<int>(o_ncnt);
  j.n_hist = a.at<int>(o_nhist); j.beta = a.at<float>(o_beta); j.pstp = a.at<float>(o_pstp);
  j.ptent = a.at<float>(o_ptent); j.ptentn = a.at<int>(o_ptentn); j.pcur = a.at<float>(o_pcur);
  j.rndst = a.at<unsigned char>(o_rndst); j.status = a.at<int>(o_status);
  j.work = j.work_bytes ? (void *)a.at<unsigned char>(o_work) : nullptr;

  int rc = CMC_OK;
#define CMC_TRY(x) do { if ((rc = (x)) != CMC_OK) return rc; } while (0)
  CMC_TRY(h2d(const_cast<float *>(j.coor), coor, ncoor, s));
  CMC_TRY(h2d(const_cast<float *>(j.dat), dat, ndat, s));
  CMC_TRY(h2d(const_cast<float *>(j.std2r), std2r, ndat, s));
  CMC_TRY(h2d(const_cast<int *>(j.icoor), icoor, nicoor, s));
  CMC_TRY(h2d(const_cast<int *>(j.idat), idat, nidat, s));
  if (Model::kRowsInEval) {   // a plugin's chi^2 sums whole chi2m rows
    CMC_TRY(h2d(j.datm, datm, ndatm, s));
    CMC_TRY(h2d(j.chi2m, chi2m, nrep * ndat, s));
  }
  CMC_TRY(h2d(const_cast<int *>(j.pdescr), pdescr, nptot, s));
  CMC_TRY(h2d(const_cast<int *>(j.ivar), ivar, nprm, s));
  CMC_TRY(h2d(const_cast<int *>(j.invar), invar, nptot, s));
  CMC_TRY(h2d(const_cast<float *>(j.pmint), pmint, nptot, s));
  CMC_TRY(h2d(const_cast<float *>(j.pmaxt), pmaxt, nptot, s));
  CMC_TRY(h2d(j.tcur, tcur, nrep, s));
  CMC_TRY(h2d(j.flag, flag, nrep, s));
  CMC_TRY(h2d(j.chi2c, chi2c, nrep, s));
  CMC_TRY(h2d(j.n_acpt, n_acpt, nprm * nrep, s));
  CMC_TRY(h2d(j.n_exch, n_exch, nrep, s));
  CMC_TRY(h2d(j.n_cnt, n_cnt, nprm * nrep, s));
  CMC_TRY(h2d(j.n_hist, n_hist, (size_t)nadj * nprm * nrep, s));
  CMC_TRY(h2d(const_cast<float *>(j.beta), beta, nbeta, s));
  CMC_TRY(h2d(j.pstp, pstp, nprm * nrep, s));
  CMC_TRY(h2d(j.ptent, ptent, nrep, s));
  CMC_TRY(h2d(j.ptentn, ptentn, nrep, s));
  CMC_TRY(h2d(j.pcur, pcur, nrep * nptot, s));
  // the generator states go in as well (src/mcmcjob.cu:724): curand_init
  // rewrites their fields and leaves the padding bytes as the caller's
  CMC_TRY(h2d(j.rndst, rndst, 48 * nrep, s));
  CMC_CUDA(cudaMemsetAsync(j.status, 0, sizeof(int), s));

  CMC_TRY(run_sweep<Model>(j, s));

  CMC_TRY(d2h(rndst, j.rndst, 48 * nrep, s));
  CMC_TRY(d2h(pout, j.pout, (size_t)nprm * nrep * niter, s));
  CMC_TRY(d2h(tout, j.tout, nrep * niter, s));
  CMC_TRY(d2h(chi2, j.chi2, (size_t)nseq * niter, s));
  CMC_TRY(d2h(tcur, j.tcur, nrep, s));
  CMC_TRY(d2h(n_acpt, j.n_acpt, nprm * nrep, s));
  CMC_TRY(d2h(n_cnt, j.n_cnt, nprm * nrep, s));
  CMC_TRY(d2h(n_exch, j.n_exch, nrep, s));
  CMC_TRY(d2h(n_hist, j.n_hist, (size_t)nadj * nprm * nrep, s));
  CMC_TRY(d2h(pstp, j.pstp, nprm * nrep, s));
  CMC_TRY(d2h(ptent, j.ptent, nrep, s));
  CMC_TRY(d2h(ptentn, j.ptentn, nrep, s));
  CMC_TRY(d2h(pcur, j.pcur, nrep * nptot, s));
  CMC_TRY(d2h(flag, j.flag, nrep, s));
  CMC_TRY(d2h(chi2c, j.chi2c, nrep, s));
  CMC_TRY(d2h(datm, j.datm, (size_t)ndatm, s));
  CMC_TRY(d2h(chi2m, j.chi2m, nrep * ndat, s));
  int st = 0;
  CMC_TRY(read_status(j.status, s, &st));
#undef CMC_TRY
  if (st) return fail(st, std::string("mcmc_cuda: ") + status_text(st));
  return CMC_OK;
}

template <class Model>
int host_eval(int mode, float *coor, float *dat, float *std2r, int *icoor, int *idat,
              float *datm, float *chi2m, float *pcur, float *chi2c, int *flag, int imodel,
              int ncoor, int ndat, int nicoor, int nidat, int ndatm, int nptot, int nbeta,
              int nseq)
{
  if (!coor || !idat || !datm || !pcur || (mode == 1 && (!dat || !std2r || !chi2m || !chi2c)))
    return fail(CMC_ERR_ARG, "a required array pointer is NULL");
  if (nptot < 1 || nbeta < 1 || nseq < 1 || ndat < 1 || nidat < 1 || ncoor < 0 || nicoor < 0 ||
      ndatm < 0)
    return fail(CMC_ERR_ARG, "invalid sizes");
  const size_t nrep = (size_t)nbeta * nseq;
  cudaStream_t s = cudaStreamPerThread;
  cmc_job j;
  std::memset(&j, 0, sizeof(j));
  j.ncoor = ncoor; j.ndat = ndat; j.nicoor = nicoor; j.nidat = nidat; j.ndatm = ndatm;
  j.nptot = nptot; j.nbeta = nbeta; j.nseq = nseq; j.imodel = imodel; j.npass = 2;
  for (int i = 0; i < 4; ++i) j.hidat[i] = i < nidat ? idat[i] : 0;
  Arena a;
  const size_t o_coor = a.take(4 * (size_t)ncoor), o_dat = a.take(4 * (size_t)ndat),
               o_std = a.take(4 * (size_t)ndat), o_icoor = a.take(4 * (size_t)std::max(nicoor, 1)),
               o_idat = a.take(4 * (size_t)nidat), o_datm = a.take(4 * (size_t)std::max(ndatm, 1)),
               o_chi2m = a.take(4 * nrep * ndat), o_pcur = a.take(4 * nrep * nptot),
               o_chi2c = a.take(4 * nrep), o_flag = a.take(4 * nrep), o_status = a.take(16);
  {
    cmc_job probe = j;
    probe.datm = reinterpret_cast<float *>(16);
    probe.chi2m = reinterpret_cast<float *>(16);
    j.work_bytes = work_bytes<Model>(probe, mode);
  }
  const size_t o_work = a.take(j.work_bytes);
  DevBuf buf;
  buf.s = s;
  if (host_api_alloc(&buf.p, a.off, s) != cudaSuccess) {
    buf.p = nullptr;
    return fail(CMC_ERR_NOMEM, "device allocation failed");
  }
  a.base = (unsigned char *)buf.p;
  j.coor = a.at<float>(o_coor); j.dat = a.at<float>(o_dat); j.std2r = a.at<float>(o_std);
  j.icoor = a.at<int>(o_icoor); j.idat = a.at<int>(o_idat); j.datm = a.at<float>(o_datm);
  j.chi2m = a.at<float>(o_chi2m); j.pcur = a.at<float>(o_pcur); j.chi2c = a.at<float>(o_chi2c);
  j.flag = a.at<int>(o_flag); j.status = a.at<int>(o_status);
  j.work = j.work_bytes ? (void *)a.at<unsigned char>(o_work) : nullptr;
  int rc = CMC_OK;
#define CMC_TRY(x) do { if ((rc = (x)) != CMC_OK) return rc; } while (0)
  CMC_TRY(h2d(const_cast<float *>(j.coor), coor, ncoor, s));
  CMC_TRY(h2d(const_cast<int *>(j.idat), idat, nidat, s));
  CMC_TRY(h2d(j.pcur, pcur, nrep * nptot, s));
  CMC_TRY(h2d(j.datm, datm, (size_t)ndatm, s));
  if (mode == 1) {
    CMC_TRY(h2d(const_cast<float *>(j.dat), dat, ndat, s));
    CMC_TRY(h2d(const_cast<float *>(j.std2r), std2r, ndat, s));
    CMC_TRY(h2d(const_cast<int *>(j.icoor), icoor, nicoor, s));
    CMC_TRY(h2d(j.chi2m, chi2m, nrep * ndat, s));
    CMC_TRY(h2d(j.chi2c, chi2c, nrep, s));
  }
  if (flag && mode == 1) {
    CMC_TRY(h2d(j.flag, flag, nrep, s));
  } else {
    // calc_model: the reference leaves flag uninitialised (src/mcmcjob.cu:269);
    // every parameter set is evaluated here.
    CMC_CUDA(cudaMemsetAsync(j.flag, 0, 4 * nrep, s));
    j.flag = nullptr;
  }
  CMC_CUDA(cudaMemsetAsync(j.status, 0, sizeof(int), s));
  CMC_TRY(run_eval<Model>(j, mode, s));
  CMC_TRY(d2h(datm, j.datm, (size_t)ndatm, s));
  if (mode == 1) {
    CMC_TRY(d2h(chi2m, j.chi2m, nrep * ndat, s));
    CMC_TRY(d2h(chi2c, j.chi2c, nrep, s));
  }
  int st = 0;
  CMC_TRY(read_status(j.status, s, &st));
#undef CMC_TRY
  if (st) return fail(st, status_text(st));
  return CMC_OK;
}

}  // namespace cmc
