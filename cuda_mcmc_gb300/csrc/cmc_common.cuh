// cmc_common.cuh -- pieces shared by the sweep and evaluation kernels and by
// the host layer: the random source, the shared-memory plan, the per-CTA view.
//
// The sweep they serve (cmc_sweep.cuh), in brief:
//
// Work decomposition on the GPU:
//   * one thread-block CLUSTER per sequence iseq; its G CTAs own R = nbeta/G
//     temperatures each (CTA rank c owns ibeta in [c*R, (c+1)*R));
//   * thread r < R of a CTA owns replica r: its RNG state, its proposal,
//     its Metropolis decision and its step-size adaptation;
//   * every thread of the CTA evaluates the model for all R replicas over a
//     strided share of the data; per-replica chi^2 partials are reduced with
//     warp shuffles and a fixed-order shared-memory pass (deterministic);
//   * the replica exchange of a sequence runs on warp 0 of cluster rank 0,
//     with the ibeta = 0 replica's generator, over chi^2 values gathered from
//     the other CTAs through distributed shared memory; the winning
//     permutation is then applied by every CTA pulling its new parameter
//     rows from their owners (DSMEM), between cluster barriers.
// The spread layout (cmc_sweep.cuh) instead shares all replicas evenly among
// the CTAs of one cooperative launch, R or R-1 each, and runs each
// sequence's exchange on the CTA holding its ibeta = 0 replica through
// global memory.
//
// The algorithm is the reference's (src/gpu_mcmc.cu):
//   init_rng :228-239, init_pcur :245-267, gen_proposal :361-411,
//   calc_chi2_terms/calc_chi2 :273-350, spmp_mcmc :426-474,
//   adjust_steps :480-526, replica_exchange :533-626, run_mcmc :682-763,
// with the same per-replica order of random draws, so that with the same
// seed it walks the same chains (cuRAND XORWOW, curand_init(seed, ist, 0)).
#pragma once
#include <cooperative_groups.h>
#include <cstring>
#include <cuda_runtime.h>
#include <curand_kernel.h>

#include "cmc_job.h"

namespace cmc {
namespace cg = cooperative_groups;

// main iterations staged in shared memory per record flush
#ifndef CMC_KCH
#define CMC_KCH 32
#endif
constexpr int kCH = CMC_KCH;
constexpr int kMaxThreads = 256;
constexpr int kRepF = 4;         // per-replica floats: ptent, chi2c, chi2n, beta
constexpr int kRepI = 4;         // per-replica ints: ptentn, flag, kchosen, evaluated
constexpr int kMaxRetry = 64;    // bound on the k-redraw loops (u == 1.0 exactly)

// Angle wrapped into [-pi, pi], the value of the reference's atan2(sin p,
// cos p) (src/gpu_mcmc.cu:389-393): p - 2 pi n with n = rint(p / (2 pi)),
// in double precision and rounded once to float, i.e. the float nearest the
// exact wrap (the reference's float sin / cos / atan2 come within an ulp or
// two of it).  A short fixed sequence (multiply, rint, fma, conversion) with
// nothing left to contraction, so every kernel rounds it identically.
__device__ __forceinline__ float wrap_pi(float p)
{
  const double x = (double)p;
  const double n = rint(x * 0.15915494309189533577);
  return (float)fma(-6.283185307179586477, n, x);
}

__device__ __forceinline__ void set_status(int *st, int code)
{
  if (st) atomicCAS(st, 0, code);
}

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// One replica's random source: the reference's cuRAND XORWOW state, or an
// injected stream pair with cursors.
struct Rng {
  curandStateXORWOW st;
  unsigned pad;   // bytes 36-39 of the stored 48-byte state (padding before the double)
  const float *u, *n;
  int cu, cn, lu, ln;
  bool inj;
  bool ovf;

  // The stored state, word by word: the fields (d, v[5], the Box-Muller
  // flags and cached values), then the 4 padding bytes and the cached
  // double.  The reference runs curand_init on its device copy of the
  // caller's array and copies the array back, so the padding keeps the
  // caller's bytes: they are read and written back unchanged here.
  __device__ void store_state(unsigned char *p) const
  {
    unsigned *w = reinterpret_cast<unsigned *>(p);
    w[0] = st.d;
#pragma unroll
    for (int i = 0; i < 5; ++i) w[1 + i] = st.v[i];
    w[6] = (unsigned)st.boxmuller_flag;
    w[7] = (unsigned)st.boxmuller_flag_double;
    w[8] = __float_as_uint(st.boxmuller_extra);
    w[9] = pad;
    const unsigned long long e = (unsigned long long)__double_as_longlong(st.boxmuller_extra_double);
    w[10] = (unsigned)e;
    w[11] = (unsigned)(e >> 32);
  }

  __device__ float uniform()
  {
    if (inj) {
      if (cu < lu) return u[cu++];
      ovf = true;
      return 0.5f;
    }
    return curand_uniform(&st);
  }
  __device__ float normal()
  {
    if (inj) {
      if (cn < ln) return n[cn++];
      ovf = true;
      return 0.0f;
    }
    return curand_normal(&st);
  }
  // Index in [0, n) drawn as (int)(n*u), redrawn while it equals n
  // (curand_uniform can return exactly 1.0), src/gpu_mcmc.cu:369-372.
  __device__ int index(int n, int *status)
  {
    for (int t = 0; t < kMaxRetry; ++t) {
      int k = (int)((float)n * uniform());
      if (k < n) return k;
    }
    set_status(status, CMC_ERR_STREAM);
    return n - 1;
  }
};

// Copy of lane `src`'s value of a trivially copyable object on every lane of
// the (fully active) warp, word by word.
template <class V>
__device__ __forceinline__ V warp_broadcast(const V &v, int src)
{
  static_assert(sizeof(V) % 4 == 0, "warp_broadcast: size must be a multiple of 4 bytes");
  constexpr int kW = (int)(sizeof(V) / 4);
  int w[kW];
  memcpy(w, &v, sizeof(V));
#pragma unroll
  for (int i = 0; i < kW; ++i) w[i] = __shfl_sync(0xffffffffu, w[i], src);
  V out;
  memcpy(&out, w, sizeof(V));
  return out;
}

__host__ __device__ inline unsigned align16(unsigned x) { return (x + 15u) & ~15u; }

// Shared-memory plan of one CTA; the same function sizes the launch on the
// host and carves the buffer on the device.  `hist` holds the burn-in
// accept/reject history n_hist as one bit per entry: [R][nprm][hist_words(nadj)].
struct SmemPlan {
  unsigned params, plast, ptmp, blk, rf, ri, sf, si, hist, tab, consts, red, xch, stage,
      scratch, total;
};

__host__ __device__ inline int hist_words(int nadj) { return (nadj + 31) / 32; }

__host__ __device__ inline SmemPlan make_plan(int R, int nthreads, int nptot, int nprm,
                                              int nbeta, int nadj, unsigned consts_bytes,
                                              unsigned scratch_bytes)
{
  SmemPlan p;
  unsigned o = 0;
  p.params = o;  o = align16(o + 4u * R * nptot);
  p.plast = o;   o = align16(o + 4u * R * nptot);
  p.ptmp = o;    o = align16(o + 4u * (R * nptot + R));
  p.blk = o;     o = align16(o + 4u * R * nptot);
  p.rf = o;      o = align16(o + 4u * R * kRepF);
  p.ri = o;      o = align16(o + 4u * R * kRepI);
  p.sf = o;      o = align16(o + 4u * R * nprm);
  p.si = o;      o = align16(o + 4u * R * nprm * 4);
  p.hist = o;    o = align16(o + 4u * R * nprm * hist_words(nadj));
  p.tab = o;     o = align16(o + 4u * (nprm + 3 * nptot));
  p.consts = o;  o = align16(o + consts_bytes * R);
  p.red = o;     o = align16(o + 4u * R * (nthreads / 32));
  p.xch = o;     o = align16(o + 4u * 5 * nbeta);
  p.stage = o;   o = align16(o + 4u * (R * nprm * kCH + nbeta * kCH + kCH));
  p.scratch = o; o = align16(o + scratch_bytes);
  p.total = o;
  return p;
}

// ---- spread layout (cmc_sweep.cuh): host and device arithmetic ------------

// CTA b of N over nrep replicas: first replica and count (nrep >= N).
__host__ __device__ inline void spread_range(int nrep, int N, int b, int &start, int &cnt)
{
  const int q = nrep / N, rem = nrep % N;
  cnt = q + (b < rem ? 1 : 0);
  start = b * q + (b < rem ? b : rem);
}

// The CTA holding replica f (inverse of spread_range).
__host__ __device__ inline int spread_cta_of(int nrep, int N, int f)
{
  const int q = nrep / N, rem = nrep % N, big = rem * (q + 1);
  return f < big ? f / (q + 1) : rem + (f - big) / q;
}

// Sequence group g of ngroups: sequences [seq0, seq0 + n), the first
// nseq % ngroups groups one sequence larger.  A spread launch runs its groups
// one after the other on all of its CTAs (only one group's phase regions in
// use at a time).
__host__ __device__ inline void spread_group(int nseq, int ngroups, int g, int &seq0, int &n)
{
  const int q = nseq / ngroups, rem = nseq % ngroups;
  n = q + (g < rem ? 1 : 0);
  seq0 = g * q + (g < rem ? g : rem);
}

// Global-memory exchange area of a spread launch (in job.work after the
// model's scratch; spread_ctl_bytes).  The per-iteration buffers are double
// buffered by iteration parity: a CTA rewrites a buffer two iterations later,
// after every reader of the sequence has arrived at the iteration between.
struct SpreadCtl {
  int *arrive;   // [nseq] CTAs that published this launch's iterations (zeroed per launch)
  int *done;     // [nseq] exchanges completed this launch
  int *abort;    // [1] set when a wait ran out: every CTA stops waiting
  float *xp;     // [2][nrep][nptot] parameters before the exchange
  float *xc;     // [2][nrep] chi^2 before the exchange
  int *xperm;    // [2][nrep] source temperature of each slot after the exchange
  float *xchi;   // [2][nrep] chi^2 after the exchange
  int hold;      // test hook: the owner of this sequence never completes its
                 // exchange, so that every wait runs out (-1: none; set from
                 // the environment variable CMC_SPREAD_HOLD_SEQ)
  int ngroups;   // sequence groups run one after the other (spread_group)
};

__host__ __device__ inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Bytes of the SpreadCtl area; the counters (first block) are zeroed before
// every launch.
__host__ __device__ inline size_t spread_ctl_counter_bytes(int nseq)
{
  return align256(4 * (2 * (size_t)nseq + 1));
}
__host__ __device__ inline size_t spread_ctl_bytes(int nseq, int nbeta, int nptot)
{
  const size_t nrep = (size_t)nseq * nbeta;
  return spread_ctl_counter_bytes(nseq) + align256(4 * 2 * nrep * nptot) + 3 * align256(4 * 2 * nrep);
}
__host__ __device__ inline SpreadCtl spread_ctl_at(unsigned char *base, int nseq, int nbeta,
                                                   int nptot)
{
  const size_t nrep = (size_t)nseq * nbeta;
  SpreadCtl c;
  c.arrive = reinterpret_cast<int *>(base);
  c.done = c.arrive + nseq;
  c.abort = c.done + nseq;
  size_t o = spread_ctl_counter_bytes(nseq);
  c.xp = reinterpret_cast<float *>(base + o);  o += align256(4 * 2 * nrep * nptot);
  c.xc = reinterpret_cast<float *>(base + o);  o += align256(4 * 2 * nrep);
  c.xperm = reinterpret_cast<int *>(base + o); o += align256(4 * 2 * nrep);
  c.xchi = reinterpret_cast<float *>(base + o);
  c.hold = -1;
  c.ngroups = 1;
  return c;
}

// Per-CTA view handed to the model policies.
template <class Model, int R>
struct Cta {
  const cmc_job *job;
  const typename Model::Packed *pk;
  typename Model::Consts *consts;   // [R]
  const int *flag;                  // [R]
  float *scratch;
  int ist[R];                       // global replica index of each local replica
  int tid, nthreads;
  int ph_region;                    // first of R consecutive per-replica regions of a
                                    // global model scratch (disjoint between CTAs)
  int model_i;                      // one int and one float a model may cache at
  float model_f;                    // setup (read once per launch, held in registers)
};


template <class Model, int R>
__device__ __forceinline__ void block_reduce(float (&acc)[R], float *red, int tid, int nw)
{
  const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    float v = warp_sum(acc[r]);
    if (lane == 0) red[r * nw + warp] = v;
  }
}

}  // namespace cmc
