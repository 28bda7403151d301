// cmc_sweep.cuh -- the fused MCMC-RE sweep kernels (one launch per run).
// The work decomposition and the reference functions it restates are
// described at the top of cmc_common.cuh.
#pragma once
#include <cuda/atomic>

#include "cmc_common.cuh"

namespace cmc {

// Minimum resident CTAs per SM the register allocation is sized for
// (ptxas: 65536 / (kMaxThreads * CMC_MIN_BLOCKS) registers per thread).
#ifndef CMC_MIN_BLOCKS
#define CMC_MIN_BLOCKS 2
#endif

// ---- replica layouts ----------------------------------------------------------
// Which replicas the R local slots of a CTA hold, and who runs the exchange.

// Cluster layout: the G = nbeta/R CTAs of a cluster run one sequence; slot r
// of cluster rank k is temperature k*R + r; the exchange runs on rank 0 over
// distributed shared memory.
template <int R>
struct ClusterLayout {
  static constexpr bool kSpread = false;
  int rank, seq;
  __device__ __forceinline__ bool active(int) const { return true; }
  __device__ __forceinline__ int ibeta(int r) const { return rank * R + r; }
  __device__ __forceinline__ int iseq(int) const { return seq; }
  __device__ __forceinline__ bool owner() const { return rank == 0; }
  __device__ __forceinline__ int own_seq() const { return seq; }
  __device__ __forceinline__ int ph_region(int nbeta) const { return seq * nbeta + rank * R; }
};

// Spread layout: the N CTAs of a cooperative launch (all resident at once)
// share the replicas evenly, sequence-major (replica f = iseq*nbeta +
// ibeta): CTA b holds f in [gstart, gstart + cnt) with cnt = nrep/N or one
// more (spread_range), so
// that no SM holds more than ceil(N/SMs) CTAs' worth, whatever nseq is (64 x
// 32 replicas on 152 SMs: 293 CTAs of 6-7 replicas instead of 256 clusters'
// CTAs of 8 on some SMs and 0 on others).  With R <= nbeta a CTA spans at
// most two sequences and holds at most one sequence's ibeta = 0 replica,
// whose generator draws that sequence's exchange; that CTA (the owner) runs
// the exchange through global memory.
struct SpreadLayout {
  static constexpr bool kSpread = true;
  int gstart, cnt, nbeta;
  int seq_lo, seq_hi;   // sequences held (seq_hi is seq_lo or seq_lo + 1)
  int own, own_r;       // owned sequence (or -1) and the local slot of its ibeta 0
  int own_ncta;         // CTAs holding replicas of the owned sequence
  int region0;          // first of the CTA's global phase regions
  __device__ __forceinline__ bool active(int r) const { return r < cnt; }
  __device__ __forceinline__ int ibeta(int r) const { return (gstart + r) % nbeta; }
  __device__ __forceinline__ int iseq(int r) const { return (gstart + r) / nbeta; }
  __device__ __forceinline__ bool owner() const { return own >= 0; }
  __device__ __forceinline__ int own_seq() const { return own; }
  __device__ __forceinline__ int own_slot() const { return own_r; }
  __device__ __forceinline__ int ph_region(int) const { return region0; }
};

// CTA b of N spreading the nseq sequences from seq0 on (nbeta replicas each);
// replica and sequence indices are the job's.
__host__ __device__ __forceinline__ SpreadLayout make_spread_layout(int nbeta, int seq0, int nseq,
                                                                    int N, int b, int region0)
{
  const int nrep = nbeta * nseq;
  SpreadLayout lay;
  int start = 0;
  spread_range(nrep, N, b, start, lay.cnt);
  start += seq0 * nbeta;
  lay.nbeta = nbeta;
  lay.gstart = start;
  lay.seq_lo = start / nbeta;
  lay.seq_hi = (start + lay.cnt - 1) / nbeta;
  lay.own = -1;
  lay.own_r = 0;
  if (start % nbeta == 0) {
    lay.own = lay.seq_lo;
  } else if (lay.seq_hi > lay.seq_lo) {
    lay.own = lay.seq_hi;
    lay.own_r = lay.seq_hi * nbeta - start;
  }
  lay.own_ncta = 0;
  if (lay.own >= 0)
    lay.own_ncta = spread_cta_of(nrep, N, (lay.own - seq0) * nbeta + nbeta - 1) - b + 1;
  lay.region0 = region0;
  return lay;
}

// Waits until *flag >= target (acquire).  The first kSpinFast polls follow
// each other directly (the waits of an exchange last microseconds; sleeping
// between polls cost 2 % of the 64 x 32 sweep's time in a 32 ns - 1 us
// back-off), later ones 256 ns apart.  Bounded: after kSpinLimit polls (about
// a second) it sets the abort flag and CMC_ERR_TIMEOUT and returns false; it
// also returns false as soon as another CTA has aborted.
constexpr unsigned kSpinFast = 4096;
constexpr unsigned kSpinLimit = 1u << 20;
__device__ __forceinline__ bool spin_until_geq(int *flag, int target, int *abort, int *status)
{
  cuda::atomic_ref<int, cuda::thread_scope_device> f(*flag), a(*abort);
  for (unsigned n = 0; n < kSpinLimit; ++n) {
    if (f.load(cuda::memory_order_acquire) >= target) return true;
    if (a.load(cuda::memory_order_relaxed) != 0) return false;
    if (n >= kSpinFast) __nanosleep(256);
  }
  a.store(1, cuda::memory_order_relaxed);
  set_status(status, CMC_ERR_TIMEOUT);
  return false;
}

// replica_exchange (src/gpu_mcmc.cu:533-626) for nbeta <= 32 on warp 0 of
// the exchange owner: slot s on lane s, chi^2 (`chi`, each lane's on entry),
// tcur, owner and n_exch in registers, swaps by shuffles.  Every lane runs a
// copy of the ibeta = 0 replica's generator (held by thread `own_slot`; the
// same draws), so k and u are known warp-wide and the attempt loop has no
// shared-memory round trips; that thread keeps the advanced generator.  The
// results go to x_chi2 / x_tcur / x_perm / x_nexch.
__device__ __forceinline__ void warp_exchange(float chi, bool burn, Rng &rng, int own_slot,
                                              int nbeta, const float *x_beta, float *x_chi2,
                                              int *x_tcur, int *x_perm, int *x_nexch,
                                              int *status)
{
  const int lane = threadIdx.x & 31;
  const bool slot = lane < nbeta;
  const float bt = slot ? x_beta[lane] : 0.0f;
  int tc = slot ? x_tcur[lane] : 0, own = lane, nx = slot ? x_nexch[lane] : 0;
  Rng xr = warp_broadcast(rng, own_slot);
  const int nb1 = nbeta - 1;
  for (int ib = 0; ib < nbeta; ++ib) {
    const int k = xr.index(nb1, status);
    const float ck = __shfl_sync(0xffffffffu, chi, k);
    const float ck1 = __shfl_sync(0xffffffffu, chi, k + 1);
    const float bk = __shfl_sync(0xffffffffu, bt, k);
    const float bk1 = __shfl_sync(0xffffffffu, bt, k + 1);
    const int tk = __shfl_sync(0xffffffffu, tc, k), tk1 = __shfl_sync(0xffffffffu, tc, k + 1);
    const int ok = __shfl_sync(0xffffffffu, own, k), ok1 = __shfl_sync(0xffffffffu, own, k + 1);
    const float a = expf(-0.5f * (bk1 - bk) * (ck - ck1));
    const float alpha = (a < 1.0f) ? a : 1.0f;
    const float u = xr.uniform();
    if (u <= alpha) {
      if (lane == k) {
        chi = ck1; tc = tk1; own = ok1;
        if (!burn) nx += 1;
      } else if (lane == k + 1) {
        chi = ck; tc = tk; own = ok;
      }
    }
  }
  if (lane == own_slot) rng = xr;
  if (slot) {
    x_chi2[lane] = chi;
    x_tcur[lane] = tc;
    x_perm[lane] = own;
    x_nexch[lane] = nx;
  }
}

// ---- per-replica state of a CTA's R slots -------------------------------------

// Shared-memory views of a sweep CTA (make_plan) and the steps of the
// reference's per-replica kernels on one slot; slot r's steps run on the
// thread holding slot r's generator.  Layouts give each slot's (ibeta, iseq)
// and whether it is active (a spread CTA one replica short leaves its last
// slot empty: flag 0, never proposed, evaluated on zero constants).
template <class Model, int R>
struct SweepState {
  const cmc_job *job;
  int nbeta, nseq, nptot, nprm, nadj, HW, NW;
  bool block;
  float *params, *plast, *ptmp, *blk;   // [R][nptot] each (ptmp: + [R])
  float *s_ptent, *s_chi2c, *s_chi2n, *s_beta;
  int *s_ptentn, *s_flag, *s_k, *s_evald;
  float *s_pstp;                        // [R][nprm]
  int *s_ncnt, *s_nacpt;                // [R][nprm]
  int *s_hsum, *s_hslow;                // running history sum, 1: ring holds values other than 0/1
  unsigned *s_hbits;                    // [R][nprm][HW] history bits
  int *s_ivar, *s_pdescr;
  float *s_pmin, *s_pmax;
  typename Model::Consts *s_consts;     // [R]
  float *s_red;                         // [R][NW] chi^2 partials of the last evaluation
  float *x_chi2, *x_beta;               // exchange owner: [nbeta] each
  int *x_perm, *x_tcur, *x_nexch;
  float *st_p;                          // [R][nprm][kCH] staged pout rows
  int *st_t;                            // [nbeta][kCH] staged tout (exchange owner)
  float *st_c;                          // [kCH] staged chi2 (exchange owner)
  float *scratch;                       // model scratch

  __device__ void bind(const cmc_job &j, const SmemPlan &P, unsigned char *smem, int nw)
  {
    job = &j;
    nbeta = j.nbeta; nseq = j.nseq; nptot = j.nptot; nprm = j.nprm; nadj = j.nadj;
    HW = hist_words(nadj);
    NW = nw;
    block = (j.prop_mode == CMC_PROP_BLOCK);
    params = (float *)(smem + P.params);
    plast = (float *)(smem + P.plast);
    ptmp = (float *)(smem + P.ptmp);
    blk = (float *)(smem + P.blk);
    float *rf = (float *)(smem + P.rf);
    int *ri = (int *)(smem + P.ri);
    s_ptent = rf; s_chi2c = rf + R; s_chi2n = rf + 2 * R; s_beta = rf + 3 * R;
    s_ptentn = ri; s_flag = ri + R; s_k = ri + 2 * R; s_evald = ri + 3 * R;
    s_pstp = (float *)(smem + P.sf);
    s_ncnt = (int *)(smem + P.si);
    s_nacpt = s_ncnt + R * nprm;
    s_hsum = s_nacpt + R * nprm;
    s_hslow = s_hsum + R * nprm;
    s_hbits = (unsigned *)(smem + P.hist);
    s_ivar = (int *)(smem + P.tab);
    s_pdescr = s_ivar + nprm;
    s_pmin = (float *)(s_pdescr + nptot);
    s_pmax = s_pmin + nptot;
    s_consts = (typename Model::Consts *)(smem + P.consts);
    s_red = (float *)(smem + P.red);
    x_chi2 = (float *)(smem + P.xch);
    x_perm = (int *)(x_chi2 + nbeta);
    x_tcur = x_perm + nbeta;
    x_nexch = x_tcur + nbeta;
    x_beta = (float *)(x_nexch + nbeta);
    st_p = (float *)(smem + P.stage);
    st_t = (int *)(st_p + R * nprm * kCH);
    st_c = (float *)(st_t + nbeta * kCH);
    scratch = (float *)(smem + P.scratch);
  }

  // ---- loads (the CTA's threads tid of T) --------------------------------------
  __device__ void load_tables(int tid, int T)
  {
    for (int i = tid; i < nprm; i += T) s_ivar[i] = job->ivar[i];
    for (int i = tid; i < nptot; i += T) {
      s_pdescr[i] = job->pdescr[i];
      s_pmin[i] = job->pmint[i];
      s_pmax[i] = job->pmaxt[i];
    }
  }
  template <class Lay>
  __device__ void load_rows(const Lay &lay, int tid, int T)
  {
    for (int i = tid; i < R * nptot; i += T) {
      const int r = i / nptot, j = i - r * nptot;
      float v = 0.0f;
      if (lay.active(r)) {
        const int ist = lay.ibeta(r) * nseq + lay.iseq(r);
        v = job->pcur[(size_t)ist * nptot + j];
      }
      params[i] = v;
      plast[i] = v;
    }
    for (int i = tid; i < R * nprm; i += T) {
      const int r = i / nprm, k = i - r * nprm;
      int h = 0, slow = 0;
      if (lay.active(r)) {
        const int ibeta = lay.ibeta(r), iseq = lay.iseq(r);
        const size_t gi = ((size_t)k * nbeta + ibeta) * nseq + iseq;
        s_pstp[i] = job->pstp[gi];
        s_ncnt[i] = job->n_cnt[gi];
        s_nacpt[i] = job->n_acpt[gi];
        // n_hist[a][k][ibeta][iseq] for a = 0..nadj-1 -> one bit each; a ring
        // holding other values than 0/1 keeps using the global array
        for (int w = 0; w < HW; ++w) {
          unsigned bits = 0u;
          for (int b = 0; b < 32 && 32 * w + b < nadj; ++b) {
            const int v =
                job->n_hist[(((size_t)nprm * (32 * w + b) + k) * nbeta + ibeta) * nseq + iseq];
            h += v;
            slow |= (v != 0 && v != 1);
            bits |= (v != 0 ? 1u : 0u) << b;
          }
          s_hbits[i * HW + w] = bits;
        }
      } else {
        s_pstp[i] = 0.0f;
        s_ncnt[i] = 0;
        s_nacpt[i] = 0;
        for (int w = 0; w < HW; ++w) s_hbits[i * HW + w] = 0u;
      }
      s_hsum[i] = h;
      s_hslow[i] = slow;
    }
  }
  __device__ void load_exchange(int iseq, int tid, int T)
  {
    for (int s = tid; s < nbeta; s += T) {
      x_tcur[s] = job->tcur[s * nseq + iseq];
      x_nexch[s] = job->n_exch[s * nseq + iseq];
      x_beta[s] = job->beta[s];
    }
  }
  // slot r's scalars and generator (init_rng, src/gpu_mcmc.cu:228-239)
  template <class Lay>
  __device__ void load_slot(const Lay &lay, int r, Rng &rng)
  {
    rng.inj = (job->rng_mode == CMC_RNG_INJECTED);
    rng.ovf = false;
    rng.pad = 0u;
    rng.u = rng.n = nullptr;
    rng.cu = rng.cn = rng.lu = rng.ln = 0;
    s_k[r] = 0;
    s_evald[r] = 0;
    s_flag[r] = 0;
    s_chi2c[r] = 0.0f;
    s_ptent[r] = 0.0f;
    s_ptentn[r] = 0;
    s_beta[r] = 0.0f;
    if (!lay.active(r)) return;
    const int ibeta = lay.ibeta(r), iseq = lay.iseq(r), ist = ibeta * nseq + iseq;
    s_ptent[r] = job->ptent[ist];
    s_chi2c[r] = job->chi2c[ist];
    s_beta[r] = job->beta[ibeta];
    s_ptentn[r] = job->ptentn[ist];
    s_flag[r] = job->flag[ist];
    if (rng.inj) {
      rng.u = job->inj_u + (size_t)ist * job->inj_lu;
      rng.n = job->inj_n + (size_t)ist * job->inj_ln;
      rng.lu = job->inj_lu;
      rng.ln = job->inj_ln;
      rng.cu = job->do_init ? 0 : job->inj_cur[2 * ist];
      rng.cn = job->do_init ? 0 : job->inj_cur[2 * ist + 1];
    } else {
      rng.pad = reinterpret_cast<const unsigned *>(job->rndst + (size_t)48 * ist)[9];
      if (job->do_init) {
        // the replica's subsequence in the unsharded run (ist when unsharded)
        const unsigned long long sub =
            job->nseq_total > 0
                ? (unsigned long long)ibeta * job->nseq_total + job->seq_offset + iseq
                : (unsigned long long)ist;
        curand_init(job->seed, sub, 0ull, &rng.st);
      } else {
        rng.st = reinterpret_cast<const curandStateXORWOW *>(job->rndst)[ist];
      }
    }
  }

  // ---- per-slot steps ------------------------------------------------------------
  // init_pcur (src/gpu_mcmc.cu:245-267) and the constants of the first chi^2
  template <class C>
  __device__ void init_slot(int r, Rng &rng, C &cta)
  {
    s_flag[r] = 1;
    for (int i = 0; i < nprm; ++i) {
      const int k = s_ivar[i];
      const float u = rng.uniform();
      float p = __fmaf_rn(s_pmax[k] - s_pmin[k], u, s_pmin[k]);
      if (s_pdescr[k] == 2) p = wrap_pi(p);
      params[r * nptot + k] = p;
    }
    for (int j = 0; j < nptot; ++j) plast[r * nptot + j] = params[r * nptot + j];
    Model::prepare(cta, r, &params[r * nptot]);
    s_evald[r] = 1;
  }
  __device__ float red_sum(int r) const
  {
    float s = 0.f;
    for (int w = 0; w < NW; ++w) s += s_red[r * NW + w];
    return s;
  }
  // spmp_mcmc (src/gpu_mcmc.cu:426-474) and, in burn-in, adjust_steps
  // (:480-526) for slot r after its proposal has been evaluated.
  __device__ void accept_adjust(int r, bool burn, int ibeta, int iseq, Rng &rng)
  {
    const int k = s_k[r];
    if (s_flag[r] != 0) {
      const float c2 = red_sum(r);
      s_chi2n[r] = c2;
      const float a = expf(-0.5f * s_beta[r] * (c2 - s_chi2c[r]));
      const float alpha = (a < 1.0f) ? a : 1.0f;
      const float u = rng.uniform();
      if (u <= alpha) {
        s_chi2c[r] = c2;
        s_nacpt[r * nprm + k] += 1;
      } else {
        if (block)
          for (int j = 0; j < nptot; ++j) params[r * nptot + j] = blk[r * nptot + j];
        else
          params[r * nptot + s_ptentn[r]] = s_ptent[r];
        s_flag[r] = 0;
      }
    }
    if (burn) {
      const int ik = r * nprm + k;
      const int cnt = s_ncnt[ik];
      int modn = cnt % nadj;
      if (modn < 0) modn += nadj;   // guards a negative n_cnt from the caller
      const int nw = (s_flag[r] != 0) ? 1 : 0;
      if (s_hslow[ik]) {
        int *hp = &job->n_hist[(((size_t)nprm * modn + k) * nbeta + ibeta) * nseq + iseq];
        s_hsum[ik] += nw - *hp;
        *hp = nw;
      } else {
        unsigned &word = s_hbits[ik * HW + (modn >> 5)];
        const unsigned bit = 1u << (modn & 31);
        s_hsum[ik] += nw - ((word & bit) ? 1 : 0);
        word = nw ? (word | bit) : (word & ~bit);
      }
      const float rate = (float)s_hsum[ik] / (float)((nadj < cnt) ? nadj : cnt);
      if (rate < 0.30f)
        s_pstp[ik] = (float)((double)s_pstp[ik] / 1.01);
      else
        s_pstp[ik] = (float)((double)s_pstp[ik] * 1.01);
      s_ncnt[ik] = cnt + 1;
    }
  }
  // gen_proposal (src/gpu_mcmc.cu:361-411) for slot r, or in block mode all
  // nprm parameters at once, p_ivar[i] += pstp[0] * (L z)_i with z ~ N(0, I)
  // drawn in order z_0..z_{nprm-1} and (L z)_i accumulated over j = 0..i by
  // fmaf (the pre-proposal row kept in blk for the rejection path); then the
  // model constants when the proposal is inside the prior box (a proposal
  // outside is rejected without evaluation).
  template <class C>
  __device__ void propose(int r, int iseq, Rng &rng, C &cta)
  {
    if (block) {
      const float *L = job->prop_chol + (size_t)iseq * nprm * nprm;
      float *acc = ptmp + r * nptot;
      for (int j = 0; j < nptot; ++j) blk[r * nptot + j] = params[r * nptot + j];
      for (int i = 0; i < nprm; ++i) acc[i] = 0.0f;
      for (int j = 0; j < nprm; ++j) {
        const float z = rng.normal();
        for (int i = j; i < nprm; ++i) acc[i] = __fmaf_rn(__ldg(&L[i * nprm + j]), z, acc[i]);
      }
      const float sd = s_pstp[r * nprm];
      bool out = false;
      for (int i = 0; i < nprm; ++i) {
        const int t = s_ivar[i];
        float p = __fmaf_rn(sd, acc[i], blk[r * nptot + t]);
        if (s_pdescr[t] == 2) p = wrap_pi(p);
        out |= (p < s_pmin[t]) || (p > s_pmax[t]);
        params[r * nptot + t] = p;
      }
      s_k[r] = 0;
      s_ptentn[r] = s_ivar[0];
      s_ptent[r] = blk[r * nptot + s_ivar[0]];
      if (out) {
        for (int j = 0; j < nptot; ++j) params[r * nptot + j] = blk[r * nptot + j];
        s_flag[r] = 0;
        return;
      }
    } else {
      const int k = rng.index(nprm, job->status);
      const int t = s_ivar[k];
      float p = params[r * nptot + t];
      s_k[r] = k;
      s_ptentn[r] = t;
      s_ptent[r] = p;
      const float sd = s_pstp[r * nprm + k];
      const float rn = rng.normal();
      p = __fmaf_rn(sd, rn, p);
      if (s_pdescr[t] == 2) p = wrap_pi(p);
      if ((p < s_pmin[t]) || (p > s_pmax[t])) {
        s_flag[r] = 0;
        return;
      }
      params[r * nptot + t] = p;
    }
    s_flag[r] = 1;
    for (int j = 0; j < nptot; ++j) plast[r * nptot + j] = params[r * nptot + j];
    Model::prepare(cta, r, &params[r * nptot]);
    s_evald[r] = 1;
  }

  // ---- records (pout / tout / chi2 of main iteration m) ----------------------------
  // Every slot's row into staging column m % kCH.
  __device__ void stage_rows(int slot, int tid, int T)
  {
    for (int i = tid; i < R * nprm; i += T) {
      const int r = i / nprm, k = i - r * nprm;
      st_p[i * kCH + slot] = params[r * nptot + s_ivar[k]];
    }
  }
  // The staged columns [0, cnt) of the active slots to pout columns col0 ..
  template <class Lay>
  __device__ void flush_rows(const Lay &lay, int cnt, size_t col0, int tid, int T)
  {
    const size_t ntot = (size_t)job->niter_total;
    for (int i = tid; i < R * nprm * cnt; i += T) {
      const int rk = i / cnt, c = i - rk * cnt;
      const int r = rk / nprm, k = rk - r * nprm;
      if (!lay.active(r)) continue;
      job->pout[(((size_t)k * nbeta + lay.ibeta(r)) * nseq + lay.iseq(r)) * ntot + col0 + c] =
          st_p[rk * kCH + c];
    }
  }
  __device__ void stage_exchange(int slot, int tid, int T)
  {
    for (int s = tid; s < nbeta; s += T) st_t[s * kCH + slot] = x_tcur[s];
    if (tid == 0) st_c[slot] = x_chi2[0];
  }
  __device__ void flush_exchange(int iseq, int cnt, size_t col0, int tid, int T)
  {
    const size_t ntot = (size_t)job->niter_total;
    for (int i = tid; i < nbeta * cnt; i += T) {
      const int s = i / cnt, c = i - s * cnt;
      job->tout[((size_t)s * nseq + iseq) * ntot + col0 + c] = st_t[s * kCH + c];
    }
    for (int c = tid; c < cnt; c += T) job->chi2[(size_t)iseq * ntot + col0 + c] = st_c[c];
  }

  // ---- write-back ------------------------------------------------------------------
  template <class Lay>
  __device__ void store_rows(const Lay &lay, int tid, int T)
  {
    for (int i = tid; i < R * nptot; i += T) {
      const int r = i / nptot, j = i - r * nptot;
      if (!lay.active(r)) continue;
      const int ist = lay.ibeta(r) * nseq + lay.iseq(r);
      job->pcur[(size_t)ist * nptot + j] = params[i];
    }
    for (int i = tid; i < R * nprm; i += T) {
      const int r = i / nprm, k = i - r * nprm;
      if (!lay.active(r)) continue;
      const int ibeta = lay.ibeta(r), iseq = lay.iseq(r);
      const size_t gi = ((size_t)k * nbeta + ibeta) * nseq + iseq;
      job->pstp[gi] = s_pstp[i];
      job->n_cnt[gi] = s_ncnt[i];
      job->n_acpt[gi] = s_nacpt[i];
      if (!s_hslow[i] && job->nburn > 0) {
        for (int a = 0; a < nadj; ++a)
          job->n_hist[(((size_t)nprm * a + k) * nbeta + ibeta) * nseq + iseq] =
              (s_hbits[i * HW + (a >> 5)] >> (a & 31)) & 1u;
      }
    }
  }
  __device__ void store_exchange(int iseq, int tid, int T)
  {
    for (int s = tid; s < nbeta; s += T) {
      job->tcur[s * nseq + iseq] = x_tcur[s];
      job->n_exch[s * nseq + iseq] = x_nexch[s];
    }
  }
  template <class Lay>
  __device__ void store_slot(const Lay &lay, int r, const Rng &rng)
  {
    if (!lay.active(r)) return;
    const int ist = lay.ibeta(r) * nseq + lay.iseq(r);
    job->chi2c[ist] = s_chi2c[r];
    job->flag[ist] = s_flag[r];
    job->ptent[ist] = s_ptent[r];
    job->ptentn[ist] = s_ptentn[r];
    if (rng.inj) {
      job->inj_cur[2 * ist] = rng.cu;
      job->inj_cur[2 * ist + 1] = rng.cn;
    } else {
      rng.store_state(job->rndst + (size_t)48 * ist);
    }
    if (rng.ovf) set_status(job->status, CMC_ERR_STREAM);
  }
};

// ---- the spread layout's exchange through global memory ------------------------------
// Run by all T threads of the CTA after the slot threads accepted their last
// proposals.  1. every CTA publishes its rows and chi^2 (double buffered by
// iteration parity), fences, and counts in at each sequence it holds
// (release); 2. the owner waits (acquire) for (iteration + 1) x the CTAs
// holding its sequence, runs the nbeta attempts, writes the permutation and
// the permuted chi^2 and stores done = iteration + 1 (release); 3. every CTA
// waits for done of its sequences and pulls its new rows.  Deadlock-free by
// induction over iterations (arrivals never wait; an owner's wait needs only
// this iteration's arrivals, which need only the previous iteration's done;
// all CTAs are resident).  A buffer is rewritten two iterations later, after
// each of its readers has arrived at the iteration in between.  Returns false
// after an abort (a wait ran out).
template <class Model, int R>
__device__ bool spread_exchange(SweepState<Model, R> &S, const SpreadLayout &lay,
                                const SpreadCtl &ctl, int iter, bool burn, Rng &rng, int tid,
                                int T, int *s_ok)
{
  using AtomicInt = cuda::atomic_ref<int, cuda::thread_scope_device>;
  const int nbeta = S.nbeta, nptot = S.nptot;
  const size_t nrep = (size_t)nbeta * S.nseq, par = (size_t)(iter & 1);
  float *xp = ctl.xp + par * nrep * nptot;
  float *xc = ctl.xc + par * nrep;
  int *xperm = ctl.xperm + par * nrep;
  float *xchi = ctl.xchi + par * nrep;
  const int cnt = lay.cnt;
  __syncthreads();   // the last accept_adjust may have restored a row
  for (int i = tid; i < cnt * nptot; i += T) xp[(size_t)lay.gstart * nptot + i] = S.params[i];
  for (int r = tid; r < cnt; r += T) xc[lay.gstart + r] = S.s_chi2c[r];
  __threadfence();
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    for (int s = lay.seq_lo; s <= lay.seq_hi; ++s)
      AtomicInt(ctl.arrive[s]).fetch_add(1, cuda::memory_order_release);
  }
  if (lay.owner() && tid < 32) {
    const int s = lay.own_seq();
    int ok = 1;
    if (tid == 0) {
      ok = spin_until_geq(&ctl.arrive[s], (iter + 1) * lay.own_ncta, ctl.abort, S.job->status);
      __threadfence();
    }
    ok = __shfl_sync(0xffffffffu, ok, 0);
    if (ok) {
      const float chi = (tid < nbeta) ? __ldcg(&xc[(size_t)s * nbeta + tid]) : 0.0f;
      warp_exchange(chi, burn, rng, lay.own_slot(), nbeta, S.x_beta, S.x_chi2, S.x_tcur,
                    S.x_perm, S.x_nexch, S.job->status);
      if (tid < nbeta) {
        xperm[(size_t)s * nbeta + tid] = S.x_perm[tid];
        xchi[(size_t)s * nbeta + tid] = S.x_chi2[tid];
      }
      __threadfence();
      __syncwarp();
      if (tid == 0 && s != ctl.hold)
        AtomicInt(ctl.done[s]).store(iter + 1, cuda::memory_order_release);
    }
  }
  if (tid == 0) {
    int ok = 1;
    for (int s = lay.seq_lo; s <= lay.seq_hi && ok; ++s)
      ok = spin_until_geq(&ctl.done[s], iter + 1, ctl.abort, S.job->status) ? 1 : 0;
    __threadfence();
    *s_ok = ok;
  }
  __syncthreads();
  if (!*s_ok) return false;
  for (int i = tid; i < cnt * nptot; i += T) {
    const int r = i / nptot, j = i - r * nptot, f = lay.gstart + r;
    const int src = __ldcg(&xperm[f]);
    S.params[i] = __ldcg(&xp[((size_t)(f - f % nbeta) + src) * nptot + j]);
  }
  for (int r = tid; r < cnt; r += T) S.s_chi2c[r] = __ldcg(&xchi[lay.gstart + r]);
  __syncthreads();
  return true;
}

// ---- cluster and spread layouts: one body for all R slots ---------------------------

// Relaxed device-scope read of a flag another agent (a host copy) may set.
__device__ __forceinline__ int read_flag(const int *p)
{
  return cuda::atomic_ref<int, cuda::thread_scope_device>(*const_cast<int *>(p))
      .load(cuda::memory_order_relaxed);
}

// The replicas of layout `lay` on the calling CTA (in the cluster layout, all
// CTAs of the cluster call this with the same sequence).  `smem` is the CTA's
// dynamic shared memory, at least make_plan(...).total bytes for this job;
// `ctl` is used by the spread layout only.  `cancel` (cluster layout, may be
// null): a flag read by cluster rank 0 at every exchange; once set, the
// cluster stops after that exchange, its records and state written back.
template <class Model, int R, class Lay>
__device__ void run_replicas(const cmc_job &job, const typename Model::Packed &pk, const Lay &lay,
                             const SpreadCtl &ctl, const int *cancel, unsigned char *smem)
{
  const int tid = threadIdx.x, T = blockDim.x, NW = T >> 5;
  const int nbeta = job.nbeta, nseq = job.nseq, nptot = job.nptot, nprm = job.nprm;

  const SmemPlan P = make_plan(R, T, nptot, nprm, nbeta, job.nadj, sizeof(typename Model::Consts),
                               Model::scratch_bytes(pk, R));
  SweepState<Model, R> S;
  S.bind(job, P, smem, NW);
  __shared__ int s_ok, s_stop;

  Cta<Model, R> cta;
  cta.job = &job;
  cta.pk = &pk;
  cta.consts = S.s_consts;
  cta.flag = S.s_flag;
  cta.scratch = S.scratch;
  cta.tid = tid;
  cta.nthreads = T;
#pragma unroll
  for (int r = 0; r < R; ++r) cta.ist[r] = lay.active(r) ? lay.ibeta(r) * nseq + lay.iseq(r) : 0;
  cta.ph_region = lay.ph_region(nbeta);

  // ---- load tables and state ------------------------------------------------
  S.load_tables(tid, T);
  S.load_rows(lay, tid, T);
  if (lay.owner()) S.load_exchange(lay.own_seq(), tid, T);
  Rng rng;
  if (tid < R) S.load_slot(lay, tid, rng);
  Model::setup(cta, tid, T);
  __syncthreads();

  // ---- init_pcur + first chi^2 (src/gpu_mcmc.cu:245-267, 714-719) ---------
  if (job.do_init) {
    if (tid < R && lay.active(tid)) S.init_slot(tid, rng, cta);
    __syncthreads();
    float acc[R];
    Model::template eval<R>(cta, acc);
    block_reduce<Model, R>(acc, S.s_red, tid, NW);
    __syncthreads();
    if (tid < R && lay.active(tid)) S.s_chi2c[tid] = S.red_sum(tid);
    __syncthreads();
  }

  // The accept step of proposal n is fused with proposal n+1 on the slot's
  // thread, so that one barrier per proposal disappears.
  const int nsteps = job.nburn + job.niter;
  for (int step = 0; step < nsteps; ++step) {
    const bool burn = step < job.nburn;
    for (int ipm = 0; ipm < nprm; ++ipm) {
      if (tid < R && lay.active(tid)) {
        const int r = tid;
        if (ipm > 0) S.accept_adjust(r, burn, lay.ibeta(r), lay.iseq(r), rng);
        S.propose(r, lay.iseq(r), rng, cta);
      }
      __syncthreads();
      // calc_chi2_terms x npass + the chi^2 sum (src/gpu_mcmc.cu:273-325, 447-448)
      float acc[R];
      Model::template eval<R>(cta, acc);
      block_reduce<Model, R>(acc, S.s_red, tid, NW);
      __syncthreads();
    }
    if (tid < R && lay.active(tid)) S.accept_adjust(tid, burn, lay.ibeta(tid), lay.iseq(tid), rng);

    // ---- replica_exchange (src/gpu_mcmc.cu:533-626) ------------------------
    // nbeta attempts in the reference's order, drawn from the ibeta = 0
    // replica's generator.
    int stop = 0;
    if constexpr (!Lay::kSpread) {
      cg::cluster_group cluster = cg::this_cluster();
      const int rank = lay.rank;
      float *x_chi2 = S.x_chi2, *x_beta = S.x_beta;
      int *x_perm = S.x_perm, *x_tcur = S.x_tcur, *x_nexch = S.x_nexch;
      cluster.sync();
      // one reading of the cancel flag for the whole cluster (rank 0's,
      // read by every CTA after the next cluster barrier)
      if (rank == 0 && tid == 0) s_stop = (cancel != nullptr && read_flag(cancel) != 0) ? 1 : 0;
      if (nbeta <= 32) {
        if (rank == 0 && tid < 32) {
          const float chi =
              (tid < nbeta) ? cluster.map_shared_rank(S.s_chi2c, tid / R)[tid % R] : 0.0f;
          warp_exchange(chi, burn, rng, 0, nbeta, x_beta, x_chi2, x_tcur, x_perm, x_nexch,
                        job.status);
        }
      } else {
        if (rank == 0) {
          // gather the nbeta chi^2 values in parallel (one remote load each)
          for (int s = tid; s < nbeta; s += T) {
            x_chi2[s] = cluster.map_shared_rank(S.s_chi2c, s / R)[s % R];
            x_perm[s] = s;
          }
          __syncthreads();
        }
        if (rank == 0 && tid == 0) {
          const int nb1 = nbeta - 1;
          for (int ib = 0; ib < nbeta; ++ib) {
            const int k = rng.index(nb1, job.status);
            const float a =
                expf(-0.5f * (x_beta[k + 1] - x_beta[k]) * (x_chi2[k] - x_chi2[k + 1]));
            const float alpha = (a < 1.0f) ? a : 1.0f;
            const float u = rng.uniform();
            if (u <= alpha) {
              int ti = x_tcur[k]; x_tcur[k] = x_tcur[k + 1]; x_tcur[k + 1] = ti;
              int pi = x_perm[k]; x_perm[k] = x_perm[k + 1]; x_perm[k + 1] = pi;
              float cc = x_chi2[k]; x_chi2[k] = x_chi2[k + 1]; x_chi2[k + 1] = cc;
              if (!burn) x_nexch[k] += 1;
            }
          }
        }
      }
      cluster.sync();
      stop = *cluster.map_shared_rank(&s_stop, 0);
      {
        const int *perm0 = cluster.map_shared_rank(x_perm, 0);
        const float *chi0 = cluster.map_shared_rank(x_chi2, 0);
        for (int i = tid; i < R * nptot; i += T) {
          int r = i / nptot, j = i - r * nptot;
          int src = perm0[rank * R + r];
          const float *rp = cluster.map_shared_rank(S.params, src / R);
          S.ptmp[i] = rp[(src % R) * nptot + j];
        }
        if (tid < R) S.ptmp[R * nptot + tid] = chi0[rank * R + tid];
      }
      cluster.sync();
      for (int i = tid; i < R * nptot; i += T) S.params[i] = S.ptmp[i];
      if (tid < R) S.s_chi2c[tid] = S.ptmp[R * nptot + tid];
      __syncthreads();
    } else {
      // after an abort every CTA leaves the iteration loop and writes its
      // state back with the error status set
      if (!spread_exchange<Model, R>(S, lay, ctl, step, burn, rng, tid, T, &s_ok)) break;
    }
    Model::after_exchange(cta);

    // ---- record pout / tout / chi2 (main stage) ---------------------------
    if (!burn) {
      const int m = step - job.nburn;
      const int slot = m % kCH;
      S.stage_rows(slot, tid, T);
      if (lay.owner()) S.stage_exchange(slot, tid, T);
      if (slot == kCH - 1 || m == job.niter - 1 || stop) {
        __syncthreads();
        const size_t col0 = (size_t)job.itr0 + (m - slot);
        S.flush_rows(lay, slot + 1, col0, tid, T);
        if (lay.owner()) S.flush_exchange(lay.own_seq(), slot + 1, col0, tid, T);
      }
      __syncthreads();
    }
    if (stop) break;
  }

  // ---- write the state back ------------------------------------------------
  S.store_rows(lay, tid, T);
  if (lay.owner()) S.store_exchange(lay.own_seq(), tid, T);
  if (tid < R) S.store_slot(lay, tid, rng);
  // Model rows of each replica's last evaluation (datm / chi2m outputs).
  Model::template final_rows<R>(cta, S.plast, S.s_evald);
  // No CTA may leave (or start its next sequence) while another can still
  // read its shared memory.
  if constexpr (!Lay::kSpread) cg::this_cluster().sync();
}

// ---- kernels ------------------------------------------------------------------------

// One launch for one job: cluster c runs sequence c.  (The kernel bodies are
// device functions so that a model compiled into a loadable module can wrap
// them in kernels of its own; see module_plugin.cu.)
template <class Model, int R>
__device__ __forceinline__ void sweep_body(const cmc_job &job, const typename Model::Packed &pk)
{
  extern __shared__ __align__(16) unsigned char smem[];
  cg::cluster_group cluster = cg::this_cluster();
  ClusterLayout<R> lay;
  lay.rank = (int)cluster.block_rank();
  lay.seq = blockIdx.x / (int)cluster.num_blocks();
  run_replicas<Model, R>(job, pk, lay, SpreadCtl{}, nullptr, smem);
}

template <class Model, int R>
__global__ void __launch_bounds__(kMaxThreads, CMC_MIN_BLOCKS)
sweep_kernel(const cmc_job job, const typename Model::Packed pk)
{
  sweep_body<Model, R>(job, pk);
}

// One cooperative launch of N = gridDim.x CTAs in the spread layout, over
// ctl.ngroups sequence groups in turn (the sequences' chains are independent,
// so the grouping changes no result; it bounds the phase regions in use).
// The host checks that the N CTAs are resident at once and that nbeta <= 32,
// N <= every group's nrep and ceil(nrep / N) <= R <= nbeta for the largest
// (every CTA's count fits its R slots, and a CTA spans at most two
// sequences); with phases in global memory, that the job's phase area holds
// N*R regions.
template <class Model, int R>
__device__ __forceinline__ void spread_body(const cmc_job &job, const typename Model::Packed &pk,
                                            const SpreadCtl &ctl)
{
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_abort;
  for (int g = 0; g < ctl.ngroups; ++g) {
    // a group starts once every thread of the CTA is done with the last
    // group's shared memory; none starts after an abort (one reading of the
    // flag for the whole CTA)
    if (threadIdx.x == 0) s_abort = (g > 0 && read_flag(ctl.abort) != 0) ? 1 : 0;
    __syncthreads();
    if (s_abort) break;
    int seq0 = 0, n = 0;
    spread_group(job.nseq, ctl.ngroups, g, seq0, n);
    const SpreadLayout lay = make_spread_layout(job.nbeta, seq0, n, (int)gridDim.x,
                                                (int)blockIdx.x, (int)blockIdx.x * R);
    run_replicas<Model, R>(job, pk, lay, ctl, nullptr, smem);
  }
}

template <class Model, int R>
__global__ void __launch_bounds__(kMaxThreads, CMC_MIN_BLOCKS)
spread_kernel(const cmc_job job, const typename Model::Packed pk, const SpreadCtl ctl)
{
  spread_body<Model, R>(job, pk, ctl);
}

// Persistent launch over a work list of (job, sequence) items of many
// independent jobs (fits): each cluster takes the next item from an atomic
// counter (the list is sorted by decreasing cost, so the tail is short),
// copies that job's descriptor into shared memory, applies this launch's
// iteration window (do_init, nburn, niter, itr0) and runs the sequence.
// counter[0] is the work-list counter, counter[1] the cancel flag
// (cmc_batch_cancel): once it is set no cluster takes another item and a
// running one stops after its next exchange.
template <class Model, int R>
__device__ __forceinline__ void batch_body(const cmc_job *jobs, const typename Model::Packed *pks,
                                           const int2 *items, int nitems, int *counter,
                                           int do_init, int nburn, int niter, int itr0)
{
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ cmc_job s_job;
  __shared__ typename Model::Packed s_pk;
  __shared__ int s_item;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  for (;;) {
    if (rank == 0 && threadIdx.x == 0)
      s_item = (read_flag(counter + 1) != 0) ? nitems : atomicAdd(counter, 1);
    cluster.sync();
    const int it = *cluster.map_shared_rank(&s_item, 0);
    cluster.sync();
    if (it >= nitems) break;
    const int2 w = items[it];
    {
      const int *src = reinterpret_cast<const int *>(&jobs[w.x]);
      int *dst = reinterpret_cast<int *>(&s_job);
      for (int i = threadIdx.x; i < (int)(sizeof(cmc_job) / 4); i += blockDim.x) dst[i] = src[i];
      const int *psrc = reinterpret_cast<const int *>(&pks[w.x]);
      int *pdst = reinterpret_cast<int *>(&s_pk);
      for (int i = threadIdx.x; i < (int)(sizeof(s_pk) / 4); i += blockDim.x) pdst[i] = psrc[i];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      s_job.do_init = do_init;
      s_job.nburn = nburn;
      s_job.niter = niter;
      s_job.itr0 = itr0;
    }
    __syncthreads();
    ClusterLayout<R> lay;
    lay.rank = rank;
    lay.seq = w.y;
    run_replicas<Model, R>(s_job, s_pk, lay, SpreadCtl{}, counter + 1, smem);
  }
}

template <class Model, int R>
__global__ void __launch_bounds__(kMaxThreads, CMC_MIN_BLOCKS)
batch_kernel(const cmc_job *jobs, const typename Model::Packed *pks, const int2 *items,
             int nitems, int *counter, int do_init, int nburn, int niter, int itr0)
{
  batch_body<Model, R>(jobs, pks, items, nitems, counter, do_init, nburn, niter, itr0);
}

}  // namespace cmc
