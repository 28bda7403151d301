// model_sgra.cuh -- built-in fast path for the Sgr A* crescent + Gaussian
// visibility model: amplitudes (pass 0) and closure phases (pass 1).
//
// Same model as the reference's examples/sgra_model_fit/model.cuh:
//   sgra_model9  (imodel == 1)  :322-462   Zsp Re rq ecc fade gax aq gq th
//   sgra_model13 (imodel == 2)  :120-315   Zsp Re rq ecc fade gr gax aq gq
//                                          alpha beta eta th
//   model() dispatcher          :9-115     amplitude + phase for id < nvis,
//                                          closures phi_i + phi_j - phi_k
//                                          (cpExt 0) or from three model
//                                          phases on a triangle (cpExt 1).
//
// Restated for the GPU:
//   * The ring terms are written with F1(x) = J1(x)/x and F2(x) = J2(x)/x^2,
//     both smooth even functions with finite limits at x = 0:
//       ree = 0.5 (h+h0) Rex J1(x)/rho         = [0.5 (h+h0) Rex kex]   F1(x)
//       ime = (h-h0)/(4 pi) [pi Rex (J0-J2)/rho^2 - J1/rho^3] U
//           = -(h-h0)/(4 pi) x J2(x)/rho^3 U  = [-(h-h0)/(4 pi) kex^3] F2(x) U
//     with x = kex rho, kex = 2 pi Rex (J0 - J2 = 2 J0 - 2 J1/x).  This removes
//     the reference's rho <= 1e-7 branch (model.cuh:389-417): its limits are
//     F1(0) = 1/2 and F2(0) = 1/8.
//   * All parameter-only quantities (h, h0, d, rotations, weights, ...) are
//     computed once per proposal per replica (prepare) instead of per datum.
//   * F1/F2 come from piecewise polynomial tables (bessel_table.cuh); the
//     data points are packed sorted by |uv|, so the 32 lanes of a warp read
//     the same (or two neighbouring) table intervals for any replica.
//   * sin/cos of pi*t and atan2 are float32 polynomials (fastmath.cuh).
//   * Closure phases are formed from unit phasors z = V/|V| of the model:
//     the residual wrap(obs - (phi_i + phi_j - phi_k)) equals
//     arg(e^{i obs} conj(z_i z_j conj z_k)), one atan2 per closure.  When
//     the phasors do not fit in shared memory, phases are stored instead
//     and the residual is wrapped arithmetically.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>

#include "cmc_job.h"
#include "fastmath.cuh"

namespace cmc {

// Per-replica constants of the accurate forward pass (the gradient and
// Fisher kernels, model_sgra_grad.cuh).
struct SgraConsts {
  float cth, sth;   // rotation by th
  float kex, kin;   // 2 pi Rex, 2 pi Rin (nrad)
  float ae, be;     // outer ring: ree = ae F1(kex rho), ime = be F2(kex rho) U
  float ai, bi;     // inner ring
  float dsh;        // inner-ring displacement phase / pi = dsh * U
  float gc, gs;     // Gaussian axes rotation
  float gx, gy;     // Gaussian exponent coefficients
  float gpu, gpv;   // Gaussian phase / pi = gpu u + gpv v
  float zr, zg;     // ring and Gaussian weights
  int inner, gauss, ring;
  int bigx;         // some Bessel argument of this replica is beyond the table
};

// Per-replica constants of the sampling path (prepare, once per proposal),
// folded for the fewest operations per model term and held as four float4
// (four 128-bit shared-memory loads per term):
//   * Bessel arguments as table coordinates: t = kex8 rho - 1/2 with
//     kex8 = kBesselSub |2 pi Rex| (F1, F2 are even);
//   * the ring weight zr folded into the ring coefficients ae, be, ai, bi;
//   * sin / cos arguments in radians: dsh = 2 pi d, gpu / gpv likewise;
//   * the Gaussian exponent in base 2 with the axis scales folded into the
//     rotation: log2 e (gx ug^2 + gy vg^2) = ug'^2 + vg'^2,
//     ug' = gcx u + gsx v, vg' = gcy v - gsy u;
//   * a switched-off ring (sgra_model13 Gaussian only) has all of its
//     coefficients zero, so its terms vanish without a select.
struct __align__(16) SgraFastConsts {
  float4 rot;    // cth, sth, kex8, kin8
  float4 ring;   // zr ae, zr be, zr ai, zr bi: ree = ae F1 - ..., ime = be F2 U - ...
  float4 gax;    // gcx, gsx, gcy, gsy
  float4 gph;    // dsh, gpu, gpv, zg: ring shift phase dsh U, Gaussian phase gpu u + gpv v
  int bigx;      // some Bessel argument of this replica is beyond the table
  int pad[3];
};

// Model visibility V = Vre + i Vim of one replica at (u, v), |uv| = rho.
// Straight-line code: a switched-off component (no inner disk: ai = bi = 0;
// no Gaussian: zg = 0; no ring: its coefficients 0) contributes zero, so the
// evaluations of different replicas can be interleaved.  Every multiply-add
// is an explicit fmaf (no a*b + c*d left for the compiler to contract either
// way), so that the sweep and batch kernels, compiled separately, round
// identically.
template <bool BIG = true>
__device__ __forceinline__ float2 sgra_vis(const SgraFastConsts &c, const float4 *btab, float u,
                                          float v, float rho)
{
  const float4 k = c.rot, w = c.ring, g = c.gax, q = c.gph;
  const float U = fmaf(u, k.x, v * k.y);
  float f1, f2, g1, g2, sd, cd;
  bessel_f12_at<BIG>(btab, fmaf(k.z, rho, -0.5f), f1, f2);
  bessel_f12_at<BIG>(btab, fmaf(k.w, rho, -0.5f), g1, g2);
  sincos_fast(q.x * U, &sd, &cd);
  const float rei = w.z * g1, imi = w.w * g2 * U;
  const float re = fmaf(w.x, f1, -fmaf(rei, cd, -(imi * sd)));
  const float im = fmaf(w.y * f2, U, -fmaf(rei, sd, imi * cd));
  const float ug = fmaf(u, g.x, v * g.y), vg = fmaf(v, g.z, -(u * g.w));
  const float ga = q.w * ex2_ftz(-fmaf(ug, ug, vg * vg));
  float sg, cg;
  sincos_fast(fmaf(q.y, u, q.z * v), &sg, &cg);
  return make_float2(fmaf(ga, cg, re), fmaf(ga, sg, im));
}

// Phases kept in global memory (phase mode 2) are written and read back by
// the same CTA within one proposal; the stores and loads carry an L2
// evict-last policy so that the resident replicas' phase regions stay in L2
// rather than being written back to HBM in between (CMC_PHASE_L2_HINT = 0:
// plain stores and loads).
#ifndef CMC_PHASE_L2_HINT
#define CMC_PHASE_L2_HINT 1
#endif
__device__ __forceinline__ unsigned long long l2_evict_last_policy()
{
  unsigned long long pol = 0ull;
#if CMC_PHASE_L2_HINT
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
#endif
  return pol;
}
template <bool GL>
__device__ __forceinline__ void store_phase(float *p, float v, unsigned long long pol)
{
#if CMC_PHASE_L2_HINT
  if constexpr (GL) {
    asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(p), "f"(v), "l"(pol)
                 : "memory");
    return;
  }
#endif
  (void)pol;
  *p = v;
}
template <bool GL>
__device__ __forceinline__ float load_phase(const float *p, unsigned long long pol)
{
#if CMC_PHASE_L2_HINT
  if constexpr (GL) {
    float v;
    asm volatile("ld.global.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol)
                 : "memory");
    return v;
  }
#endif
  (void)pol;
  return *p;
}

// Data packing kernels (defined once, in the library translation unit).
__global__ void sgra_points_kernel(const float *coor, const float *dat, const float *std2r,
                                   int nvis, int ncph, int cpext, float4 *raw, float *key);
__global__ void sgra_mark_kernel(const int *icoor, int nvis, int ncph, int cpext, int *used);
__global__ void rank_kernel(const float *key, const int *used, int n, int *newpos);
__global__ void sgra_scatter_kernel(const float4 *raw, const float *key, const int *newpos,
                                    const int *used, int npts, const int *icoor,
                                    const float *dat, const float *std2r, int nvis, int ncph,
                                    int cpext, float4 *vis, float *rho, int *orig, int4 *cli,
                                    float4 *clf, int *aux, int *status);

// CMC_BRANCHFREE: evaluate every local replica, inactive ones included (their
// sums are discarded), so that the R independent evaluations interleave.
#ifndef CMC_BRANCHFREE
#define CMC_BRANCHFREE 1
#endif

struct SgraModel {
  using Consts = SgraFastConsts;
  struct Packed {
    const float4 *vis;   // [npts] sorted by |uv|: u, v, amp_obs, 1/sigma^2 (0: triangle point)
    const float *rho;    // [npts] |uv| of vis
    const int *orig;     // [npts] index of vis[i] in the caller's order
    const int4 *cli;     // [ncph] sorted-point indices i, j, k of closure c
    const float4 *clf;   // [ncph] cos obs, sin obs, 1/sigma^2, obs
    float *gph;          // [nrep][npts] phases in global memory (phasor == 2), or null
    const int *aux;      // [0]: nused -- points [0, nused) are closure corners and need a
                         // phase; [1]: max |uv| (float bits)
    int nvis, npts, ncph, cpext, npass, imodel, phasor, ndat, nrep;
  };

  // Phase storage (Packed::phasor): 1 = unit phasors in shared memory, 0 =
  // phases in shared memory, 2 = phases in global memory (L2), one npts-long
  // region per replica in job.work after the packed data.  Mode 2 frees the
  // shared memory that large data sets need for their phases, so that more
  // replicas per CTA and more CTAs per SM fit; it is offered from
  // kGlobalPhaseMinPts points on and when job.work holds the regions.
  static constexpr bool kGlobalPhases = true;
  static constexpr int kGlobalPhaseMinPts = 2048;

  static constexpr bool kRowsInEval = false;
  // instantiated replicas-per-CTA counts: 1, 2, 4, 8 (cluster layout), 1..8
  // (spread layout; a one-short CTA's unused slot writes phases of its own,
  // in shared memory or in the CTA's own global region)
  static constexpr int kMaxR = 8;
  static constexpr bool kSpread = true;
  static constexpr unsigned kTabBytes =
      (unsigned)sizeof(float4) * kBesselIntervals * ((kBesselDeg + 1) / 2);

  // data points one replica's evaluation runs over
  __host__ __device__ static int points(const Packed &pk) { return pk.npts + pk.ncph; }

  // shared scratch: Bessel table, then phasors [R][npts] (float2) or phases
  // (float); the table only when the phases live in global memory
  __host__ __device__ static unsigned scratch_bytes(const Packed &pk, int R)
  {
    if (pk.phasor == 2) return kTabBytes;
    return kTabBytes + (unsigned)R * (unsigned)pk.npts * (pk.phasor ? 8u : 4u);
  }

  // the phases of local replica 0 of a CTA (replica r at + r * npts)
  template <class Cta>
  __device__ static float *phase_area(const Cta &cta)
  {
    const Packed &pk = *cta.pk;
    if (pk.phasor == 2) return pk.gph + (size_t)cta.ph_region * pk.npts;
    return cta.scratch + kTabBytes / 4;
  }

  // ---- host side: sizes, validation, packing ------------------------------
  // mode 0: sweep, 1: calc_modchi2, 2: calc_model.
  static int host_dims(const cmc_job &j, int mode, Packed &pk, const char **err)
  {
    const int nrep = j.nbeta * j.nseq;
    pk.nvis = j.hidat[0];
    pk.cpext = (j.nidat >= 3 && mode != 2) ? j.hidat[2] : 0;
    pk.ncph = (mode == 2) ? 0 : j.ndat - pk.nvis;
    pk.npass = (mode == 0) ? j.npass : 2;
    pk.imodel = j.imodel;
    pk.ndat = j.ndat;
    if (pk.npass < 2) pk.ncph = 0;   // closures are a pass-1 product
    pk.npts = pk.nvis + (pk.cpext ? 3 * pk.ncph : 0);
    pk.phasor = 1;
    pk.nrep = nrep;
    pk.gph = nullptr;
    pk.aux = nullptr;
    if (j.nidat < 1 || pk.nvis < 0 || pk.nvis > j.ndat) {
      *err = "Sgr A* model: idat[0] (nvis) must be in [0, ndat]";
      return CMC_ERR_ARG;
    }
    if (j.imodel != 1 && j.imodel != 2) {
      *err = "Sgr A* model: imodel must be 1 (sgra_model9) or 2 (sgra_model13)";
      return CMC_ERR_MODEL;
    }
    if (j.nptot < (j.imodel == 1 ? 9 : 13)) {
      *err = "Sgr A* model: nptot must be >= 9 (imodel 1) or >= 13 (imodel 2)";
      return CMC_ERR_ARG;
    }
    if (pk.cpext) {
      if (j.ncoor < 2 * pk.nvis + 4 * pk.ncph) {
        *err = "Sgr A* model: cpExt=1 needs ncoor >= 2*nvis + 4*ncph";
        return CMC_ERR_ARG;
      }
    } else if (j.ncoor < 2 * pk.nvis || j.nicoor < 3 * pk.ncph) {
      *err = "Sgr A* model: needs ncoor >= 2*nvis and nicoor >= 3*ncph";
      return CMC_ERR_ARG;
    }
    const long long need = (long long)nrep * (j.ndat + pk.nvis);
    if (j.datm != nullptr && j.ndatm < need) {
      *err = "Sgr A* model: ndatm must be >= nbeta*nseq*(ndat + nvis) (amplitude/closure "
             "head plus the phase tail)";
      return CMC_ERR_ARG;
    }
    if (pk.npts >= kGlobalPhaseMinPts && j.work != nullptr &&
        j.work_bytes >= host_work_bytes(pk))
      pk.gph = reinterpret_cast<float *>(static_cast<unsigned char *>(j.work) +
                                         host_work_bytes_min(pk));
    return CMC_OK;
  }

  // the packed data (what every launch needs), 256-byte aligned
  static size_t host_work_bytes_min(const Packed &pk)
  {
    const size_t b = (size_t)pk.npts * 52 + (size_t)pk.ncph * 32 + 512;
    return (b + 255) & ~(size_t)255;
  }

  // packed data + the global phase regions when the data set is large enough
  // to use them (cmc_work_bytes reports this size): one per replica, and
  // kMaxR more for the spread layout, whose CTAs own R regions each
  // (N*R <= nrep + R - 1)
  static size_t host_work_bytes(const Packed &pk)
  {
    size_t b = host_work_bytes_min(pk);
    if (pk.npts >= kGlobalPhaseMinPts)
      b += ((size_t)pk.nrep + kMaxR) * pk.npts * sizeof(float);
    return b;
  }

  static int host_pack(const cmc_job &j, Packed &pk, void *work, cudaStream_t s);

  // Bessel table into shared memory; every local replica's constants zeroed
  // (a valid in-table state for replicas not yet prepared).
  template <class Cta>
  __device__ static void setup(Cta &cta, int tid, int T)
  {
    // cached: model_i = nused (points that need a phase), model_f = max |uv|
    const Packed &pk = *cta.pk;
    constexpr int kWords =
        (int)(sizeof(SgraFastConsts) / 4) * (int)std::extent<decltype(Cta::ist)>::value;
    int *cz = reinterpret_cast<int *>(cta.consts);
    for (int i = tid; i < kWords; i += T) cz[i] = 0;
    cta.model_i = (pk.ncph > 0 && pk.npass >= 2) ? __ldg(&pk.aux[0]) : 0;
    cta.model_f = (pk.npts > 0) ? __int_as_float(__ldg(&pk.aux[1])) : 0.0f;
    float4 *tab = reinterpret_cast<float4 *>(cta.scratch);
    const float4 *src = &kBesselTab[0][0];
    for (int i = tid; i < (int)(kTabBytes / sizeof(float4)); i += T) tab[i] = src[i];
  }

  template <class Cta>
  __device__ static void after_exchange(Cta &) {}

  // Its sines and cosines use sincos_fma (explicit FMAs only): the init and
  // proposal paths of the sweep and batch kernels must round them the same.
  template <class Cta>
  __device__ static void prepare(Cta &cta, int r, const float *p)
  {
    SgraFastConsts &c = cta.consts[r];
    const float pi = 3.1415926535897931f;
    const int im = cta.pk->imodel;
    const float Zsp = p[0], Re = p[1], rq = p[2], ecc = p[3], fade = p[4];
    float gr = 0.f, gax, aq, gq, alpha = 0.f, beta = 0.f, eta = 0.f, th;
    if (im == 1) {
      gax = p[5]; aq = p[6]; gq = p[7]; th = p[8];
    } else {
      gr = p[5]; gax = p[6]; aq = p[7]; gq = p[8];
      alpha = p[9]; beta = p[10]; eta = p[11]; th = p[12];
    }
    // Two divisions in all (1/Rex and h): this runs on one thread per replica
    // between the evaluations, so its latency is paid once per proposal.
    // Products that feed a sum are __fmul_rn (never contracted), so the sweep
    // and batch kernels round them identically.
    const float Rex = Re * 4.84813681109536e-3f;   // uas -> nrad: (pi/180)/3600*1e3
    const float Rin = __fmul_rn(rq, Rex);
    float d = __fmul_rn(ecc, Rex - Rin);
    if (im != 1) {
      float se, ce;
      sincos_fma(eta - th, &se, &ce);
      d = __fmul_rn(d, ce);
    }
    const float dr = __fmul_rn(d, 1.0f / Rex);
    const float h = (2.0f / pi) / fmaf(fmaf(-(Rin * Rin), 1.0f + dr, Rex * Rex), fade,
                                       fmaf(-(Rin * Rin), 1.0f - dr, Rex * Rex));
    const float h0 = __fmul_rn(fade, h);
    const float hm = (h - h0) * (-0.25f / pi);      // -(h - h0) / (4 pi)
    float sth, cth;
    sincos_fma(th, &sth, &cth);
    const float kex = 2.0f * pi * Rex;
    const float kin = 2.0f * pi * Rin;
    const bool inner = (Rin != 0.0f);
    float ae = 0.5f * (h + h0) * Rex * kex;
    float be = hm * (kex * kex * kex);
    float ai = inner ? 0.5f * fmaf(-dr, h - h0, h + h0) * Rin * kin : 0.0f;
    float bi = inner ? hm * rq * (kin * kin * kin) : 0.0f;
    float dsh = 2.0f * d;
    float kex8 = fabsf(kex) * (float)kBesselSub, kin8 = fabsf(kin) * (float)kBesselSub;
    // Gaussian: exponent (pi / (2 sqrt(2 ln 2)))^2 2 (FWHM projections)^2,
    // i.e. pi^2 / (4 ln 2) (gsx^2 ug^2 + gsy^2 vg^2); in base 2 the axis
    // scales are K gsx and K gsy with K = sqrt(log2 e pi^2 / (4 ln 2)) =
    // pi / (2 ln 2)
    const float K = 2.2661800709135966f;
    const float sy = K * (gax * Rex), sx = aq * sy;
    float gc, gs, gpu, gpv;
    bool gauss = !(gax == 0.0f || aq == 0.0f || gq == 0.0f);
    if (im == 1) {
      const float gshift = Rin - d;
      gc = cth;
      gs = sth;
      gpu = -2.0f * gshift * cth;
      gpv = -2.0f * gshift * sth;
    } else {
      float sa, ca;
      sincos_fma(beta, &gs, &gc);
      sincos_fma(alpha, &sa, &ca);
      gpu = -2.0f * gr * Rex * ca;
      gpv = -2.0f * gr * Rex * sa;
    }
    float zr = Zsp, zg = 0.0f;
    if (gauss) {
      zr = Zsp * (1.0f - gq);
      zg = Zsp * gq;
    }
    if (im != 1 && gq == 1.0f) {   // sgra_model13: Gaussian only (model.cuh:204-210)
      zr = 0.0f;
      ae = be = ai = bi = dsh = kex8 = kin8 = 0.0f;
      zg = Zsp;
      gauss = !(gax == 0.0f || aq == 0.0f);
    }
    if (!gauss) zg = 0.0f;
    c.rot = make_float4(cth, sth, kex8, kin8);
    c.ring = make_float4(zr * ae, zr * be, zr * ai, zr * bi);
    c.gax = make_float4(gc * sx, gs * sx, gc * sy, gs * sy);
    c.gph = make_float4(pi * dsh, pi * gpu, pi * gpv, zg);
    // the straight-line loops may use the table while every coordinate
    // t = kex8 rho - 1/2 of the data stays below kBesselIntervals - 3/2 (one
    // interval of margin for the rounding of the products)
    c.bigx = !(fmaxf(kex8, kin8) * cta.model_f < (float)(kBesselIntervals - 1));
    c.pad[0] = c.pad[1] = c.pad[2] = 0;
  }

  // chi^2 of every active replica over all data (both passes).  The phase
  // storage mode and the need for the out-of-table Bessel path are uniform
  // over the CTA: each combination is its own straight-line loop.  The
  // table-only loop runs when no local replica, active or not (the inactive
  // ones are evaluated too, with their last or zeroed constants), reaches
  // beyond the table: its lookups need no index check.
  template <int R, class Cta>
  __device__ static void eval(Cta &cta, float (&acc)[R])
  {
    bool big = false;
#pragma unroll
    for (int r = 0; r < R; ++r) big |= (cta.consts[r].bigx != 0);
    if (cta.pk->phasor == 1) {
      if (big) eval_impl<R, true, true, false>(cta, acc);
      else eval_impl<R, true, false, false>(cta, acc);
    } else if (cta.pk->phasor == 0) {
      if (big) eval_impl<R, false, true, false>(cta, acc);
      else eval_impl<R, false, false, false>(cta, acc);
    } else {
      if (big) eval_impl<R, false, true, true>(cta, acc);
      else eval_impl<R, false, false, true>(cta, acc);
    }
  }

  // PH: unit phasors (else phases); GL: phases in global memory.
  template <int R, bool PH, bool BIG, bool GL, class Cta>
  __device__ static void eval_impl(Cta &cta, float (&acc)[R])
  {
    const Packed &pk = *cta.pk;
    const int tid = cta.tid, T = cta.nthreads, npts = pk.npts;
    const float4 *btab = reinterpret_cast<const float4 *>(cta.scratch);
    float *zs = GL ? pk.gph + (size_t)cta.ph_region * npts : cta.scratch + kTabBytes / 4;
    float2 *z = reinterpret_cast<float2 *>(zs);
    const unsigned long long pol = GL ? l2_evict_last_policy() : 0ull;
#if !CMC_BRANCHFREE
    bool act[R];
#pragma unroll
    for (int r = 0; r < R; ++r) act[r] = cta.flag[r] != 0;
#endif
    // Every local replica is evaluated (branch-free); the sums of the
    // inactive ones (flag 0) are never read, so their terms need no mask.
#pragma unroll
    for (int r = 0; r < R; ++r) acc[r] = 0.0f;
    // One model term per (point, replica); the points are packed closure
    // corners first, so only the first nused need a phase: each thread walks
    // its stride through [0, nused) with phases, then on without.
    auto terms = [&](int i, const float4 d, const float rho, auto with_phase) {
#pragma unroll
      for (int r = 0; r < R; ++r) {
#if !CMC_BRANCHFREE
        if (!act[r]) continue;
#endif
        const float2 V = sgra_vis<BIG>(cta.consts[r], btab, d.x, d.y, rho);
        const float n2 = fmaf(V.x, V.x, V.y * V.y);
        if (PH) {
          const float rs = (n2 > 0.0f) ? rsqrt_ftz(n2) : 0.0f;
          const float dif = fmaf(-n2, rs, d.z);
          acc[r] = fmaf(dif * dif, d.w, acc[r]);
          if constexpr (decltype(with_phase)::value)
            z[r * npts + i] = (n2 > 0.0f) ? make_float2(V.x * rs, V.y * rs)
                                          : make_float2(1.f, 0.f);
        } else {
          // |V| = n2 / sqrt(n2), n2 held off zero (and denormals): |V| -> 0
          const float dif = fmaf(-n2, rsqrt_ftz(fmaxf(n2, 1e-30f)), d.z);
          acc[r] = fmaf(dif * dif, d.w, acc[r]);
          if constexpr (decltype(with_phase)::value)
            store_phase<GL>(&zs[r * npts + i], atan2_poly(V.y, V.x), pol);
        }
      }
    };
    // The next point's data is loaded one iteration ahead (its L2 latency
    // overlaps this point's terms when the data set outgrows L1), two ahead
    // with phases in global memory and up to 4 replicas per CTA (large data
    // sets, whose points stream from L2 behind the phase traffic, at the
    // replica counts where the registers allow it).
    constexpr int kAhead = (GL && R <= 4) ? 2 : 1;
    const int nused = cta.model_i;
    int i = tid;
    float4 dn[kAhead];
    float rn[kAhead];
#pragma unroll
    for (int a = 0; a < kAhead; ++a) {
      dn[a] = make_float4(0.f, 0.f, 0.f, 0.f);
      rn[a] = 0.0f;
      if (i + a * T < npts) {
        dn[a] = __ldg(&pk.vis[i + a * T]);
        rn[a] = __ldg(&pk.rho[i + a * T]);
      }
    }
    auto next = [&](int i, float4 &d, float &rho) {
      d = dn[0];
      rho = rn[0];
#pragma unroll
      for (int a = 0; a + 1 < kAhead; ++a) {
        dn[a] = dn[a + 1];
        rn[a] = rn[a + 1];
      }
      if (i + kAhead * T < npts) {
        dn[kAhead - 1] = __ldg(&pk.vis[i + kAhead * T]);
        rn[kAhead - 1] = __ldg(&pk.rho[i + kAhead * T]);
      }
    };
    for (; i < nused; i += T) {
      float4 d;
      float rho;
      next(i, d, rho);
      terms(i, d, rho, std::true_type{});
    }
    for (; i < npts; i += T) {
      float4 d;
      float rho;
      next(i, d, rho);
      terms(i, d, rho, std::false_type{});
    }
    if (pk.ncph == 0 || pk.npass < 2) return;
    __syncthreads();   // also orders the global phase stores before the reads (GL)
    // closure indices and data one closure ahead, likewise
    int4 qn = make_int4(0, 0, 0, 0);
    float4 fn = make_float4(0.f, 0.f, 0.f, 0.f);
    if (tid < pk.ncph) {
      qn = __ldg(&pk.cli[tid]);
      fn = __ldg(&pk.clf[tid]);
    }
    for (int c = tid; c < pk.ncph; c += T) {
      const int4 q = qn;
      const float4 f = fn;
      if (c + T < pk.ncph) {
        qn = __ldg(&pk.cli[c + T]);
        fn = __ldg(&pk.clf[c + T]);
      }
#pragma unroll
      for (int r = 0; r < R; ++r) {
#if !CMC_BRANCHFREE
        if (!act[r]) continue;
#endif
        float dif;
        if (PH) {
          const float2 a = z[r * npts + q.x], b = z[r * npts + q.y], e = z[r * npts + q.z];
          // m = a * b * conj(e): model closure phasor
          const float abr = fmaf(a.x, b.x, -(a.y * b.y)), abi = fmaf(a.x, b.y, a.y * b.x);
          const float mr = fmaf(abr, e.x, abi * e.y), mi = fmaf(abi, e.x, -(abr * e.y));
          // residual phasor e^{i obs} * conj(m)
          dif = atan2_poly(fmaf(f.y, mr, -(f.x * mi)), fmaf(f.x, mr, f.y * mi));
        } else {
          const float x = f.w - (load_phase<GL>(&zs[r * npts + q.x], pol) +
                                 load_phase<GL>(&zs[r * npts + q.y], pol) -
                                 load_phase<GL>(&zs[r * npts + q.z], pol));
          dif = fmaf(-6.2831853071795865f, rintf(x * 0.15915494309189535f), x);
        }
        acc[r] = fmaf(dif * dif, f.z, acc[r]);
      }
    }
  }

  // calc_model (pass 0 only): amplitudes into datm[ist*ndat + i] and phases
  // into the tail datm[nchi2m + ist*nvis + i] (src/gpu_mcmc.cu:633-658).
  template <int R, class Cta>
  __device__ static void model_rows(Cta &cta, const int *flags)
  {
    const cmc_job &job = *cta.job;
    const Packed &pk = *cta.pk;
    const float4 *btab = reinterpret_cast<const float4 *>(cta.scratch);
    const int tid = cta.tid, T = cta.nthreads, nvis = pk.nvis, ndat = pk.ndat;
    const size_t nchi2m = (size_t)job.nbeta * job.nseq * ndat;
    for (int i = tid; i < pk.npts; i += T) {
      const int o = __ldg(&pk.orig[i]);
      if (o >= nvis) continue;
      const float4 d = __ldg(&pk.vis[i]);
      const float rho = __ldg(&pk.rho[i]);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if (!flags[r]) continue;
        const size_t ist = (size_t)cta.ist[r];
        const float2 V = sgra_vis(cta.consts[r], btab, d.x, d.y, rho);
        job.datm[ist * ndat + o] = sqrtf(fmaf(V.x, V.x, V.y * V.y));
        job.datm[nchi2m + ist * nvis + o] = atan2f(V.y, V.x);
      }
    }
  }

  // datm / chi2m rows of each replica's last evaluation, reference layout:
  // datm[ist*ndat + id] amplitudes and closures, datm[nchi2m + ist*nvis + i]
  // phases (model.cuh:38-43), chi2m[ist*ndat + id] terms (gpu_mcmc.cu:305-323).
  template <int R, class Cta>
  __device__ static void final_rows(Cta &cta, const float *plast, const int *evald)
  {
    const cmc_job &job = *cta.job;
    const Packed &pk = *cta.pk;
    if (job.datm == nullptr || job.chi2m == nullptr) return;
    const float4 *btab = reinterpret_cast<const float4 *>(cta.scratch);
    const int tid = cta.tid, T = cta.nthreads, npts = pk.npts, nvis = pk.nvis;
    const int ndat = pk.ndat, nptot = job.nptot;
    const size_t nchi2m = (size_t)job.nbeta * job.nseq * ndat;
    float *ph = phase_area(cta);               // phases [R][npts]
    __syncthreads();
    if (tid < R && evald[tid]) prepare(cta, tid, plast + tid * nptot);
    __syncthreads();
    for (int i = tid; i < npts; i += T) {
      const float4 d = __ldg(&pk.vis[i]);
      const float rho = __ldg(&pk.rho[i]);
      const int o = __ldg(&pk.orig[i]);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if (!evald[r]) continue;
        const float2 V = sgra_vis(cta.consts[r], btab, d.x, d.y, rho);
        const float amp = sqrtf(fmaf(V.x, V.x, V.y * V.y));
        const float phase = atan2f(V.y, V.x);
        ph[r * npts + i] = phase;
        if (o < nvis) {
          const size_t ist = (size_t)cta.ist[r];
          const float dif = d.z - amp;
          job.datm[ist * ndat + o] = amp;
          job.datm[nchi2m + ist * nvis + o] = phase;
          job.chi2m[ist * ndat + o] = (dif * dif) * d.w;
        }
      }
    }
    if (pk.ncph == 0 || pk.npass < 2) return;
    __syncthreads();
    for (int c = tid; c < pk.ncph; c += T) {
      const int4 q = __ldg(&pk.cli[c]);
      const float4 f = __ldg(&pk.clf[c]);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if (!evald[r]) continue;
        const size_t ist = (size_t)cta.ist[r];
        const float cph = ph[r * npts + q.x] + ph[r * npts + q.y] - ph[r * npts + q.z];
        const float m = atan2f(sinf(cph), cosf(cph));
        float dif = f.w - m;
        dif = atan2f(sinf(dif), cosf(dif));
        job.datm[ist * ndat + nvis + c] = m;
        job.chi2m[ist * ndat + nvis + c] = (dif * dif) * f.z;
      }
    }
  }
};

#ifndef CMC_INSTANCE_TU
// ---- packing: reference layout -> |uv|-sorted fast-path arrays ------------

// Points in the caller's order: visibilities (coor = [u0,v0,u1,v1,...], dat,
// std2r) and, for cpExt == 1, the three corners of each closure triangle
// ([u1,v1,u2,v2] per closure after the visibilities; u3 = -(u1+u2),
// v3 = -(v1+v2), model.cuh:88-94) with zero amplitude weight.  key = |uv|
// (NaN -> +inf so that the order stays total).
__global__ void sgra_points_kernel(const float *coor, const float *dat, const float *std2r,
                                   int nvis, int ncph, int cpext, float4 *raw, float *key)
{
  const int npts = nvis + (cpext ? 3 * ncph : 0);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npts; i += gridDim.x * blockDim.x) {
    float u, v, a = 0.0f, w = 0.0f;
    if (i < nvis) {
      u = coor[2 * i]; v = coor[2 * i + 1]; a = dat[i]; w = std2r[i];
    } else {
      const int c = (i - nvis) / 3, t = (i - nvis) - 3 * c;
      const int o = 2 * nvis + 4 * c;
      if (t == 0) { u = coor[o]; v = coor[o + 1]; }
      else if (t == 1) { u = coor[o + 2]; v = coor[o + 3]; }
      else { u = -(coor[o] + coor[o + 2]); v = -(coor[o + 1] + coor[o + 3]); }
    }
    raw[i] = make_float4(u, v, a, w);
    const float rho = sqrtf(u * u + v * v);
    key[i] = (rho == rho) ? rho : __int_as_float(0x7f800000);
  }
}

// used[p] = 1 for every point a closure phase reads: the three visibilities
// of each triangle (cpExt = 0) or the triangle corners (cpExt = 1).
// Out-of-range indices are skipped here (the scatter reports them).
__global__ void sgra_mark_kernel(const int *icoor, int nvis, int ncph, int cpext, int *used)
{
  const int npts = nvis + (cpext ? 3 * ncph : 0);
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncph; c += gridDim.x * blockDim.x) {
    if (cpext) {
      used[nvis + 3 * c] = used[nvis + 3 * c + 1] = used[nvis + 3 * c + 2] = 1;
    } else {
      for (int t = 0; t < 3; ++t) {
        const int a = icoor[3 * c + t];
        if (a >= 0 && a < npts) used[a] = 1;
      }
    }
  }
}

// newpos[i] = rank of (!used[i], key[i], i) in lexicographic order: closure
// corners first, each group by |uv|; a deterministic total order, so the
// packing is identical from run to run.
__global__ void rank_kernel(const float *key, const int *used, int n, int *newpos)
{
  __shared__ float tile[256];
  __shared__ int utile[256];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const float ki = (i < n) ? key[i] : 0.0f;
  const int ui = (i < n && used[i]) ? 0 : 1;
  int cnt = 0;
  for (int base = 0; base < n; base += 256) {
    const int j = base + threadIdx.x;
    tile[threadIdx.x] = (j < n) ? key[j] : 0.0f;
    utile[threadIdx.x] = (j < n && used[j]) ? 0 : 1;
    __syncthreads();
    const int m = min(256, n - base);
    for (int t = 0; t < m; ++t) {
      const float kj = tile[t];
      const int uj = utile[t];
      cnt += (uj < ui) || (uj == ui && ((kj < ki) || (kj == ki && base + t < i)));
    }
    __syncthreads();
  }
  if (i < n) newpos[i] = cnt;
}

__global__ void sgra_scatter_kernel(const float4 *raw, const float *key, const int *newpos,
                                    const int *used, int npts, const int *icoor,
                                    const float *dat, const float *std2r, int nvis, int ncph,
                                    int cpext, float4 *vis, float *rho, int *orig, int4 *cli,
                                    float4 *clf, int *aux, int *status)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npts + ncph;
       i += gridDim.x * blockDim.x) {
    if (i < npts) {
      const int p = newpos[i];
      vis[p] = raw[i];
      rho[p] = key[i];
      orig[p] = i;
      if (used[i]) atomicAdd(&aux[0], 1);
      atomicMax(&aux[1], __float_as_int(key[i]));   // keys are >= 0 (or +inf)
    } else {
      const int c = i - npts;
      int a, b, e;
      if (cpext) {
        a = nvis + 3 * c; b = a + 1; e = a + 2;
      } else {
        a = icoor[3 * c]; b = icoor[3 * c + 1]; e = icoor[3 * c + 2];
        if (a < 0 || a >= nvis || b < 0 || b >= nvis || e < 0 || e >= nvis) {
          if (status) atomicCAS(status, 0, (int)CMC_ERR_ARG);
          a = b = e = 0;
        }
      }
      const float obs = dat[nvis + c];
      float so, co;
      sincosf(obs, &so, &co);
      cli[c] = make_int4(newpos[a], newpos[b], newpos[e], 0);
      clf[c] = make_float4(co, so, std2r[nvis + c], obs);
    }
  }
}

int SgraModel::host_pack(const cmc_job &j, Packed &pk, void *work, cudaStream_t s)
{
  unsigned char *w = (unsigned char *)work;
  const size_t n = (size_t)pk.npts, nc = (size_t)pk.ncph;
  auto al = [](size_t x) { return (x + 15) & ~(size_t)15; };
  size_t o = 0;
  float4 *vis = (float4 *)(w + o); o += al(16 * n);
  float *rho = (float *)(w + o);   o += al(4 * n);
  int *orig = (int *)(w + o);      o += al(4 * n);
  int4 *cli = (int4 *)(w + o);     o += al(16 * nc);
  float4 *clf = (float4 *)(w + o); o += al(16 * nc);
  float4 *raw = (float4 *)(w + o); o += al(16 * n);
  float *key = (float *)(w + o);   o += al(4 * n);
  int *newpos = (int *)(w + o);    o += al(4 * n);
  int *used = (int *)(w + o);      o += al(4 * n);
  int *aux = (int *)(w + o);
  pk.vis = vis; pk.rho = rho; pk.orig = orig; pk.cli = cli; pk.clf = clf; pk.aux = aux;
  if (cudaMemsetAsync(aux, 0, 4 * sizeof(int), s) != cudaSuccess) return CMC_ERR_CUDA;
  if (n == 0) return CMC_OK;
  if (cudaMemsetAsync(used, 0, 4 * n, s) != cudaSuccess) return CMC_ERR_CUDA;
  const int blocks = (int)std::min<size_t>((n + nc + 255) / 256, 4096);
  sgra_points_kernel<<<blocks, 256, 0, s>>>(j.coor, j.dat, j.std2r, pk.nvis, pk.ncph, pk.cpext,
                                            raw, key);
  if (nc > 0)
    sgra_mark_kernel<<<(unsigned)std::min<size_t>((nc + 255) / 256, 4096), 256, 0, s>>>(
        j.icoor, pk.nvis, pk.ncph, pk.cpext, used);
  rank_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(key, used, (int)n, newpos);
  sgra_scatter_kernel<<<blocks, 256, 0, s>>>(raw, key, newpos, used, (int)n, j.icoor, j.dat,
                                             j.std2r, pk.nvis, pk.ncph, pk.cpext, vis, rho, orig,
                                             cli, clf, aux, j.status);
  return cudaGetLastError() == cudaSuccess ? CMC_OK : CMC_ERR_CUDA;
}
#endif  // CMC_INSTANCE_TU

}  // namespace cmc
