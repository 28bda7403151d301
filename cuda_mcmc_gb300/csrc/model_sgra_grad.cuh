// model_sgra_grad.cuh -- hand-written adjoint of the Sgr A* model + chi^2.
//
// chi^2(p) = sum_i w_i (a_i - |V_i|)^2 + sum_c w_c wrap(obs_c - (phi_i + phi_j - phi_k))^2
// (the terms of src/gpu_mcmc.cu:305-323 with the model of
// examples/sgra_model_fit/model.cuh), differentiated with respect to the
// parameters p:
//   1. the 17 per-replica constants C(p) of the visibility formula
//      (sgra_consts_t, the same algebra as SgraModel::prepare) are
//      differentiated in forward mode (dual numbers, one direction per
//      parameter) -> dC/dp;
//   2. a forward pass over the data gives V_i, the amplitude residual adjoint
//      A_bar_i = -2 w_i (a_i - |V_i|) and the phases phi_i;
//   3. a pass over the closures gives d_c and scatters the phase adjoints
//      phi_bar (-2 w_c d_c to i and j, +2 w_c d_c to k);
//   4. a reverse sweep per point through V(C) (sgra_vis_bwd) accumulates
//      C_bar = sum_i dV_i/dC^T (Vre_bar, Vim_bar), with
//      Vre_bar = A_bar Vre/|V| - phi_bar Vim/|V|^2, Vim_bar = A_bar Vim/|V| + phi_bar Vre/|V|^2;
//   5. dchi^2/dp = dC/dp^T C_bar.
// Bessel derivatives: F1' = -x F2 and F2' = -x F3 with F3(x) = J3(x)/x^3.
#pragma once
#include "model_sgra.cuh"

namespace cmc {

// ---- forward-mode dual numbers (value, derivative along one direction) -----
struct Dual {
  float v, d;
};
__device__ __forceinline__ Dual dual(float v, float d = 0.0f) { return Dual{v, d}; }
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Dual operator-(Dual a) { return {-a.v, -a.d}; }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
__device__ __forceinline__ Dual operator/(Dual a, Dual b)
{
  const float q = a.v / b.v;
  return {q, (a.d - q * b.d) / b.v};
}
__device__ __forceinline__ Dual operator/(Dual a, float s) { return {a.v / s, a.d / s}; }
__device__ __forceinline__ Dual operator*(float s, Dual a) { return {s * a.v, s * a.d}; }
__device__ __forceinline__ Dual operator*(Dual a, float s) { return {s * a.v, s * a.d}; }
__device__ __forceinline__ Dual operator+(Dual a, float s) { return {a.v + s, a.d}; }
__device__ __forceinline__ Dual operator+(float s, Dual a) { return {a.v + s, a.d}; }
__device__ __forceinline__ Dual operator-(float s, Dual a) { return {s - a.v, -a.d}; }
__device__ __forceinline__ Dual operator-(Dual a, float s) { return {a.v - s, a.d}; }
__device__ __forceinline__ Dual operator/(float s, Dual a)
{
  const float q = s / a.v;
  return {q, -q * a.d / a.v};
}
__device__ __forceinline__ void dsincos(Dual a, Dual *s, Dual *c)
{
  float sv, cv;
  sincosf(a.v, &sv, &cv);
  *s = {sv, cv * a.d};
  *c = {cv, -sv * a.d};
}
__device__ __forceinline__ Dual dcos(Dual a)
{
  Dual s, c;
  dsincos(a, &s, &c);
  return c;
}
__device__ __forceinline__ float val(float x) { return x; }
__device__ __forceinline__ float val(Dual x) { return x.v; }
__device__ __forceinline__ void dsincos(float a, float *s, float *c) { sincosf(a, s, c); }
__device__ __forceinline__ float dcos(float a) { return cosf(a); }

// most parameters a gradient call handles (sgra_model13 has 13)
constexpr int kMaxGradParams = 16;

// order of the per-replica constants in the vector C
enum SgraC { kCth, kSth, kKex, kKin, kAe, kBe, kAi, kBi, kDsh, kGc, kGs, kGx, kGy, kGpu, kGpv,
             kZr, kZg, kNC };

// The constants of SgraModel::prepare for scalar type S (float or Dual).
template <class S>
__device__ void sgra_consts_t(const S *p, int im, S (&c)[kNC], int &inner, int &gauss,
                              int &ring)
{
  const float pi = 3.1415926535897931f;
  const S zero = S{}, Zsp = p[0], Re = p[1], rq = p[2], ecc = p[3], fade = p[4];
  S gr = zero, gax, aq, gq, alpha = zero, beta = zero, eta = zero, th;
  if (im == 1) {
    gax = p[5]; aq = p[6]; gq = p[7]; th = p[8];
  } else {
    gr = p[5]; gax = p[6]; aq = p[7]; gq = p[8];
    alpha = p[9]; beta = p[10]; eta = p[11]; th = p[12];
  }
  const S Rex = (pi / 180.0f) * (Re / 3600.0f) * 1e3f;   // uas -> nrad
  const S Rin = rq * Rex;
  S d = ecc * (Rex - Rin);
  if (im != 1) d = d * dcos(eta - th);
  const S h = (2.0f / pi) / ((Rex * Rex - Rin * Rin * (1.0f + d / Rex)) * fade
                             + (Rex * Rex - Rin * Rin * (1.0f - d / Rex)));
  const S h0 = fade * h;
  dsincos(th, &c[kSth], &c[kCth]);
  c[kKex] = (2.0f * pi) * Rex;
  c[kKin] = (2.0f * pi) * Rin;
  c[kAe] = 0.5f * (h + h0) * Rex * c[kKex];
  c[kBe] = -((h - h0) / (4.0f * pi)) * (c[kKex] * c[kKex] * c[kKex]);
  inner = (val(Rin) != 0.0f);
  c[kAi] = inner ? 0.5f * (h + h0 - d * (h - h0) / Rex) * Rin * c[kKin] : zero;
  c[kBi] = inner ? -((h - h0) / (4.0f * pi)) * rq * (c[kKin] * c[kKin] * c[kKin]) : zero;
  c[kDsh] = 2.0f * d;
  const float gcoef = 3.5597039f;
  const S gsy = gax * Rex, gsx = aq * gsy;
  c[kGx] = gcoef * gsx * gsx;
  c[kGy] = gcoef * gsy * gsy;
  gauss = !(val(gax) == 0.0f || val(aq) == 0.0f || val(gq) == 0.0f);
  if (im == 1) {
    const S gshift = Rin - d;
    c[kGc] = c[kCth];
    c[kGs] = c[kSth];
    c[kGpu] = -2.0f * gshift * c[kCth];
    c[kGpv] = -2.0f * gshift * c[kSth];
  } else {
    S sa, ca;
    dsincos(beta, &c[kGs], &c[kGc]);
    dsincos(alpha, &sa, &ca);
    c[kGpu] = -2.0f * gr * Rex * ca;
    c[kGpv] = -2.0f * gr * Rex * sa;
  }
  if (gauss) {
    c[kZr] = Zsp * (1.0f - gq);
    c[kZg] = Zsp * gq;
  } else {
    c[kZr] = Zsp;
    c[kZg] = zero;
  }
  ring = 1;
  if (im != 1 && val(gq) == 1.0f) {
    ring = 0;
    c[kZg] = Zsp;
    gauss = !(val(gax) == 0.0f || val(aq) == 0.0f);
  }
  if (!gauss) c[kZg] = zero;
}

// F3 = J3(x)/x^3 from its table (row-major coefficients a_0..a_deg per
// interval); beyond the table J3 = 4 J2/x - J1.
__device__ __forceinline__ float bessel_f3_tab(const float *tab3, float x)
{
  x = fabsf(x);
  if (x < (float)kBesselXmax) {
    const float xs = x * (float)kBesselSub;
    const int i = min((int)xs, kBesselIntervals - 1);
    const float d = xs - ((float)i + 0.5f);
    const float *c = tab3 + i * (kBesselDeg + 1);
    float p = c[kBesselDeg];
#pragma unroll
    for (int k = kBesselDeg - 1; k >= 0; --k) p = fmaf(p, d, c[k]);
    return p;
  }
  const float ix = 1.0f / x;
  const float j0 = j0f(x), j1 = j1f(x);
  const float j2 = 2.0f * j1 * ix - j0;
  return (4.0f * j2 * ix - j1) * ix * ix * ix;
}

// sgra_vis with accurate sin / cos / exp (the forward pass of the gradient).
__device__ __forceinline__ void sgra_vis_acc(const SgraConsts &c, int ring, const float4 *btab,
                                             float u, float v, float rho, float2 &V)
{
  const float U = fmaf(u, c.cth, v * c.sth);
  float f1, f2, g1, g2, sd, cd;
  bessel_f12_tab<true>(btab, c.kex * rho, f1, f2);
  bessel_f12_tab<true>(btab, c.kin * rho, g1, g2);
  sincospif(c.dsh * U, &sd, &cd);
  const float rei = c.ai * g1, imi = c.bi * g2 * U;
  const float re = c.ae * f1 - (rei * cd - imi * sd);
  const float im = c.be * f2 * U - (rei * sd + imi * cd);
  float vre = ring ? c.zr * re : 0.0f;
  float vim = ring ? c.zr * im : 0.0f;
  const float ug = fmaf(u, c.gc, v * c.gs), vg = fmaf(v, c.gc, -u * c.gs);
  const float ga = c.zg * expf(-fmaf(c.gx * ug, ug, c.gy * vg * vg));
  float sg, cg;
  sincospif(fmaf(c.gpu, u, c.gpv * v), &sg, &cg);
  V.x = fmaf(ga, cg, vre);
  V.y = fmaf(ga, sg, vim);
}

// Reverse sweep of sgra_vis for one point: adds dV/dC^T (vre_bar, vim_bar) to cb.
__device__ __forceinline__ void sgra_vis_bwd(const float (&C)[kNC], int ring, const float4 *btab,
                                             const float *tab3, float u, float v, float rho,
                                             float vre_bar, float vim_bar, float (&cb)[kNC])
{
  const float pi = 3.14159265358979324f;
  // forward intermediates (accurate sin/cos: this is a checking / Fisher path)
  const float U = fmaf(u, C[kCth], v * C[kSth]);
  const float xe = C[kKex] * rho, xi = C[kKin] * rho;
  float f1, f2, g1, g2;
  bessel_f12_tab<true>(btab, xe, f1, f2);
  bessel_f12_tab<true>(btab, xi, g1, g2);
  const float f3 = bessel_f3_tab(tab3, xe), g3 = bessel_f3_tab(tab3, xi);
  float sd, cd;
  sincospif(C[kDsh] * U, &sd, &cd);
  const float rei = C[kAi] * g1, imi = C[kBi] * g2 * U;
  const float re = C[kAe] * f1 - (rei * cd - imi * sd);
  const float im = C[kBe] * f2 * U - (rei * sd + imi * cd);
  const float ug = fmaf(u, C[kGc], v * C[kGs]), vg = fmaf(v, C[kGc], -u * C[kGs]);
  const float E = expf(-fmaf(C[kGx] * ug, ug, C[kGy] * vg * vg));
  const float psi = fmaf(C[kGpu], u, C[kGpv] * v);
  float sg, cg;
  sincospif(psi, &sg, &cg);
  // Gaussian: Vre += zg E cg, Vim += zg E sg
  const float ga_bar = vre_bar * cg + vim_bar * sg;
  const float ga = C[kZg] * E;
  const float psi_bar = (-vre_bar * sg + vim_bar * cg) * ga * pi;   // d(sin, cos)/d(pi psi)
  cb[kGpu] += psi_bar * u;
  cb[kGpv] += psi_bar * v;
  cb[kZg] += ga_bar * E;
  const float q_bar = -ga_bar * C[kZg] * E;
  cb[kGx] += q_bar * ug * ug;
  cb[kGy] += q_bar * vg * vg;
  const float ug_bar = q_bar * 2.0f * C[kGx] * ug, vg_bar = q_bar * 2.0f * C[kGy] * vg;
  cb[kGc] += ug_bar * u + vg_bar * v;
  cb[kGs] += ug_bar * v - vg_bar * u;
  if (!ring) return;
  // ring: Vre += zr re, Vim += zr im
  cb[kZr] += vre_bar * re + vim_bar * im;
  const float re_bar = vre_bar * C[kZr], im_bar = vim_bar * C[kZr];
  float U_bar = 0.0f;
  cb[kAe] += re_bar * f1;
  const float f1_bar = re_bar * C[kAe];
  cb[kBe] += im_bar * f2 * U;
  const float f2_bar = im_bar * C[kBe] * U;
  U_bar += im_bar * C[kBe] * f2;
  const float rei_bar = -re_bar * cd - im_bar * sd;
  const float imi_bar = re_bar * sd - im_bar * cd;
  const float cd_bar = -re_bar * rei - im_bar * imi;
  const float sd_bar = re_bar * imi - im_bar * rei;
  cb[kAi] += rei_bar * g1;
  const float g1_bar = rei_bar * C[kAi];
  cb[kBi] += imi_bar * g2 * U;
  const float g2_bar = imi_bar * C[kBi] * U;
  U_bar += imi_bar * C[kBi] * g2;
  const float th_bar = (sd_bar * cd - cd_bar * sd) * pi;            // theta = pi dsh U
  cb[kDsh] += th_bar * U;
  U_bar += th_bar * C[kDsh];
  const float xe_bar = -xe * (f1_bar * f2 + f2_bar * f3);
  const float xi_bar = -xi * (g1_bar * g2 + g2_bar * g3);
  cb[kKex] += xe_bar * rho;
  cb[kKin] += xi_bar * rho;
  cb[kCth] += U_bar * u;
  cb[kSth] += U_bar * v;
}

// Per-CTA prologue of the gradient and Fisher kernels for replica ist: the
// Bessel tables into shared memory, the constants C and their Jacobian
// dC/dp [kNC][nptot] (forward mode, thread k < nptot differentiates along
// parameter k).  Layout of the dynamic shared memory: btab | tab3 | C [kNC] |
// jac [kNC][nptot] | p [kMaxGradParams] | flags [3] | rest (returned).
struct GradCta {
  const float4 *btab;
  const float *tab3;
  const float *jac;
  float C[kNC];
  SgraConsts sc;
  int ring;
  float *rest;
};

__device__ inline GradCta grad_prologue(const cmc_job &job, const SgraModel::Packed &pk, int ist,
                                        unsigned char *smem)
{
  const int tid = threadIdx.x, T = blockDim.x, nptot = job.nptot;
  float4 *btab = reinterpret_cast<float4 *>(smem);
  const int ntab = kBesselIntervals * ((kBesselDeg + 1) / 2);
  float *tab3 = reinterpret_cast<float *>(btab + ntab);
  float *Cs = tab3 + kBesselIntervals * (kBesselDeg + 1);
  float *jac = Cs + kNC;
  float *s_p = jac + kNC * nptot;
  int *s_flags = reinterpret_cast<int *>(s_p + kMaxGradParams);
  for (int i = tid; i < ntab; i += T) btab[i] = (&kBesselTab[0][0])[i];
  for (int i = tid; i < kBesselIntervals * (kBesselDeg + 1); i += T)
    tab3[i] = (&kBesselTab3[0][0])[i];
  for (int i = tid; i < nptot; i += T) s_p[i] = job.pcur[(size_t)ist * nptot + i];
  __syncthreads();
  if (tid < nptot) {
    Dual pd[kMaxGradParams];
#pragma unroll
    for (int j = 0; j < kMaxGradParams; ++j)
      pd[j] = dual(j < nptot ? s_p[j] : 0.0f, j == tid ? 1.0f : 0.0f);
    Dual cd[kNC];
    int inner, gauss, ring;
    sgra_consts_t<Dual>(pd, pk.imodel, cd, inner, gauss, ring);
    for (int j = 0; j < kNC; ++j) jac[j * nptot + tid] = cd[j].d;
    if (tid == 0) {
      for (int j = 0; j < kNC; ++j) Cs[j] = cd[j].v;
      s_flags[0] = inner;
      s_flags[1] = gauss;
      s_flags[2] = ring;
    }
  }
  __syncthreads();
  GradCta g;
  g.btab = btab;
  g.tab3 = tab3;
  g.jac = jac;
#pragma unroll
  for (int j = 0; j < kNC; ++j) g.C[j] = Cs[j];
  g.ring = s_flags[2];
  SgraConsts &sc = g.sc;
  sc.cth = g.C[kCth]; sc.sth = g.C[kSth]; sc.kex = g.C[kKex]; sc.kin = g.C[kKin];
  sc.ae = g.C[kAe]; sc.be = g.C[kBe]; sc.ai = g.C[kAi]; sc.bi = g.C[kBi]; sc.dsh = g.C[kDsh];
  sc.gc = g.C[kGc]; sc.gs = g.C[kGs]; sc.gx = g.C[kGx]; sc.gy = g.C[kGy]; sc.gpu = g.C[kGpu];
  sc.gpv = g.C[kGpv]; sc.zr = g.C[kZr]; sc.zg = g.C[kZg];
  sc.inner = s_flags[0]; sc.gauss = s_flags[1]; sc.ring = g.ring; sc.bigx = 1;
  g.rest = reinterpret_cast<float *>(s_flags + 4);
  return g;
}

inline size_t grad_prologue_floats(int nptot)
{
  return (size_t)kBesselIntervals * ((kBesselDeg + 1) / 2) * 4 +
         (size_t)kBesselIntervals * (kBesselDeg + 1) + kNC + (size_t)kNC * nptot +
         kMaxGradParams + 4;
}

// One CTA per replica (ist = blockIdx.x): chi^2 and dchi^2/dp.  Shared
// memory: the prologue, then the reductions [kNC + 1][NW]; per-point phases
// and adjoints live in gwork[ist][3][npts] (global).
__global__ void __launch_bounds__(256) sgra_grad_kernel(const cmc_job job,
                                                        const SgraModel::Packed pk, float *grad,
                                                        float *gwork)
{
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x, T = blockDim.x, NW = T >> 5, lane = tid & 31, warp = tid >> 5;
  const int ist = blockIdx.x, nptot = job.nptot, npts = pk.npts;
  const bool active = job.flag == nullptr || job.flag[ist] != 0;
  if (!active) {   // uniform over the CTA
    for (int k = tid; k < nptot; k += T) grad[(size_t)ist * nptot + k] = 0.0f;
    if (tid == 0) job.chi2c[ist] = 0.0f;
    return;
  }
  const GradCta g = grad_prologue(job, pk, ist, smem);
  float *red = g.rest;                                        // [kNC + 1][NW]
  float *ph = gwork + (size_t)ist * 3 * npts;                 // [npts] phases
  float *abar = ph + npts;                                    // [npts] d chi2 / d|V|
  float *pbar = abar + npts;                                  // [npts] d chi2 / d phase
  float c2 = 0.0f;
  // pass A: amplitude terms, amplitude adjoints, phases
  for (int i = tid; i < npts; i += T) {
    const float4 d = __ldg(&pk.vis[i]);
    const float rho = __ldg(&pk.rho[i]);
    float2 V;
    sgra_vis_acc(g.sc, g.ring, g.btab, d.x, d.y, rho, V);
    const float A = sqrtf(fmaf(V.x, V.x, V.y * V.y));
    const float r = d.z - A;
    c2 = fmaf(r * r, d.w, c2);
    abar[i] = -2.0f * d.w * r;
    ph[i] = atan2f(V.y, V.x);
    pbar[i] = 0.0f;
  }
  __syncthreads();
  // pass B: closure terms; phase adjoints (-2 w d to i and j, +2 w d to k)
  if (pk.npass >= 2) {
    for (int c = tid; c < pk.ncph; c += T) {
      const int4 q = __ldg(&pk.cli[c]);
      const float4 f = __ldg(&pk.clf[c]);
      const float x = f.w - (ph[q.x] + ph[q.y] - ph[q.z]);
      const float dw = fmaf(-6.2831853071795865f, rintf(x * 0.15915494309189535f), x);
      c2 = fmaf(dw * dw, f.z, c2);
      const float gg = -2.0f * f.z * dw;
      atomicAdd(&pbar[q.x], gg);
      atomicAdd(&pbar[q.y], gg);
      atomicAdd(&pbar[q.z], -gg);
    }
  }
  __syncthreads();
  // pass C: reverse sweep per point
  float cb[kNC];
#pragma unroll
  for (int j = 0; j < kNC; ++j) cb[j] = 0.0f;
  for (int i = tid; i < npts; i += T) {
    const float4 d = __ldg(&pk.vis[i]);
    const float rho = __ldg(&pk.rho[i]);
    const float ab = abar[i], pb = pbar[i];
    if (ab == 0.0f && pb == 0.0f) continue;
    float2 V;
    sgra_vis_acc(g.sc, g.ring, g.btab, d.x, d.y, rho, V);
    const float n2 = fmaf(V.x, V.x, V.y * V.y);
    if (!(n2 > 0.0f)) continue;
    const float A = sqrtf(n2);
    const float vre_bar = ab * V.x / A - pb * V.y / n2;
    const float vim_bar = ab * V.y / A + pb * V.x / n2;
    sgra_vis_bwd(g.C, g.ring, g.btab, g.tab3, d.x, d.y, rho, vre_bar, vim_bar, cb);
  }
  // reduce cb[kNC] and c2 over the CTA
#pragma unroll
  for (int j = 0; j < kNC; ++j) {
    const float sum = warp_sum(cb[j]);
    if (lane == 0) red[j * NW + warp] = sum;
  }
  {
    const float sum = warp_sum(c2);
    if (lane == 0) red[kNC * NW + warp] = sum;
  }
  __syncthreads();
  if (tid < nptot) {
    float gk = 0.0f;
    for (int j = 0; j < kNC; ++j) {
      float cbj = 0.0f;
      for (int w = 0; w < NW; ++w) cbj += red[j * NW + w];
      gk = fmaf(cbj, g.jac[j * nptot + tid], gk);
    }
    grad[(size_t)ist * nptot + tid] = gk;
  }
  if (tid == 0) {
    float sum = 0.0f;
    for (int w = 0; w < NW; ++w) sum += red[kNC * NW + w];
    job.chi2c[ist] = sum;
  }
}

// Gauss-Newton Fisher information of chi^2/2 for replica ist = blockIdx.x:
//   F = sum_i w_i dA_i dA_i^T + sum_c w_c dphi_c dphi_c^T,
// dA_i, dphi_c the gradients with respect to p of the model amplitude of
// visibility i and of the closure phase c (dphi_c = dphi_i + dphi_j - dphi_k).
// Per point, dV/dC comes from two reverse sweeps (seeds 1 and i); then
// F_C [kNC][kNC] accumulates in C-space and F = dC/dp^T F_C dC/dp.
// gwork[ist]: amplitude rows [npts][kNC + 1] (dA/dC, w), phase rows
// [npts][kNC] (dphi/dC), closure rows [ncph][kNC + 1].
__global__ void __launch_bounds__(256) sgra_fisher_kernel(const cmc_job job,
                                                          const SgraModel::Packed pk,
                                                          float *fisher, float *gwork)
{
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x, T = blockDim.x;
  const int ist = blockIdx.x, nptot = job.nptot, npts = pk.npts;
  const int ncph = (pk.npass >= 2) ? pk.ncph : 0;
  constexpr int W1 = kNC + 1;
  const bool active = job.flag == nullptr || job.flag[ist] != 0;
  if (!active) {
    for (int k = tid; k < nptot * nptot; k += T) fisher[(size_t)ist * nptot * nptot + k] = 0.0f;
    return;
  }
  const GradCta g = grad_prologue(job, pk, ist, smem);
  float *FC = g.rest;                                          // [kNC][kNC]
  float *arow = gwork + (size_t)ist * ((size_t)npts * (W1 + kNC) + (size_t)ncph * W1);
  float *prow = arow + (size_t)npts * W1;
  float *crow = prow + (size_t)npts * kNC;
  for (int i = tid; i < npts; i += T) {
    const float4 d = __ldg(&pk.vis[i]);
    const float rho = __ldg(&pk.rho[i]);
    float2 V;
    sgra_vis_acc(g.sc, g.ring, g.btab, d.x, d.y, rho, V);
    const float n2 = fmaf(V.x, V.x, V.y * V.y);
    float cr[kNC], ci[kNC];
#pragma unroll
    for (int j = 0; j < kNC; ++j) cr[j] = ci[j] = 0.0f;
    const bool ok = n2 > 0.0f;
    if (ok) {
      sgra_vis_bwd(g.C, g.ring, g.btab, g.tab3, d.x, d.y, rho, 1.0f, 0.0f, cr);
      sgra_vis_bwd(g.C, g.ring, g.btab, g.tab3, d.x, d.y, rho, 0.0f, 1.0f, ci);
    }
    const float ia = ok ? rsqrtf(n2) : 0.0f, in2 = ok ? 1.0f / n2 : 0.0f;
#pragma unroll
    for (int j = 0; j < kNC; ++j) {
      arow[(size_t)i * W1 + j] = (V.x * cr[j] + V.y * ci[j]) * ia;
      prow[(size_t)i * kNC + j] = (V.x * ci[j] - V.y * cr[j]) * in2;
    }
    arow[(size_t)i * W1 + kNC] = d.w;
  }
  __syncthreads();
  for (int c = tid; c < ncph; c += T) {
    const int4 q = __ldg(&pk.cli[c]);
    const float4 f = __ldg(&pk.clf[c]);
#pragma unroll
    for (int j = 0; j < kNC; ++j)
      crow[(size_t)c * W1 + j] = prow[(size_t)q.x * kNC + j] + prow[(size_t)q.y * kNC + j] -
                                 prow[(size_t)q.z * kNC + j];
    crow[(size_t)c * W1 + kNC] = f.z;
  }
  __syncthreads();
  // F_C: one thread per upper-triangle entry (j <= l)
  constexpr int kPairs = kNC * (kNC + 1) / 2;
  for (int e = tid; e < kPairs; e += T) {
    int j = 0, rem = e;
    while (rem >= kNC - j) { rem -= kNC - j; ++j; }
    const int l = j + rem;
    float acc = 0.0f;
    for (int i = 0; i < npts; ++i) {
      const float *r = arow + (size_t)i * W1;
      acc = fmaf(r[kNC] * r[j], r[l], acc);
    }
    for (int c = 0; c < ncph; ++c) {
      const float *r = crow + (size_t)c * W1;
      acc = fmaf(r[kNC] * r[j], r[l], acc);
    }
    FC[j * kNC + l] = acc;
    FC[l * kNC + j] = acc;
  }
  __syncthreads();
  for (int e = tid; e < nptot * nptot; e += T) {
    const int a = e / nptot, b = e - a * nptot;
    float acc = 0.0f;
    for (int j = 0; j < kNC; ++j) {
      const float ja = g.jac[j * nptot + a];
      if (ja == 0.0f) continue;
      float t = 0.0f;
      for (int l = 0; l < kNC; ++l) t = fmaf(FC[j * kNC + l], g.jac[l * nptot + b], t);
      acc = fmaf(ja, t, acc);
    }
    fisher[(size_t)ist * nptot * nptot + e] = acc;
  }
}

inline size_t sgra_fisher_gwork_floats(const SgraModel::Packed &pk)
{
  const size_t ncph = (pk.npass >= 2) ? (size_t)pk.ncph : 0;
  return (size_t)pk.npts * (2 * kNC + 1) + ncph * (kNC + 1);
}

inline size_t sgra_fisher_smem(int nptot)
{
  return (grad_prologue_floats(nptot) + (size_t)kNC * kNC) * 4;
}

inline size_t sgra_grad_smem(int nptot, int T)
{
  return (grad_prologue_floats(nptot) + (size_t)(kNC + 1) * (T / 32)) * 4;
}

}  // namespace cmc
