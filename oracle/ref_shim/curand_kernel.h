/* Host stand-in for <curand_kernel.h> (test infrastructure).
 *
 * When oracle/ref_build.py compiles the reference's kernels for the CPU, every
 * curand_uniform()/curand_normal() call on rndst[ist] reads the next value of
 * replica ist's INJECTED stream instead of generating one.  The state keeps
 * the two stream cursors. */
#pragma once
typedef struct curandStateInjected { int cu, cn; } curandState;
typedef curandState curandStateXORWOW;

extern curandState *g_ref_rndst_base;   /* rndst[0] of the running job */
extern const float *g_ref_u, *g_ref_n;  /* [nrep][lu], [nrep][ln]       */
extern int g_ref_lu, g_ref_ln, g_ref_overflow;

static inline void curand_init(unsigned long long, unsigned long long,
                               unsigned long long, curandState *st)
{
    st->cu = 0;
    st->cn = 0;
}

static inline float curand_uniform(curandState *st)
{
    long ist = (long)(st - g_ref_rndst_base);
    if (st->cu >= g_ref_lu) { g_ref_overflow = 1; return 0.5f; }
    return g_ref_u[ist * g_ref_lu + st->cu++];
}

static inline float curand_normal(curandState *st)
{
    long ist = (long)(st - g_ref_rndst_base);
    if (st->cn >= g_ref_ln) { g_ref_overflow = 1; return 0.0f; }
    return g_ref_n[ist * g_ref_ln + st->cn++];
}
