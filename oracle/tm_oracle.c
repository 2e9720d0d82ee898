/*
 * tm_oracle.c -- CPU oracle (TEST INFRASTRUCTURE ONLY; see tm_oracle.h).
 * Build: gcc -std=c11 -O2 -ffp-contract=off -fno-fast-math -fPIC -shared -fopenmp
 * (the Makefile beside this file).  -ffp-contract=off matters on aarch64,
 * where GCC would otherwise fuse a*b+c and change the last bit.
 */
#include "tm_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "tm_zig_table.inc"

/* attempts of every rejection loop of the samplers before TMO_STATUS_SAMPLER_CAP
 * (the library's kSamplerCap; tests lower it to 1 to make the cap path run, as
 * the library's TM_PROBE_SAMPLER_CAP1 does) */
static int tmo_cap = 64;
void tmo_set_sampler_cap(int cap) { tmo_cap = cap < 1 ? 1 : cap; }

/* Philox4x32-10: J. K. Salmon, M. A. Moraes, R. O. Dror, D. E. Shaw,
 * "Parallel random numbers: as easy as 1, 2, 3", SC'11.  Ten rounds of
 * (c0,c1,c2,c3) -> (hi(M1 c2)^c1^k0, lo(M1 c2), hi(M0 c0)^c3^k1, lo(M0 c0))
 * with the Weyl key schedule between rounds. */
void tmo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* ---- double instantiation ---- */
#define T double
#define TM_IS_F64 1
#define FN(name) name##_f64
#define TC(x) ((double)(x))
#define FMA fma
#define SQRT sqrt
#define INV_SQRT(x) (1.0 / sqrt(x))
#define FABS fabs
#define FLOOR floor
#define RINT rint
#define TRUNC trunc
#define LN2_HI 0x1.62e42fee00000p-1
#define LN2_LO 0x1.a39ef35793c76p-33
#define INVLN2 0x1.71547652b82fep+0
#define EXP_XMAX 709.782712893384
#define EXP_XMIN (-745.1332191019411)
#include "tm_oracle_prec.inc"
#undef T
#undef TM_IS_F64
#undef FN
#undef TC
#undef FMA
#undef SQRT
#undef INV_SQRT
#undef FABS
#undef FLOOR
#undef RINT
#undef TRUNC
#undef LN2_HI
#undef LN2_LO
#undef INVLN2
#undef EXP_XMAX
#undef EXP_XMIN

/* ---- float instantiation ---- */
#define T float
#define TM_IS_F64 0
#define FN(name) name##_f32
#define TC(x) ((float)(x))
#define FMA fmaf
#define SQRT sqrtf
/* correctly rounded 1/sqrt(x) in float: the double quotient rounded once (checked
 * exhaustively over [1, 4), which covers every normal float by scaling by 4) */
#define INV_SQRT(x) ((float)(1.0 / sqrt((double)(x))))
#define FABS fabsf
#define FLOOR floorf
#define RINT rintf
#define TRUNC truncf
#define LN2_HI 0x1.62ep-1f
#define LN2_LO 0x1.0bfbe8p-15f
#define INVLN2 0x1.715476p+0f
#define EXP_XMAX 88.72283f
#define EXP_XMIN (-103.972084f)
#include "tm_oracle_prec.inc"

/* Dornic constants, stochasticSPDP.cpp:952-954 (beta, lambda) with the
 * beta == 0 limit lambda = 2/(sigma^2 dt) (cf. sde_RFT...DEF.f:48-59).
 * mean_a1/mean_a2 give the conditional mean of the Dornic kernel,
 * E[rho*] = e^{beta dt} rho + alpha (e^{beta dt}-1)/beta. */
void tmo_dornic_consts_compute(double lin, double D, double sigma, double dt, double dx, tmo_dornic_consts* o)
{
    double beta = lin - (4.0 * D) / (dx * dx);
    double e = tmo_exp_f64(beta * dt);
    double lambda, a2;
    if (beta == 0.0) {
        lambda = 2.0 / ((sigma * sigma) * dt);
        a2 = dt;
    } else {
        lambda = (2.0 * beta) / ((sigma * sigma) * (e - 1.0));
        a2 = (e - 1.0) / beta;
    }
    o->beta = beta;
    o->lambda = lambda;
    o->expbdt = e;
    o->pm = lambda * e;
    o->inv_lambda = 1.0 / lambda;
    o->mean_a1 = e;
    o->mean_a2 = a2;
}

#define TMO_BATCH_RUN(SFX, TT)                                                                            \
    int tmo_dp_batch_run_##SFX(const tmo_dp_params* p, const int* L, const uint64_t* seed, TT* const* rho,   \
                               int n_inst, int64_t n_steps, int n_threads)                                   \
    {                                                                                                        \
        int err = 0;                                                                                         \
        if (n_threads > 0) omp_set_num_threads(n_threads);                                                   \
        _Pragma("omp parallel for schedule(dynamic, 1) reduction(| : err)")                                  \
        for (int k = 0; k < n_inst; ++k) {                                                                   \
            int64_t n = (int64_t)L[k] * L[k];                                                                \
            TT* tmp = (TT*)malloc(sizeof(TT) * n);                                                           \
            if (!tmp) { err |= 1; continue; }                                                                \
            TT* A = rho[k];                                                                                  \
            TT* B = tmp;                                                                                     \
            uint32_t st = 0;                                                                                 \
            for (int64_t s = 0; s < n_steps; ++s) {                                                          \
                tmo_dp_step_##SFX(&p[k], L[k], seed[k], s, A, B, &st);                                       \
                TT* t = A; A = B; B = t;                                                                     \
            }                                                                                                \
            if (A != rho[k]) memcpy(rho[k], A, sizeof(TT) * n);                                              \
            free(tmp);                                                                                       \
        }                                                                                                    \
        return err ? -1 : 0;                                                                                 \
    }
/* Many independent DP instances on host threads (OpenMP over instances): the CPU baseline. */
TMO_BATCH_RUN(f32, float)
TMO_BATCH_RUN(f64, double)

/* FKE advection-diffusion of a consumer field (advdiff_FKE_MultiSp,
 * simulations/Rietkerk_FPE/rietkerk_bjork_FKE.cpp:3614-3695): every site with
 * rho >= eps spreads its mass over four separable Gaussian kernels -- pure
 * diffusion (weight gamma^2), diffusion x advection and advection x diffusion
 * (gamma - gamma^2 each), pure advection ((1-gamma)^2) -- the advective ones
 * centred on the site shifted by round(v * pref).  out receives the moved
 * field (sites below eps contribute nothing).  Same loop order as the
 * reference, so the sums agree bit for bit. */
static int tmo_mod(int p, int L) { int r = p % L; return r < 0 ? r + L : r; }

void tmo_fke_advdiff_f64(int L, const double* rho, const double* gam, const double* vx, const double* vy,
                         double pref, double eps, const double* gD, int RD, const double* gV, int RV, double* out)
{
    memset(out, 0, sizeof(double) * (size_t)L * L);
    for (int i = 0; i < L * L; ++i) {
        if (rho[i] < eps) continue;
        const int ci = i / L, cj = i % L;
        const double g2 = gam[i] * gam[i];
        const int mux = ((int)round(ci + vx[i] * pref) + L) % L;
        const int muy = ((int)round(cj + vy[i] * pref) + L) % L;
        const double wDD = g2 * rho[i], wDV = (gam[i] - g2) * rho[i];
        const double wVV = ((1 - gam[i]) * (1 - gam[i])) * rho[i];
        for (int p = ci - RD; p <= ci + RD; ++p) {
            const int dx = abs(p - ci), row = tmo_mod(p, L) * L;
            for (int q = cj - RD; q <= cj + RD; ++q) out[row + tmo_mod(q, L)] += wDD * (gD[dx] * gD[abs(q - cj)]);
            for (int q = muy - RV; q <= muy + RV; ++q) out[row + tmo_mod(q, L)] += wDV * (gD[dx] * gV[abs(q - muy)]);
        }
        for (int p = mux - RV; p <= mux + RV; ++p) {
            const int dx = abs(p - mux), row = tmo_mod(p, L) * L;
            for (int q = cj - RD; q <= cj + RD; ++q) out[row + tmo_mod(q, L)] += wDV * (gV[dx] * gD[abs(q - cj)]);
            for (int q = muy - RV; q <= muy + RV; ++q) out[row + tmo_mod(q, L)] += wVV * (gV[dx] * gV[abs(q - muy)]);
        }
    }
}
