/*
 * tm_oracle.h -- CPU oracle for the Dornic-split lattice Langevin integrator.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the GPU path is compared
 * against; nothing in the shipped library links or calls it.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
 *
 * It restates, in plain C, the per-step algorithm of the reference's hot
 * path (HAL9K000/Trophic_Maelstorm):
 *   - DP Dornic step   simulations/Percolation_FD/stochasticSPDP.cpp:940-1068
 *                      simulations/Percolation_FD/multiSPDP.cpp:2901-2958,3222-3262
 *   - RK4 remainders   simulations/Percolation_FD/multiSPDP.cpp:1647-1664,1821-1898
 *                      simulations/Percolation_FD/stochasticSPDP.cpp:1766-1805
 *   - Rietkerk step    simulations/Rietkerk_FPE/rietkerk_bjork_FKE.cpp:3847-3849,
 *                      2363-2444, 4154-4236, 4452-4462
 *   - noise-off RK4    simulations/Rietkerk_FPE/rietkerk_bjork_FKE.cpp:1760-1856
 *                      simulations/Percolation_FD/stochasticSPDP.cpp:516-529,549-662
 *   - observables      simulations/Percolation_FD/stochasticSPDP.cpp:123-154,1003-1025
 *
 * The reference draws its Poisson and Gamma variates from libstdc++
 * (std::poisson_distribution, std::gamma_distribution, std::mt19937_64
 * seeded from std::random_device), so its streams are neither reproducible
 * nor portable.  This oracle and the GPU kernels instead share one
 * counter-based sampler specification (Philox4x32-10 keyed by the instance
 * seed, counter = (site, step, call)); the oracle implements it
 * independently, in C, from the published algorithms it names.  Agreement
 * with the reference's libstdc++ samplers is statistical (see tests/).
 *
 * Arithmetic: every floating-point operation is IEEE add/sub/mul/div/sqrt
 * or an explicit fma(); log/exp/expm1/log1p are our own (range reduction +
 * series, below), so the same inputs give the same bits on x86-64 and
 * aarch64 when compiled with -ffp-contract=off.
 */
#ifndef TM_ORACLE_H
#define TM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status bits (same meaning as the library's TM_STATUS_*) */
#define TMO_STATUS_NAN        0x1u
#define TMO_STATUS_NEGATIVE   0x2u
#define TMO_STATUS_SAMPLER_CAP 0x4u

/* remainder integrators */
#define TMO_REM_EULER_EXACT 0   /* rho/(1+b rho dt): stochasticSPDP.cpp:1064-1068   */
#define TMO_REM_RK4         1   /* RK4 of -b rho^2 - c rho^3: multiSPDP.cpp:1821-1898 */
/* samplers */
#define TMO_SAMPLER_EXACT       0  /* Poisson -> Gamma, stochasticSPDP.cpp:1054-1059   */
#define TMO_SAMPLER_REF_GAUSS100 1 /* Gaussian above 100, multiSPDP.cpp:2915-2943     */
#define TMO_SAMPLER_OFF         2  /* conditional mean of the Dornic kernel (noise off) */

typedef struct {
    double a_start;   /* linear growth a at step 0                           */
    double a_step;    /* a(s) = a_start + a_step * s                          */
    double b, c;      /* remainder -b rho^2 - c rho^3                        */
    double D, sigma, dt, dx;
    double clamp_lo, clamp_eps; /* after a step: clamp_lo <= x < clamp_eps -> 0 */
    int remainder, sampler;
} tmo_dp_params;

typedef struct {
    double R;                    /* rainfall, the control parameter 'a'       */
    double alpha, k2, W0, gmax, k1, c, d, rW;
    double DP, DW, DO, sigma, dt, dx;
    double clamp_lo, clamp_eps;  /* 0 and 1e-10 in the reference               */
    int sampler;
} tmo_rk_params;

/* attempts of every rejection loop of the samplers (default 64, the library's;
 * 1 reproduces the library under TM_PROBE_SAMPLER_CAP1) */
void     tmo_set_sampler_cap(int cap);

/* -- primitives ---------------------------------------------------------- */
void     tmo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
double   tmo_log_f64(double x);
double   tmo_exp_f64(double x);
double   tmo_log1p_f64(double x);
double   tmo_negexpm1_f64(double m);   /* 1 - exp(-m), m >= 0 */
float    tmo_log_f32(float x);
float    tmo_exp_f32(float x);
float    tmo_log1p_f32(float x);
float    tmo_negexpm1_f32(float m);
double   tmo_inv_sqrt_f64(double x);    /* 1 / sqrt(x) */
float    tmo_inv_sqrt_f32(float x);     /* correctly rounded 1 / sqrt(x) */

/* Draw n variates; variate i uses the stream of (seed, site=i, step). */
void tmo_sample_poisson_f64(double m, uint64_t seed, int64_t step, int sampler, int64_t n, double* out, uint32_t* status);
void tmo_sample_gamma_f64(double k, uint64_t seed, int64_t step, int sampler, int64_t n, double* out, uint32_t* status);
void tmo_sample_normal_f64(uint64_t seed, int64_t step, int64_t n, double* out);
void tmo_sample_poisson_f32(float m, uint64_t seed, int64_t step, int sampler, int64_t n, float* out, uint32_t* status);
void tmo_sample_gamma_f32(float k, uint64_t seed, int64_t step, int sampler, int64_t n, float* out, uint32_t* status);
void tmo_sample_normal_f32(uint64_t seed, int64_t step, int64_t n, float* out);
/* the whole Dornic draw for one site: Gamma(mu1 + Poisson(m)) * inv_lambda */
void tmo_sample_dornic_f64(double m, double mu1, double inv_lambda, uint64_t seed, int64_t step, int sampler, int64_t n, double* out, uint32_t* status);
void tmo_sample_dornic_f32(float m, float mu1, float inv_lambda, uint64_t seed, int64_t step, int sampler, int64_t n, float* out, uint32_t* status);

/* Per-step Dornic constants for a given a (or -d for Rietkerk P). */
typedef struct {
    double beta, lambda, expbdt, pm, inv_lambda, mean_a1, mean_a2;
} tmo_dornic_consts;
void tmo_dornic_consts_compute(double lin, double D, double sigma, double dt, double dx, tmo_dornic_consts* out);

/* -- one time step of one instance (Jacobi: in and out distinct) --------- */
int tmo_dp_step_f64(const tmo_dp_params* p, int L, uint64_t seed, int64_t step,
                    const double* in, double* out, uint32_t* status);
int tmo_dp_step_f32(const tmo_dp_params* p, int L, uint64_t seed, int64_t step,
                    const float* in, float* out, uint32_t* status);
/* the same with a per-site loss coefficient b_v (NULL: p->b everywhere) */
int tmo_dp_step_sb_f64(const tmo_dp_params* p, int L, uint64_t seed, int64_t step,
                       const double* in, double* out, uint32_t* status, const double* site_b);
int tmo_dp_step_sb_f32(const tmo_dp_params* p, int L, uint64_t seed, int64_t step,
                       const float* in, float* out, uint32_t* status, const float* site_b);
int tmo_rk_step_f64(const tmo_rk_params* p, int L, uint64_t seed, int64_t step,
                    const double* in /* [P|W|O] 3*L*L */, double* out, uint32_t* status);
int tmo_rk_step_f32(const tmo_rk_params* p, int L, uint64_t seed, int64_t step,
                    const float* in, float* out, uint32_t* status);

/* stages alone (for pinning against the reference's own stage functions) */
int tmo_dp_remainder_f64(const tmo_dp_params* p, int64_t n, const double* in, double* out);
int tmo_dp_remainder_f32(const tmo_dp_params* p, int64_t n, const float* in, float* out);
int tmo_rk_remainder_f64(const tmo_rk_params* p, int L, const double* in, double* out);
int tmo_rk_remainder_f32(const tmo_rk_params* p, int L, const float* in, float* out);

/* noise-off deterministic steps */
int tmo_rk_det_step_f64(const tmo_rk_params* p, int L, const double* in, double* out);
int tmo_rk_det_step_f32(const tmo_rk_params* p, int L, const float* in, float* out);
/* DP drho/dt = a rho - b rho^2 - c rho^3 + D Lap(rho); stencil 5 or 9 (4th-order
 * cross, stochasticSPDP.cpp:516-529); integrator 0 Euler, 1 RK4 */
int tmo_dp_det_step_f64(double a, double b, double c, double D, double dt, double dx,
                        int stencil, int integrator, int L, const double* in, double* out);
int tmo_dp_det_step_f32(double a, double b, double c, double D, double dt, double dx,
                        int stencil, int integrator, int L, const float* in, float* out);

/* -- observables: FP64 spatial sum and active-site count (rho > 0) ------- */
void tmo_observe_f64(const double* x, int64_t n, double* sum, double* active);
void tmo_observe_f32(const float* x, int64_t n, double* sum, double* active);

/* -- whole runs ------------------------------------------------------------
 * Advance n_steps steps from rho0; before step s (state after s updates) the
 * mean and active count are recorded for every s in meas_steps (ascending).
 * Stops early (zero rows after) once a measurement sees no active site, as
 * stochasticSPDP.cpp:1021-1022 does.  rho_final (optional) gets the last state. */
int tmo_dp_run_f64(const tmo_dp_params* p, int L, uint64_t seed, const double* rho0,
                   int64_t n_steps, const int64_t* meas_steps, int n_meas,
                   double* out_mean, double* out_active, double* rho_final, uint32_t* status);
int tmo_dp_run_f32(const tmo_dp_params* p, int L, uint64_t seed, const float* rho0,
                   int64_t n_steps, const int64_t* meas_steps, int n_meas,
                   double* out_mean, double* out_active, float* rho_final, uint32_t* status);
int tmo_rk_run_f64(const tmo_rk_params* p, int L, uint64_t seed, const double* f0,
                   int64_t n_steps, const int64_t* meas_steps, int n_meas,
                   double* out_mean /* n_meas x 3 (P,W,O) */, double* out_active,
                   double* f_final, uint32_t* status);
int tmo_rk_run_f32(const tmo_rk_params* p, int L, uint64_t seed, const float* f0,
                   int64_t n_steps, const int64_t* meas_steps, int n_meas,
                   double* out_mean, double* out_active, float* f_final, uint32_t* status);

/* FKE advection-diffusion of a consumer field (rietkerk_bjork_FKE.cpp:3614-3695). */
void tmo_fke_advdiff_f64(int L, const double* rho, const double* gam, const double* vx, const double* vy,
                         double pref, double eps, const double* gD, int RD, const double* gV, int RV, double* out);

/* Many independent DP instances on host threads (OpenMP): the CPU baseline. */
int tmo_dp_batch_run_f32(const tmo_dp_params* p /* n_inst */, const int* L, const uint64_t* seed,
                         float* const* rho /* in: initial, out: final */, int n_inst,
                         int64_t n_steps, int n_threads);
int tmo_dp_batch_run_f64(const tmo_dp_params* p, const int* L, const uint64_t* seed,
                         double* const* rho, int n_inst, int64_t n_steps, int n_threads);

#ifdef __cplusplus
}
#endif
#endif
