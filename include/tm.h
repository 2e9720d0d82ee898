/*
 * tm.h -- C ABI of the GB300 lattice Langevin integrator (libtm.so).
 *
 * Drop-in boundary for the per-instance integrators of HAL9K000/Trophic_Maelstorm:
 *   percolationDornic_2D        simulations/Percolation_FD/stochasticSPDP.cpp:940   (SPDP.h:96)
 *   dP_Dornic_2D_MultiSp        simulations/Percolation_FD/multiSPDP.cpp:2421
 *   rietkerk_DorFPE_2D_MultiSp  simulations/Rietkerk_FPE/rietkerk_bjork_FKE.cpp:3697
 *   rietkerk_Dornic_2D_MultiSp  simulations/Rietkerk_FD/rietkerk_bjork_basic.cpp:3397
 *   RK4_Wrapper_2D (noise off)  simulations/Rietkerk_FPE/rietkerk_bjork_FKE.cpp:1858
 *   percNoDiff_2D  (noise off)  simulations/Percolation_FD/stochasticSPDP.cpp:549
 * The reference calls one of these per parameter value from an OpenMP thread
 * (stochasticSPDP.cpp:1343-1369) and runs replicates serially inside it.  Here
 * one call takes a whole batch of instances -- replicates x control values x
 * lattice sizes, ragged -- and advances them together on one GPU.
 *
 * Conventions: plain C types only; host pointers are caller-owned and only
 * read/written during the call; every function returns TM_OK (0) or a
 * negative TM_ERR_* code and never exits the process (the reference calls
 * exit(1|3|4), multiSPDP.cpp:3287-3356).  Per-instance problems found on the
 * device (NaN/Inf, negative density, sampler iteration cap) are reported as
 * TM_STATUS_* bits, not as errors.  A context is used by one host thread at a
 * time; different contexts are independent.
 *
 * State layout: a batch keeps all fields of all instances in one packed
 * buffer of the batch precision (double for TM_FP64, float for TM_FP32).
 * Instance k starts at element tm_batch_instance_offset(k); inside it the
 * fields follow each other with stride tm_batch_field_stride(k) elements,
 * each field an L x L row-major periodic lattice (site i*L + j, the reference's
 * indexing).  DP has one field (rho); Rietkerk has three in the reference's
 * order [P, W, O] (rietkerk_bjork_constants_1Sp.h:5-6).
 */
#ifndef TM_H
#define TM_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TM_ABI_VERSION 1

/* return codes */
#define TM_OK            0
#define TM_ERR_INVALID  (-1)   /* bad argument                          */
#define TM_ERR_CUDA     (-2)   /* CUDA runtime error (context unusable)  */
#define TM_ERR_NOMEM    (-3)   /* device or host allocation failed       */
#define TM_ERR_STATE    (-4)   /* call not valid in the object's state   */
#define TM_ERR_TIMEOUT  (-5)   /* a bounded device-side wait ran out     */

/* per-instance status bits (OR-ed over all steps since the last reset) */
#define TM_STATUS_NAN          0x1u  /* NaN or Inf produced               */
#define TM_STATUS_NEGATIVE     0x2u  /* negative density produced         */
#define TM_STATUS_SAMPLER_CAP  0x4u  /* a rejection loop hit its cap      */
#define TM_STATUS_WAIT_TIMEOUT 0x8u  /* a bounded wait for a tile copy ran
                                        out: the instance's fields are
                                        invalid from that step on, and the
                                        call returns TM_ERR_TIMEOUT        */

/* precision of the field state; reductions are FP64 in both */
#define TM_FP64 0
#define TM_FP32 1

/* remainder (deterministic part after the Dornic draw) for the DP model */
#define TM_REM_EULER_EXACT 0   /* rho/(1 + b rho dt)        stochasticSPDP.cpp:1064-1068 */
#define TM_REM_RK4         1   /* RK4 of -b rho^2 - c rho^3 multiSPDP.cpp:1821-1898      */

/* sampler of the Dornic step */
#define TM_SAMPLER_EXACT        0  /* Poisson -> Gamma            stochasticSPDP.cpp:1054-1059 */
#define TM_SAMPLER_REF_GAUSS100 1  /* Gaussian above 100          multiSPDP.cpp:2915-2943      */
#define TM_SAMPLER_OFF          2  /* conditional mean (noise off)                             */

/* noise-off DP stencils (TM_MODEL_DP_DET) */
#define TM_STENCIL_5 5   /* 5-point Laplacian                                     */
#define TM_STENCIL_9 9   /* 4th-order cross (-1,16,-30,16,-1)/12, fP_2D :516-529  */

typedef struct tm_ctx tm_ctx;
typedef struct tm_batch tm_batch;

/* One lattice instance of a batch. */
typedef struct tm_instance {
    int32_t  L;        /* lattice side, >= 1                                         */
    int32_t  reserved;
    uint64_t seed;     /* Philox key of this instance's random stream               */
    double   a;        /* DP: linear coefficient a at step 0; Rietkerk: rainfall R  */
    double   a_step;   /* DP: a(s) = a + a_step * s (0 = fixed a); Rietkerk: unused */
} tm_instance;

/* DP Langevin model  d rho = (a rho - b rho^2 - c rho^3 + D Lap rho) dt + sigma sqrt(rho) dW
 * (stochasticSPDP.cpp:940-1068, multiSPDP.cpp:2421-3262).  a is per instance. */
typedef struct tm_dp_model {
    double b, c, D, sigma, dt, dx;
    double clamp_lo, clamp_eps;  /* after each step clamp_lo <= rho < clamp_eps -> 0;
                                    clamp_eps = 0 disables (classic); multiSPDP uses
                                    [-1e-80, 1e-12) (:3256-3259)                     */
    int32_t remainder;           /* TM_REM_*                                        */
    int32_t sampler;             /* TM_SAMPLER_*                                    */
    int32_t deterministic;       /* 1: noise-off a rho - b rho^2 - c rho^3 + D Lap rho
                                    by RK4/Euler on the lattice, no Dornic split
                                    (percNoDiff_2D); uses stencil and integrator    */
    int32_t stencil;             /* TM_STENCIL_5 / TM_STENCIL_9 (deterministic only) */
    int32_t integrator;          /* 0 Euler, 1 RK4 (deterministic only)             */
    int32_t reserved;
} tm_dp_model;

/* Rietkerk three-field vegetation model (rietkerk_bjork_FKE.cpp:1760-1785, 2363-2390):
 *   dO = R - alpha O (P + k2 W0)/(P + k2) + D_O Lap O
 *   dW = alpha O (P + k2 W0)/(P + k2) - gmax W P/(W + k1) - rW W + D_W Lap W
 *   dP = c gmax W P/(W + k1) - d P + D_P Lap P + sigma sqrt(P) dW
 * R is per instance (tm_instance.a).  With deterministic = 0 the -d P + D_P Lap P
 * + noise part is the Dornic draw and the rest is one RK4 step; with
 * deterministic = 1 the whole right-hand side is one RK4 step (RK4_Wrapper_2D). */
typedef struct tm_rietkerk_model {
    double alpha, k2, W0, gmax, k1, c, d, rW;
    double DP, DW, DO, sigma, dt, dx;
    double clamp_lo, clamp_eps;  /* reference: 0 <= x < 1e-10 -> 0 (:4460, basic.h:119) */
    int32_t sampler;             /* TM_SAMPLER_*, reference: TM_SAMPLER_REF_GAUSS100 */
    int32_t deterministic;
} tm_rietkerk_model;

/* -------------------------------------------------------------------- */
int         tm_abi_version(void);
const char* tm_error_string(int code);

/* Context on one CUDA device with its own stream. */
int   tm_create(tm_ctx** out, int device);
int   tm_destroy(tm_ctx* ctx);
void* tm_stream(tm_ctx* ctx);            /* the cudaStream_t the context launches on */
int   tm_sync(tm_ctx* ctx);

/* -- batches: device-resident state advanced step by step ------------------ */
/* Replaces the replicate/parameter loops around percolationDornic_2D
 * (stochasticSPDP.cpp:1343-1384) and rietkerk_DorFPE_2D_MultiSp (:4778-4802). */
int tm_batch_create_dp(tm_ctx* ctx, const tm_dp_model* model, const tm_instance* inst,
                       int n_inst, int precision, tm_batch** out);
int tm_batch_create_rietkerk(tm_ctx* ctx, const tm_rietkerk_model* model, const tm_instance* inst,
                             int n_inst, int precision, tm_batch** out);
int tm_batch_destroy(tm_batch* b);

int64_t tm_batch_total_elems(const tm_batch* b);          /* packed state size (elements) */
int64_t tm_batch_instance_offset(const tm_batch* b, int k);
int64_t tm_batch_field_stride(const tm_batch* b, int k);
int     tm_batch_num_fields(const tm_batch* b);            /* 1 (DP) or 3 (Rietkerk)       */
int     tm_batch_obs_width(const tm_batch* b);             /* doubles per measurement      */
int64_t tm_batch_step(const tm_batch* b);                  /* steps taken so far           */

/* State transfer; host_fields/dev_fields hold tm_batch_total_elems() elements of
 * the batch precision in the packed layout.  Upload resets the step counter to
 * `step` (the Philox counter of the next step) and revives extinct instances.
 * tm_batch_upload reads page-locked host memory (cudaHostAlloc, cudaHostRegister)
 * with a copy kernel over the host link when the buffer starts on a 16-byte
 * boundary, and other host memory through cudaMemcpyAsync; it returns after the
 * copy and the check of the uploaded state. */
int tm_batch_upload(tm_batch* b, const void* host_fields, int64_t step);
int tm_batch_download(tm_batch* b, void* host_fields);
int tm_batch_upload_device(tm_batch* b, const void* dev_fields, int64_t step);
int tm_batch_download_device(tm_batch* b, void* dev_fields);
/* Copy one instance's fields (nf * L * L elements, fields contiguous) to host:
 * the frame interface of save_frame (multiSPDP.cpp:1596-1643). */
int tm_batch_snapshot(tm_batch* b, int k, void* host_out);

/* Advance n_steps steps.  Before the step with absolute index s (i.e. on the
 * state after s steps) every s listed in meas_steps (ascending, each in
 * [tm_batch_step, tm_batch_step + n_steps]) is measured into
 * obs[(j * n_inst + k) * obs_width + f]:
 *   DP:        f0 = spatial mean of rho, f1 = number of sites with rho > 0
 *   Rietkerk:  f0..f2 = spatial means of P, W, O, f3 = sites with P > 0
 * (mean_of_vector / occupied_sites_of_vector, stochasticSPDP.cpp:123-154).  A DP
 * instance measured with no active site is extinct: it stays zero and its
 * later measurements are 0 (the early exit of stochasticSPDP.cpp:1021-1022).
 * status (optional, n_inst entries) receives the OR of TM_STATUS_* bits since
 * creation or the last upload, including those of the uploaded state itself
 * (tm_batch_upload marks a NaN/Inf with TM_STATUS_NAN and a negative value with
 * TM_STATUS_NEGATIVE, as the reference's per-step checks would on its next
 * step, multiSPDP.cpp:2949-2955, 3237-3255).  obs may be NULL when n_meas == 0.
 * Returns TM_ERR_TIMEOUT (after filling obs and status) when an instance got
 * TM_STATUS_WAIT_TIMEOUT.  The call returns after the work is queued and
 * complete (it synchronises). */
int tm_batch_advance(tm_batch* b, int64_t n_steps, const int64_t* meas_steps, int n_meas,
                     double* obs, uint32_t* status);
/* Same, without synchronising and without measurements: queues n_steps steps on
 * the context stream (CUDA graphs of the step sequence); for timing loops. */
int tm_batch_enqueue_steps(tm_batch* b, int64_t n_steps);

/* Launch shape of the step kernels: rows per warp task (DP/Dornic) and CTAs
 * per SM of the persistent grid.  0 keeps the current value.  A new batch
 * starts at 8 rows (fewer when the batch has too few tasks to fill the GPU) and
 * 4 CTAs/SM.  tm_batch_autotune times the candidates on the batch itself
 * (state is saved and restored).  Results do not depend on the launch shape. */
int tm_batch_set_launch(tm_batch* b, int rows_per_task, int ctas_per_sm);
int tm_batch_get_launch(const tm_batch* b, int* rows_per_task, int* ctas_per_sm);
int tm_batch_autotune(tm_batch* b, int steps_per_trial);

/* Spreading runs (DP, stochastic): spreading_exp_Dornic_2D
 * (stochasticSPDP.cpp:1145-1298) started from a single seed.  With enable = 1,
 * every measurement also gives f2 = the sum over occupied sites (rho > 0) of the
 * squared distance (row - cy)^2 + (col - cx)^2 from the seed site
 * (meansq_spread_of_vector, :156-170; cx, cy = -1: L/2, the reference's seed),
 * so tm_batch_obs_width becomes 3; and an instance whose border row or column
 * holds an occupied site stops before its next measurement or step, as the
 * reference's theborderwall check ends the replicate (:380-390, 1206-1213): its
 * later measurements are 0 and it downloads as zeros, like an extinct one. */
int tm_batch_set_spreading(tm_batch* b, int enable, int cx, int cy);

/* Per-site loss coefficient b_v for a DP batch (host, packed like the state):
 * the remainder uses b_v[i] in place of tm_dp_model.b -- the termite-mound
 * field of sde_RFT_2D_improved_Euler_w_mounds_RT_RK4_SNAPSHOTS_DEF.f:196-428,
 * 564-574.  NULL restores the uniform b. */
int tm_batch_set_site_coeff(tm_batch* b, const void* host_coeff);

/* Kadanoff block means of field `field` of instance k (sde_RFT...DEF.f:474-516):
 * out[(by * (L/box) + bx)] = mean over the box x box block; L % box must be 0. */
int tm_batch_box_means(tm_batch* b, int k, int field, int box, double* out);

/* -- one-shot calls: host buffers in, host results out -------------------- */
/* The whole percolationDornic_2D-style job for a batch: upload init_fields,
 * advance n_steps with measurements, return obs/status and (optionally) the
 * final fields.  Host<->device copies are part of the call. */
int tm_run_dp(tm_ctx* ctx, const tm_dp_model* model, const tm_instance* inst, int n_inst, int precision,
              const void* init_fields, int64_t n_steps, const int64_t* meas_steps, int n_meas,
              double* obs, uint32_t* status, void* final_fields);
int tm_run_rietkerk(tm_ctx* ctx, const tm_rietkerk_model* model, const tm_instance* inst, int n_inst,
                    int precision, const void* init_fields, int64_t n_steps, const int64_t* meas_steps,
                    int n_meas, double* obs, uint32_t* status, void* final_fields);

/* -- observables without allocation ---------------------------------------
 * No counterpart in the reference: it exists for callers that cannot let a
 * library allocate device memory -- for example a host application that has
 * already given the GPU's memory to its own pool allocator, or a
 * latency-sensitive loop that must not trigger cudaMalloc's implicit device
 * synchronisation.  It computes the same FP64 observables as a DP measurement
 * of tm_batch_advance (spatial mean of rho and the number of sites with
 * rho > 0, per instance) for lattices that live in the caller's own device
 * buffer, and writes them to the caller's device buffer dev_out[2*k + {0,1}].
 * It calls no cudaMalloc/cudaFree: its scratch (instance table, task table,
 * per-task partial sums) is a static TM_NOALLOC_SCRATCH_BYTES array in the
 * library image, held by every GPU that loads libtm.so until the process exits.
 *   dev_fields  device pointer, elements of `precision` (TM_FP64 / TM_FP32)
 *   L, offsets  host arrays, n_inst entries: lattice side and element offset of
 *               each instance in dev_fields (e.g. from tm_layout)
 *   stream      cudaStream_t to run on (NULL: the legacy default stream)
 * Returns TM_ERR_INVALID when the instances need more scratch than the array
 * holds: 256-byte-aligned regions of 8*n_inst + 4*n_inst + 4*(n_inst+1) bytes
 * plus 24 bytes per 32-column strip (sum over instances of ceil(L/32)).
 * The first call on a device looks up the array's device address (once per
 * device, with that device current); make that first call before any stream
 * capture.  The address is kept for the life of the process, so the entry
 * point must not be called on a device after cudaDeviceReset of that device.
 * L and offsets are copied to the scratch by an asynchronous copy on `stream`:
 * keep them unchanged until the stream has passed the call (page-locked host
 * arrays are read by that copy after the call returns).
 * All calls share the one array and leave their contents in it;
 * every value a call reads it has written itself, so nothing needs clearing,
 * but two calls that overlap on the GPU (other streams, other host threads)
 * race on the array: order them on one stream or synchronise between them.
 * The call is asynchronous on `stream`; dev_out is ready when it completes. */
#define TM_NOALLOC_SCRATCH_BYTES (4u << 20)
int tm_observe_noalloc(const void* dev_fields, int precision, const int32_t* L, const int64_t* offsets,
                       int n_inst, double* dev_out, void* stream);

/* -- pattern wavelength --------------------------------------------------
 * Radially averaged power spectrum of one L x L lattice in device memory, with
 * the semantics of the reference's estimator gen_FFT_PowerSpectra
 * (simulations/Utilities/glow_up.py:752-827): divide by the maximum (if
 * non-zero), |FFT2|^2 in double precision, mean over annuli of width binwidth
 * starting at 1 - binwidth/2, times the annulus area; empty bins are 0 (the
 * reference turns them into NaN).  kvals/power receive *n_bins values
 * (TM_ERR_INVALID if more than max_bins).  The pattern wavelength is
 * L / kvals[argmax power].  Synchronises `stream`. */
int tm_power_spectrum_device(const void* dev_field, int precision, int L, double binwidth, void* stream,
                             double* kvals, double* power, int max_bins, int* n_bins);
/* The same for field `field` of instance k of a batch's current state. */
int tm_batch_power_spectrum(tm_batch* b, int k, int field, double binwidth, double* kvals, double* power,
                            int max_bins, int* n_bins);

/* -- consumer movement: FKE advection-diffusion ---------------------------
 * Replaces advdiff_FKE_MultiSp (simulations/Rietkerk_FPE/rietkerk_bjork_FKE.cpp:
 * 3614-3695) and its CUDA kernel updateMovement (kernel_advdiff_FKE2D.cu:92-180)
 * for one consumer field on an L x L periodic lattice.  Every site with
 * rho >= eps moves its mass through the separable Gaussian stencils gD
 * (diffusion, gD[0..RD]) and gV (advection, gV[0..RV]): fraction gamma^2 by
 * diffusion around the site, (1-gamma)^2 by advection around the site shifted
 * by round(v * pref) in each axis (x = row, y = column), and gamma(1-gamma)
 * by each of the two mixed products; sites below eps end as 0.  The stencils
 * and pref are what set_global_FKE_params / precompute_gaussian
 * (rietkerk_bjork_FKE.cpp:195-338, :1735-1749) give for the species.
 *   dev_rho, dev_gamma, dev_vx, dev_vy  device, L*L row-major, `precision`
 *   dev_out  device, L*L; receives the moved field (distinct from the inputs)
 *   gD, gV   host arrays; RD, RV <= 2^20; 1 <= L <= 46340
 * Computed as two separable gathers (along rows into per-row-stencil partial
 * sums, then down columns), so the result has no atomics and does not depend
 * on scheduling; it equals the reference's scatter up to the order of the
 * floating-point additions.  Allocates scratch of three L*L arrays of the
 * precision and two of int, and synchronises `stream`. */
int tm_fke_advdiff_device(const void* dev_rho, const void* dev_gamma, const void* dev_vx, const void* dev_vy,
                          int precision, int L, double pref, double eps, const double* gD, int RD,
                          const double* gV, int RV, void* dev_out, void* stream);
/* The same operator for a per-step consumer loop: the scratch is the caller's
 * device workspace (tm_fke_workspace_bytes(precision, L) bytes, 256-byte
 * aligned, reusable from call to call), the stencils travel in the launch
 * arguments (RD, RV <= TM_FKE_WS_MAX_RADIUS), and the call only queues work on
 * `stream`: it allocates nothing, copies nothing from the host and does not
 * synchronise; dev_out is ready when the stream passes the call.  Two calls
 * sharing one workspace must be ordered on the stream.  Results equal
 * tm_fke_advdiff_device's bit for bit. */
#define TM_FKE_WS_MAX_RADIUS 127
size_t tm_fke_workspace_bytes(int precision, int L);
int tm_fke_advdiff_device_ws(const void* dev_rho, const void* dev_gamma, const void* dev_vx, const void* dev_vy,
                             int precision, int L, double pref, double eps, const double* gD, int RD,
                             const double* gV, int RV, void* dev_out, void* dev_workspace, size_t workspace_bytes,
                             void* stream);

/* -- sweep surrogate: a small network trained on the integrator's own runs --
 * No counterpart in the reference, which locates the critical point by
 * uniform sweeps of the control parameter (critical_exp_delta,
 * simulations/Percolation_FD/stochasticSPDP.cpp:1309-1422).  The surrogate
 * maps features f = (a, log L, log t), affinely normalised by the caller, to two
 * outputs (the caller's scaling of the mean density and the survival
 * fraction) through
 *     h1 = bf16(gelu(W1 f + b1)), h2 = bf16(gelu(W2 h1 + b2)),
 *     h3 = gelu(W3 h2 + b3), y = W4 h3 + b4
 * with 128 hidden units, gelu(x) = x/2 (1 + tanh(sqrt(2/pi)(x + 0.044715 x^3))),
 * every weight matrix used as the BF16 rounding (nearest even) of its FP32
 * master and all sums accumulated in FP32.  The two 128 x 128 layers and
 * their backward GEMMs run on the tensor cores.
 * Parameters: TM_MLP_NPARAMS floats W1[128][3] | b1[128] | W2[128][128] |
 * b2[128] | W3[128][128] | b3[128] | W4[2][128] | b4[2] (row-major [out][in]).
 * Loss: inv_norm * sum over samples of w0 (y0 - t0)^2 + w1 (y1 - t1)^2.  The
 * backward pass rounds dz3 = (dy W4) * gelu'(.) and dz2 = (dz3 W3) * gelu'(.) to
 * BF16 (the tensor-core operands); dz1 and all gradients stay FP32.  Partial
 * gradients of 128-sample tiles are summed in tile order, so results are
 * bit-reproducible.  The optimiser is full-batch Adam on the FP32 masters,
 * with bias corrections 1/(1 - beta^t) computed on the host in double.
 * tm_mlp_train returns TM_ERR_TIMEOUT if a bounded wait for a tensor-core
 * operation ran out (the context stays usable; the parameters keep their value
 * from before the step whose wait ran out). */
#define TM_MLP_NPARAMS 33794
typedef struct tm_mlp tm_mlp;
int tm_mlp_create(tm_ctx* ctx, const float* params, tm_mlp** out);
int tm_mlp_destroy(tm_mlp* m);
/* replace the parameters; resets the Adam moments and step count */
int tm_mlp_set_params(tm_mlp* m, const float* params);
int tm_mlp_get_params(tm_mlp* m, float* params);
/* the training set, copied to device memory: x n x 3, targets t n x 2, loss weights w n x 2 */
int tm_mlp_set_data(tm_mlp* m, const float* x, const float* t, const float* w, int n);
/* loss and gradient over the whole training set, no update (grad: TM_MLP_NPARAMS floats; either may be NULL) */
int tm_mlp_loss_grad(tm_mlp* m, float inv_norm, double* loss, float* grad);
/* `steps` full-batch Adam steps; loss_hist (optional, `steps` doubles) gets the loss before each update */
int tm_mlp_train(tm_mlp* m, int steps, float lr, float beta1, float beta2, float eps, float inv_norm,
                 double* loss_hist);
/* y (n x 2) for features x (n x 3) */
int tm_mlp_predict(tm_mlp* m, const float* x, int n, float* y);

/* -- failure probes (tests only) -----------------------------------------
 * Each flag makes one failure path of the library run on purpose, in a form
 * that faults nothing, so a test can check what the caller sees:
 *   TM_PROBE_SAMPLER_CAP1  every rejection loop of the samplers stops after one
 *                          attempt: sites whose first attempt is rejected get
 *                          TM_STATUS_SAMPLER_CAP (and the loop's fallback value);
 *                          DP batches with the Euler-exact remainder and the
 *                          exact sampler only (others: TM_ERR_INVALID)
 *   TM_PROBE_TILE_WAIT     the Rietkerk RK4 tiles issue no copy and wait on a
 *                          barrier nothing arrives at: the bounded wait runs out
 *                          with nothing in flight, the instances get
 *                          TM_STATUS_WAIT_TIMEOUT and tm_batch_advance returns
 *                          TM_ERR_TIMEOUT
 *   TM_PROBE_MLP_WAIT      the network kernel issues no MMA and waits for a commit
 *                          that never comes: tm_mlp_* return TM_ERR_TIMEOUT and
 *                          leave the parameters unchanged
 * The flags apply to batches created, and network calls made, after this call
 * on this context (a batch's step graphs keep its launch arguments); 0 clears
 * them.  The context stays usable in every case. */
#define TM_PROBE_SAMPLER_CAP1 0x1u
#define TM_PROBE_TILE_WAIT    0x2u
#define TM_PROBE_MLP_WAIT     0x4u
int tm_set_test_probe(tm_ctx* ctx, uint32_t flags);

/* Packed-layout geometry without a batch (for callers that pack host buffers
 * before creating one): offsets[k] and the total, for nf fields per instance. */
int64_t tm_layout(const tm_instance* inst, int n_inst, int nf, int64_t* offsets, int64_t* field_strides);

#ifdef __cplusplus
}
#endif
#endif
