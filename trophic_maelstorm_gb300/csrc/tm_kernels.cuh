// tm_kernels.cuh -- kernel parameter blocks and launchers shared by the
// kernel translation units and the C ABI implementation.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

// A context: one device and the stream every call on it launches on (tm_create).
struct tm_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    int num_sms = 0;
    unsigned probe = 0;            // TM_PROBE_* flags for objects created from now on (tests)
};

namespace tmg {

// Dornic constants of one instance: lambda e^{beta dt}, 1/lambda, e^{beta dt}, (e^{beta dt}-1)/beta
struct __align__(16) Dc4 { double x, y, z, w; };

// Per-instance tables in device memory (structure of arrays).
struct InstTables {
    const long long* off;          // element offset of the instance's first field
    const long long* fstride;      // elements between fields of one instance
    const int* L;
    const unsigned long long* seed;
    const double* R;               // Rietkerk rainfall (per instance)
    const Dc4* consts;         // Dornic constants: (lambda e^{beta dt}, 1/lambda, e^{beta dt}, (e^{beta dt}-1)/beta)
    int* alive;                    // DP extinction flags (nullptr: never skip)
    unsigned* status;              // TM_STATUS_* bits
};

// Warp task: 32 columns x `rows` rows of one instance: (inst, x0, y0, rows).
// Block task (RK4 tile): (inst, x0, y0, 0).

template <typename T>
struct DornicArgs {
    const T* in;                   // state (field 0 is read)
    T* out;                        // field-0 slots receive the result
    InstTables it;
    const int4* tasks;
    int n_tasks;
    const long long* step_base;    // device step counter (graph replays) or nullptr
    long long step_off;            // step = (*step_base) + step_off
    T dcoef, two_s2, b, c, dt, dt2, dt6, clo, ceps;
    int sampler;                   // 0 exact, 1 Gaussian above 100, 2 mean (noise off)
    int cubic;
    int rows_cap;                  // rows of the largest task (<= kMaxRowsPerTask)
    const T* site_b;               // per-site loss coefficient b_v (packed like the state) or nullptr
    int zero_fixed;                // a +0 draw finishes as +0, no status bit (finite b, c, dt; no site_b)
    int cap1;                      // TM_PROBE_SAMPLER_CAP1: rejection loops stop after one attempt
    uint4* dlist;                  // FP32: deferred sites (instance, site, Poisson mean, Gamma shape bits),
                                   // one segment of seg_cap entries per warp of the step kernel's grid
    unsigned* dcnt;                // FP32: entries in each warp's segment (written by the step kernel)
    long long seg_cap;             // entries per segment (all sites of one warp's tasks)
    long long dlist_cap;           // entries the list holds
    long long max_seg;             // segments dcnt holds
};

template <typename T>
struct RK4Args {
    const T* in;                   // [P|W|O] state
    const T* pstar;                // P after the Dornic draw (field-0 slots); nullptr when deterministic
    T* out;
    InstTables it;
    const int4* tasks;             // block tasks
    int n_tasks;
    T alpha, k2, k2W0, gmax, cgmax, k1, rW, d, DPx, DWx, DOx, dt2, dt6, dt, clo, ceps;
    int wait_limit;                // polls of a tile's copy barrier before the CTA gives up
    int probe_no_copy;             // TM_PROBE_TILE_WAIT: issue no copy, so the bounded wait runs out
};

template <typename T>
struct DetTileArgs {               // noise-off DP step over 64 x 32 tiles of every instance (a = it.R[k])
    const T* in;
    T* out;
    InstTables it;
    const int4* tasks;             // block tasks
    int n_tasks;
    T b, c, dlap, dk12, dt, dt2, dt6;
    int cubic;
};

// launchers (defined in the kernel translation units)
template <typename T>
cudaError_t launch_dornic(const DornicArgs<T>& a, int rem, int grid, int block, cudaStream_t s);
template <typename T>
cudaError_t launch_rk4(const RK4Args<T>& a, bool det, int grid, cudaStream_t s);
template <typename T>
cudaError_t launch_measure(const T* state, const InstTables& it, const int4* tasks, int n_tasks, int nf,
                           double* partial, int grid, int block, cudaStream_t s, int spread = 0, int cx = -1,
                           int cy = -1);
template <typename T>
cudaError_t launch_border_stop(const T* state, const InstTables& it, int n_inst, cudaStream_t s);
template <typename T>
cudaError_t launch_validate(const T* state, const InstTables& it, const int4* tasks, int n_tasks, int nf, int grid,
                            cudaStream_t s);
cudaError_t launch_finalize(const double* partial, const int* task_begin, const InstTables& it, int n_inst, int nf,
                            int dp_extinction, int spread, double* obs_row, cudaStream_t s);
cudaError_t launch_consts(const double* a0, const double* astep, int n, double diff4, double sigma2, double dt,
                          const long long* step_base, long long step_off, Dc4* out, cudaStream_t s);
cudaError_t launch_set_step(long long* d_step, long long v, cudaStream_t s);
cudaError_t launch_copy_in(const void* src, void* dst, size_t bytes, int grid, cudaStream_t s);
template <typename T>
cudaError_t launch_box_means(const T* field, int L, int box, double* out, cudaStream_t s);
template <typename T>
cudaError_t launch_dp_det(const DetTileArgs<T>& a, int stencil, int rk4, int grid, cudaStream_t s);

constexpr int kMaxRowsPerTask = 16;
constexpr int RK_TX = 64, RK_TY = 32, RK_H = 4;
constexpr int RK_RX = RK_TX + 2 * RK_H, RK_RY = RK_TY + 2 * RK_H, RK_RN = RK_RX * RK_RY;
constexpr int RK_THREADS = 512;
constexpr int RK_CTAS = 2;                 // resident RK4 tile CTAs per SM (FP32)

}  // namespace tmg
