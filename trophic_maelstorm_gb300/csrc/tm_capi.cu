// tm_capi.cu -- the C ABI (include/tm.h): contexts, ragged batches and the
// step sequence.
//
// A batch packs every field of every instance into one device buffer
// (double-buffered: the Dornic step is a Jacobi update, the reference's
// Rho_dt/DRho pair, stochasticSPDP.cpp:983-984).  Work is cut into warp
// tasks (32 columns x R rows of one instance) for the Dornic and measurement
// kernels and into 32x16 tiles for the Rietkerk RK4 kernel; one persistent
// launch per kernel covers all instances, whatever their L.  Runs of steps
// between measurements replay CUDA graphs of G steps; the step index the
// Philox counter needs is read from device memory so one graph serves every
// chunk.
#include "tm_kernels.cuh"
#include "../../include/tm.h"

#include <cuda_runtime.h>
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

using namespace tmg;

namespace {

constexpr int kGraphSteps = 32;

bool cuda_ok(cudaError_t e) { return e == cudaSuccess; }

#define TM_CUDA(call)                      \
    do {                                   \
        cudaError_t e__ = (call);          \
        if (e__ != cudaSuccess) {          \
            (void)cudaGetLastError();      \
            return TM_ERR_CUDA;            \
        }                                  \
    } while (0)

template <typename P>
cudaError_t dalloc(P** p, size_t n)
{
    *p = nullptr;
    if (n == 0) return cudaSuccess;
    return cudaMalloc((void**)p, n * sizeof(P));
}

int64_t align_up(int64_t v, int64_t a) { return (v + a - 1) / a * a; }

}  // namespace

struct tm_batch {
    tm_ctx* ctx = nullptr;
    int model = 0;       // 0 DP, 1 Rietkerk
    int precision = 0;   // TM_FP64 / TM_FP32
    int nf = 1;
    int n_inst = 0;
    tm_dp_model dpm{};
    tm_rietkerk_model rkm{};
    std::vector<tm_instance> inst;
    std::vector<int64_t> off, fstride;
    int64_t total = 0;
    size_t esize = 8;

    void* buf[2] = {nullptr, nullptr};
    int cur = 0;
    void* aux = nullptr;        // Rietkerk P* (field-0 slots)
    uint4* d_dlist = nullptr;   // FP32: sites the straight-line draw deferred, a segment per warp of the grid
    unsigned* d_dcnt = nullptr;
    long long dlist_cap = 0, max_seg = 0;
    void* site_b = nullptr;     // per-site loss coefficient (DP), packed like the state
    long long* d_step = nullptr;
    int64_t step = 0;

    long long* d_off = nullptr;
    long long* d_fstride = nullptr;
    int* d_L = nullptr;
    unsigned long long* d_seed = nullptr;
    double* d_R = nullptr;
    double* d_a0 = nullptr;
    double* d_astep = nullptr;
    Dc4* d_consts = nullptr;
    int* d_alive = nullptr;
    unsigned* d_status = nullptr;
    bool ramped = false;

    unsigned probe = 0;         // TM_PROBE_* flags of the context when the batch was created
    int spreading = 0;          // DP spreading runs: squared-distance measurement, border stop
    int spread_cx = -1, spread_cy = -1;
    int rows_per_task = 8;
    int ctas_per_sm = 4;
    int4* d_tasks = nullptr;
    int n_tasks = 0;
    int* d_task_begin = nullptr;
    int4* d_btasks = nullptr;
    int n_btasks = 0;
    double* d_partial = nullptr;
    double* d_obs = nullptr;
    int obs_cap = 0;

    cudaGraphExec_t graph[2] = {nullptr, nullptr};

    InstTables tables() const
    {
        InstTables t;
        t.off = d_off; t.fstride = d_fstride; t.L = d_L; t.seed = d_seed; t.R = d_R;
        t.consts = d_consts; t.alive = d_alive; t.status = d_status;
        return t;
    }
};

namespace {

int obs_w(const tm_batch* b) { return b->model == 0 ? (b->spreading ? 3 : 2) : 4; }

void free_graphs(tm_batch* b)
{
    for (auto& g : b->graph) {
        if (g) cudaGraphExecDestroy(g);
        g = nullptr;
    }
}

// Rows per warp task for a new batch: 8, or fewer when the batch is too small
// to give every scheduler of the GPU two tasks (one 128^2 lattice is 64 tasks of
// 8 rows).  The results do not depend on the task shape.
int default_rows(const tm_batch* b)
{
    const long long want = 2LL * 4 * std::max(1, b->ctx->num_sms);
    int R = 8;
    for (; R > 1; R >>= 1) {
        long long n = 0;
        for (int k = 0; k < b->n_inst; ++k) {
            const long long L = b->inst[k].L;
            n += ((L + R - 1) / R) * ((L + 31) / 32);
        }
        if (n >= want) break;
    }
    return R;
}

int build_tasks(tm_batch* b)
{
    // warp tasks
    std::vector<int4> tasks;
    std::vector<int> begin(b->n_inst + 1, 0);
    const int R = b->rows_per_task;
    for (int k = 0; k < b->n_inst; ++k) {
        begin[k] = (int)tasks.size();
        const int L = b->inst[k].L;
        for (int y0 = 0; y0 < L; y0 += R)
            for (int x0 = 0; x0 < L; x0 += 32) tasks.push_back(make_int4(k, x0, y0, std::min(R, L - y0)));
    }
    begin[b->n_inst] = (int)tasks.size();
    if (tasks.size() > (size_t)0x7fffffff) return TM_ERR_INVALID;
    cudaFree(b->d_tasks); b->d_tasks = nullptr;
    cudaFree(b->d_partial); b->d_partial = nullptr;
    b->n_tasks = (int)tasks.size();
    TM_CUDA(dalloc(&b->d_tasks, tasks.size()));
    TM_CUDA(dalloc(&b->d_partial, 4 * tasks.size()));
    TM_CUDA(cudaMemcpy(b->d_tasks, tasks.data(), tasks.size() * sizeof(int4), cudaMemcpyHostToDevice));
    if (!b->d_task_begin) TM_CUDA(dalloc(&b->d_task_begin, begin.size()));
    TM_CUDA(cudaMemcpy(b->d_task_begin, begin.data(), begin.size() * sizeof(int), cudaMemcpyHostToDevice));
    // 64 x 32 tiles (Rietkerk RK4, noise-off DP)
    if ((b->model == 1 || b->dpm.deterministic) && !b->d_btasks) {
        std::vector<int4> bt;
        for (int k = 0; k < b->n_inst; ++k) {
            const int L = b->inst[k].L;
            for (int y0 = 0; y0 < L; y0 += RK_TY)
                for (int x0 = 0; x0 < L; x0 += RK_TX) bt.push_back(make_int4(k, x0, y0, 0));
        }
        b->n_btasks = (int)bt.size();
        TM_CUDA(dalloc(&b->d_btasks, bt.size()));
        TM_CUDA(cudaMemcpy(b->d_btasks, bt.data(), bt.size() * sizeof(int4), cudaMemcpyHostToDevice));
    }
    if (b->precision == TM_FP32) {
        // the deferred-site list: a step grid of nw warps gives every warp a segment of
        // ceil(n_tasks / nw) tasks' sites, nw * that <= (n_tasks + nw) * R * 32 entries;
        // sized for the largest grid (64 CTAs of 8 warps per SM, at most one warp per task)
        cudaFree(b->d_dlist); b->d_dlist = nullptr;
        cudaFree(b->d_dcnt); b->d_dcnt = nullptr;
        b->max_seg = std::min<long long>((long long)b->n_tasks + 8, (long long)std::max(1, b->ctx->num_sms) * 64 * 8);
        b->dlist_cap = ((long long)b->n_tasks + b->max_seg) * R * 32;
        TM_CUDA(dalloc(&b->d_dlist, (size_t)b->dlist_cap));
        TM_CUDA(dalloc(&b->d_dcnt, (size_t)b->max_seg));
    }
    free_graphs(b);
    return TM_OK;
}

int warp_grid(const tm_batch* b, int n_tasks)
{
    const int warps_per_cta = 8;
    const int need = (n_tasks + warps_per_cta - 1) / warps_per_cta;
    const int cap = std::max(1, b->ctx->num_sms * b->ctas_per_sm);
    return std::max(1, std::min(need, cap));
}

template <typename T>
DornicArgs<T> dornic_args(const tm_batch* b, const T* in, T* out, const long long* step_base, long long step_off)
{
    DornicArgs<T> a{};
    a.in = in; a.out = out; a.it = b->tables(); a.tasks = b->d_tasks; a.n_tasks = b->n_tasks;
    a.step_base = step_base; a.step_off = step_off; a.rows_cap = b->rows_per_task;
    a.cap1 = (b->probe & TM_PROBE_SAMPLER_CAP1) ? 1 : 0;
    a.dlist = b->d_dlist;
    a.dcnt = b->d_dcnt;
    a.dlist_cap = b->dlist_cap;
    a.max_seg = b->max_seg;
    {   // one list segment per warp of the step grid, holding all sites of that warp's tasks
        const long long nw = (long long)warp_grid(b, b->n_tasks) * 8;
        a.seg_cap = ((long long)b->n_tasks + nw - 1) / nw * b->rows_per_task * 32;
    }
    a.site_b = (b->model == 0) ? (const T*)b->site_b : nullptr;
    if (b->model == 0) {
        const tm_dp_model& m = b->dpm;
        a.dcoef = (T)(m.D / (m.dx * m.dx));
        a.two_s2 = (T)(2.0 / (m.sigma * m.sigma));
        a.b = (T)m.b; a.c = (T)m.c; a.dt = (T)m.dt; a.dt2 = (T)(m.dt / 2.0); a.dt6 = (T)(m.dt / 6.0);
        a.clo = (T)m.clamp_lo; a.ceps = (T)m.clamp_eps;
        a.sampler = m.sampler; a.cubic = (m.c != 0.0);
        // the remainder and the clamp map +0 to +0 whenever these are finite
        a.zero_fixed = a.site_b == nullptr && std::isfinite(a.b) && std::isfinite(a.c) && std::isfinite(a.dt) &&
                       std::isfinite(a.dt2) && std::isfinite(a.dt6);
    } else {
        const tm_rietkerk_model& m = b->rkm;
        a.dcoef = (T)(m.DP / (m.dx * m.dx));
        a.two_s2 = (T)(2.0 / (m.sigma * m.sigma));
        a.sampler = m.sampler;
        a.it.alive = nullptr;
        a.zero_fixed = 1;  // no remainder, no clamp
    }
    return a;
}

template <typename T>
RK4Args<T> rk4_args(const tm_batch* b, const T* in, const T* pstar, T* out)
{
    const tm_rietkerk_model& m = b->rkm;
    RK4Args<T> a{};
    a.in = in; a.pstar = pstar; a.out = out; a.it = b->tables(); a.it.alive = nullptr;
    a.tasks = b->d_btasks; a.n_tasks = b->n_btasks;
    const double dx2 = m.dx * m.dx;
    a.alpha = (T)m.alpha; a.k2 = (T)m.k2; a.k2W0 = (T)(m.k2 * m.W0); a.gmax = (T)m.gmax;
    a.cgmax = (T)(m.c * m.gmax); a.k1 = (T)m.k1; a.rW = (T)m.rW; a.d = (T)m.d;
    a.DPx = (T)(m.DP / dx2); a.DWx = (T)(m.DW / dx2); a.DOx = (T)(m.DO / dx2);
    a.dt2 = (T)(m.dt / 2.0); a.dt6 = (T)(m.dt / 6.0); a.dt = (T)m.dt;
    a.clo = (T)m.clamp_lo; a.ceps = (T)m.clamp_eps;
    a.probe_no_copy = (b->probe & TM_PROBE_TILE_WAIT) ? 1 : 0;
    a.wait_limit = a.probe_no_copy ? (1 << 14) : (1 << 22);
    return a;
}

// Queue one step reading buf[src_idx], writing buf[src_idx ^ 1].
template <typename T>
cudaError_t enqueue_step_t(tm_batch* b, int src_idx, const long long* step_base, long long step_off)
{
    cudaStream_t s = b->ctx->stream;
    const T* in = (const T*)b->buf[src_idx];
    T* out = (T*)b->buf[src_idx ^ 1];
    cudaError_t e = cudaSuccess;
    if (b->model == 0) {
        const tm_dp_model& m = b->dpm;
        if (m.deterministic) {
            // noise-off lattice RK4 / Euler: one tile launch for every instance
            DetTileArgs<T> d{};
            d.in = in; d.out = out; d.it = b->tables(); d.tasks = b->d_btasks; d.n_tasks = b->n_btasks;
            d.b = (T)m.b; d.c = (T)m.c; d.cubic = (m.c != 0.0);
            d.dlap = (T)(m.D / (m.dx * m.dx));
            d.dk12 = (T)(m.D * (1.0 / ((12.0 * m.dx) * m.dx)));
            d.dt = (T)m.dt; d.dt2 = (T)(m.dt / 2.0); d.dt6 = (T)(m.dt / 6.0);
            const int grid = std::max(1, std::min(b->n_btasks, b->ctx->num_sms * 2));
            return launch_dp_det<T>(d, m.stencil, m.integrator, grid, s);
        }
        if (b->ramped) {
            e = launch_consts(b->d_a0, b->d_astep, b->n_inst, (4.0 * m.D) / (m.dx * m.dx), m.sigma * m.sigma, m.dt,
                              step_base, step_off, b->d_consts, s);
            if (e != cudaSuccess) return e;
        }
        DornicArgs<T> a = dornic_args<T>(b, in, out, step_base, step_off);
        e = launch_dornic<T>(a, m.remainder == TM_REM_RK4 ? 1 : 0, warp_grid(b, b->n_tasks), 256, s);
        if (e == cudaSuccess && b->spreading) e = launch_border_stop<T>(out, b->tables(), b->n_inst, s);
        return e;
    }
    const tm_rietkerk_model& m = b->rkm;
    const int grid_rk = std::max(1, std::min(b->n_btasks, b->ctx->num_sms * RK_CTAS));
    if (m.deterministic) {
        RK4Args<T> r = rk4_args<T>(b, in, nullptr, out);
        return launch_rk4<T>(r, true, grid_rk, s);
    }
    DornicArgs<T> a = dornic_args<T>(b, in, (T*)b->aux, step_base, step_off);
    e = launch_dornic<T>(a, 2, warp_grid(b, b->n_tasks), 256, s);
    if (e != cudaSuccess) return e;
    RK4Args<T> r = rk4_args<T>(b, in, (const T*)b->aux, out);
    return launch_rk4<T>(r, false, grid_rk, s);
}

cudaError_t enqueue_step(tm_batch* b, int src_idx, const long long* step_base, long long step_off)
{
    return b->precision == TM_FP64 ? enqueue_step_t<double>(b, src_idx, step_base, step_off)
                                   : enqueue_step_t<float>(b, src_idx, step_base, step_off);
}

int ensure_graph(tm_batch* b, int parity)
{
    if (b->graph[parity]) return TM_OK;
    cudaStream_t s = b->ctx->stream;
    cudaGraph_t g = nullptr;
    TM_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < kGraphSteps && e == cudaSuccess; ++k) e = enqueue_step(b, (parity + k) & 1, b->d_step, k);
    cudaError_t e2 = cudaStreamEndCapture(s, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        (void)cudaGetLastError();
        return TM_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&b->graph[parity], g, 0);
    cudaGraphDestroy(g);
    TM_CUDA(e);
    return TM_OK;
}

// Queue n steps from the current step (no measurements).
int run_steps(tm_batch* b, int64_t n)
{
    cudaStream_t s = b->ctx->stream;
    while (n > 0) {
        if (n >= kGraphSteps) {
            int rc = ensure_graph(b, b->cur);
            if (rc != TM_OK) return rc;
            TM_CUDA(launch_set_step(b->d_step, b->step, s));
            TM_CUDA(cudaGraphLaunch(b->graph[b->cur], s));
            b->step += kGraphSteps;
            n -= kGraphSteps;
            // kGraphSteps is even: the current buffer is unchanged
        } else {
            TM_CUDA(enqueue_step(b, b->cur, nullptr, b->step));
            b->cur ^= 1;
            b->step += 1;
            n -= 1;
        }
    }
    return TM_OK;
}

int measure_into(tm_batch* b, int j)
{
    cudaStream_t s = b->ctx->stream;
    const int W = obs_w(b);
    InstTables it = b->tables();
    if (b->model == 1) it.alive = nullptr;
    const int grid = warp_grid(b, b->n_tasks);
    cudaError_t e;
    if (b->precision == TM_FP64)
        e = launch_measure<double>((const double*)b->buf[b->cur], it, b->d_tasks, b->n_tasks, b->nf, b->d_partial,
                                   grid, 256, s, b->spreading, b->spread_cx, b->spread_cy);
    else
        e = launch_measure<float>((const float*)b->buf[b->cur], it, b->d_tasks, b->n_tasks, b->nf, b->d_partial, grid,
                                  256, s, b->spreading, b->spread_cx, b->spread_cy);
    TM_CUDA(e);
    TM_CUDA(launch_finalize(b->d_partial, b->d_task_begin, it, b->n_inst, b->nf, b->model == 0, b->spreading,
                            b->d_obs + (size_t)j * b->n_inst * W, s));
    return TM_OK;
}

int validate_instances(const tm_instance* inst, int n)
{
    if (!inst || n <= 0) return TM_ERR_INVALID;
    for (int k = 0; k < n; ++k)
        if (inst[k].L < 1 || inst[k].L > 65535) return TM_ERR_INVALID;
    return TM_OK;
}

int batch_common_init(tm_batch* b, const tm_instance* inst, int n)
{
    b->n_inst = n;
    b->inst.assign(inst, inst + n);
    b->off.resize(n);
    b->fstride.resize(n);
    b->total = tm_layout(inst, n, b->nf, b->off.data(), b->fstride.data());
    b->esize = b->precision == TM_FP64 ? 8 : 4;
    TM_CUDA(cudaMalloc(&b->buf[0], (size_t)b->total * b->esize));
    TM_CUDA(cudaMalloc(&b->buf[1], (size_t)b->total * b->esize));
    TM_CUDA(cudaMemset(b->buf[0], 0, (size_t)b->total * b->esize));
    TM_CUDA(cudaMemset(b->buf[1], 0, (size_t)b->total * b->esize));
    std::vector<long long> off(b->off.begin(), b->off.end()), fs(b->fstride.begin(), b->fstride.end());
    std::vector<int> L(n);
    std::vector<unsigned long long> seed(n);
    std::vector<double> a0(n), ast(n);
    for (int k = 0; k < n; ++k) {
        L[k] = inst[k].L; seed[k] = inst[k].seed; a0[k] = inst[k].a; ast[k] = inst[k].a_step;
    }
    TM_CUDA(dalloc(&b->d_off, n)); TM_CUDA(dalloc(&b->d_fstride, n)); TM_CUDA(dalloc(&b->d_L, n));
    TM_CUDA(dalloc(&b->d_seed, n)); TM_CUDA(dalloc(&b->d_R, n)); TM_CUDA(dalloc(&b->d_a0, n));
    TM_CUDA(dalloc(&b->d_astep, n)); TM_CUDA(dalloc(&b->d_consts, n)); TM_CUDA(dalloc(&b->d_alive, n));
    TM_CUDA(dalloc(&b->d_status, n)); TM_CUDA(dalloc(&b->d_step, 1));
    TM_CUDA(cudaMemcpy(b->d_off, off.data(), n * sizeof(long long), cudaMemcpyHostToDevice));
    TM_CUDA(cudaMemcpy(b->d_fstride, fs.data(), n * sizeof(long long), cudaMemcpyHostToDevice));
    TM_CUDA(cudaMemcpy(b->d_L, L.data(), n * sizeof(int), cudaMemcpyHostToDevice));
    TM_CUDA(cudaMemcpy(b->d_seed, seed.data(), n * sizeof(unsigned long long), cudaMemcpyHostToDevice));
    TM_CUDA(cudaMemcpy(b->d_R, a0.data(), n * sizeof(double), cudaMemcpyHostToDevice));
    TM_CUDA(cudaMemcpy(b->d_a0, a0.data(), n * sizeof(double), cudaMemcpyHostToDevice));
    TM_CUDA(cudaMemcpy(b->d_astep, ast.data(), n * sizeof(double), cudaMemcpyHostToDevice));
    std::vector<int> ones(n, 1);
    TM_CUDA(cudaMemcpy(b->d_alive, ones.data(), n * sizeof(int), cudaMemcpyHostToDevice));
    TM_CUDA(cudaMemset(b->d_status, 0, n * sizeof(unsigned)));
    TM_CUDA(cudaMemset(b->d_step, 0, sizeof(long long)));

    b->probe = b->ctx->probe;
    b->rows_per_task = default_rows(b);
    return build_tasks(b);
}

int obs_reserve(tm_batch* b, int n_meas)
{
    if (n_meas <= b->obs_cap) return TM_OK;
    const int W = obs_w(b);
    cudaFree(b->d_obs);
    b->d_obs = nullptr;
    TM_CUDA(dalloc(&b->d_obs, (size_t)n_meas * b->n_inst * W));
    b->obs_cap = n_meas;
    return TM_OK;
}

}  // namespace

// ======================================================================= C ABI
extern "C" {

int tm_abi_version(void) { return TM_ABI_VERSION; }

const char* tm_error_string(int code)
{
    switch (code) {
    case TM_OK: return "ok";
    case TM_ERR_INVALID: return "invalid argument";
    case TM_ERR_CUDA: return "CUDA runtime error";
    case TM_ERR_NOMEM: return "out of memory";
    case TM_ERR_STATE: return "invalid state for this call";
    case TM_ERR_TIMEOUT: return "a bounded device wait ran out";
    default: return "unknown error";
    }
}

int64_t tm_layout(const tm_instance* inst, int n_inst, int nf, int64_t* offsets, int64_t* field_strides)
{
    int64_t o = 0;
    for (int k = 0; k < n_inst; ++k) {
        const int64_t L = inst[k].L;
        const int64_t fs = align_up(L * L, 32);
        if (offsets) offsets[k] = o;
        if (field_strides) field_strides[k] = fs;
        o += nf * fs;
    }
    return o;
}

int tm_create(tm_ctx** out, int device)
{
    if (!out) return TM_ERR_INVALID;
    *out = nullptr;
    int n = 0;
    TM_CUDA(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return TM_ERR_INVALID;
    TM_CUDA(cudaSetDevice(device));
    tm_ctx* c = new (std::nothrow) tm_ctx;
    if (!c) return TM_ERR_NOMEM;
    c->device = device;
    if (!cuda_ok(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device)) ||
        !cuda_ok(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking))) {
        delete c;
        (void)cudaGetLastError();
        return TM_ERR_CUDA;
    }
    *out = c;
    return TM_OK;
}

int tm_destroy(tm_ctx* c)
{
    if (!c) return TM_ERR_INVALID;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    cudaStreamDestroy(c->stream);
    delete c;
    return TM_OK;
}

void* tm_stream(tm_ctx* c) { return c ? (void*)c->stream : nullptr; }

int tm_set_test_probe(tm_ctx* c, uint32_t flags)
{
    if (!c || (flags & ~(TM_PROBE_SAMPLER_CAP1 | TM_PROBE_TILE_WAIT | TM_PROBE_MLP_WAIT))) return TM_ERR_INVALID;
    c->probe = flags;
    return TM_OK;
}

int tm_sync(tm_ctx* c)
{
    if (!c) return TM_ERR_INVALID;
    TM_CUDA(cudaStreamSynchronize(c->stream));
    return TM_OK;
}

int tm_batch_destroy(tm_batch* b)
{
    if (!b) return TM_ERR_INVALID;
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    free_graphs(b);
    cudaFree(b->buf[0]); cudaFree(b->buf[1]); cudaFree(b->aux); cudaFree(b->site_b);
    cudaFree(b->d_dlist); cudaFree(b->d_dcnt);
    cudaFree(b->d_step); cudaFree(b->d_off); cudaFree(b->d_fstride); cudaFree(b->d_L); cudaFree(b->d_seed);
    cudaFree(b->d_R); cudaFree(b->d_a0); cudaFree(b->d_astep); cudaFree(b->d_consts); cudaFree(b->d_alive);
    cudaFree(b->d_status); cudaFree(b->d_tasks); cudaFree(b->d_task_begin); cudaFree(b->d_btasks);
    cudaFree(b->d_partial); cudaFree(b->d_obs);
    delete b;
    return TM_OK;
}

int tm_batch_create_dp(tm_ctx* c, const tm_dp_model* m, const tm_instance* inst, int n_inst, int precision,
                       tm_batch** out)
{
    if (!c || !m || !out) return TM_ERR_INVALID;
    *out = nullptr;
    int rc = validate_instances(inst, n_inst);
    if (rc) return rc;
    if (precision != TM_FP64 && precision != TM_FP32) return TM_ERR_INVALID;
    if (!(m->dt > 0) || !(m->dx > 0) || !(m->D >= 0)) return TM_ERR_INVALID;
    if (m->deterministic) {
        if ((m->stencil != TM_STENCIL_5 && m->stencil != TM_STENCIL_9) || (m->integrator != 0 && m->integrator != 1))
            return TM_ERR_INVALID;
    } else {
        if (m->remainder != TM_REM_EULER_EXACT && m->remainder != TM_REM_RK4) return TM_ERR_INVALID;
        if (m->sampler < 0 || m->sampler > 2) return TM_ERR_INVALID;
        if (m->sampler != TM_SAMPLER_OFF && !(m->sigma > 0)) return TM_ERR_INVALID;
    }
    // the sampler-cap probe exists for the Euler-exact, exact-sampler Dornic step only
    if ((c->probe & TM_PROBE_SAMPLER_CAP1) &&
        (m->deterministic || m->remainder != TM_REM_EULER_EXACT || m->sampler != TM_SAMPLER_EXACT))
        return TM_ERR_INVALID;
    TM_CUDA(cudaSetDevice(c->device));
    tm_batch* b = new (std::nothrow) tm_batch;
    if (!b) return TM_ERR_NOMEM;
    b->ctx = c; b->model = 0; b->precision = precision; b->nf = 1; b->dpm = *m;
    for (int k = 0; k < n_inst; ++k) b->ramped = b->ramped || inst[k].a_step != 0.0;
    rc = batch_common_init(b, inst, n_inst);
    if (rc == TM_OK && !m->deterministic) {
        if (!cuda_ok(launch_consts(b->d_a0, b->d_astep, n_inst, (4.0 * m->D) / (m->dx * m->dx),
                                   m->sigma * m->sigma, m->dt, nullptr, 0, b->d_consts, c->stream)) ||
            !cuda_ok(cudaStreamSynchronize(c->stream)))
            rc = TM_ERR_CUDA;
    }
    if (rc != TM_OK) {
        tm_batch_destroy(b);
        return rc;
    }
    *out = b;
    return TM_OK;
}

int tm_batch_create_rietkerk(tm_ctx* c, const tm_rietkerk_model* m, const tm_instance* inst, int n_inst,
                             int precision, tm_batch** out)
{
    if (!c || !m || !out) return TM_ERR_INVALID;
    *out = nullptr;
    int rc = validate_instances(inst, n_inst);
    if (rc) return rc;
    if (precision != TM_FP64 && precision != TM_FP32) return TM_ERR_INVALID;
    if (!(m->dt > 0) || !(m->dx > 0)) return TM_ERR_INVALID;
    if (!m->deterministic && (m->sampler < 0 || m->sampler > 2)) return TM_ERR_INVALID;
    if (!m->deterministic && m->sampler != TM_SAMPLER_OFF && !(m->sigma > 0)) return TM_ERR_INVALID;
    if (c->probe & TM_PROBE_SAMPLER_CAP1) return TM_ERR_INVALID;
    TM_CUDA(cudaSetDevice(c->device));
    tm_batch* b = new (std::nothrow) tm_batch;
    if (!b) return TM_ERR_NOMEM;
    b->ctx = c; b->model = 1; b->precision = precision; b->nf = 3; b->rkm = *m;
    rc = batch_common_init(b, inst, n_inst);
    if (rc == TM_OK && !m->deterministic) {
        if (!cuda_ok(cudaMalloc(&b->aux, (size_t)b->total * b->esize))) rc = TM_ERR_NOMEM;
        // P's linear part -d and its diffusion form the Dornic step (rietkerk_bjork_FKE.cpp:3847-3849)
        std::vector<double> lin(n_inst, -m->d), zero(n_inst, 0.0);
        double* d_lin = nullptr;
        double* d_zero = nullptr;
        if (rc == TM_OK &&
            (!cuda_ok(dalloc(&d_lin, n_inst)) || !cuda_ok(dalloc(&d_zero, n_inst)) ||
             !cuda_ok(cudaMemcpy(d_lin, lin.data(), n_inst * sizeof(double), cudaMemcpyHostToDevice)) ||
             !cuda_ok(cudaMemcpy(d_zero, zero.data(), n_inst * sizeof(double), cudaMemcpyHostToDevice)) ||
             !cuda_ok(launch_consts(d_lin, d_zero, n_inst, (4.0 * m->DP) / (m->dx * m->dx), m->sigma * m->sigma,
                                    m->dt, nullptr, 0, b->d_consts, c->stream)) ||
             !cuda_ok(cudaStreamSynchronize(c->stream))))
            rc = TM_ERR_CUDA;
        cudaFree(d_lin);
        cudaFree(d_zero);
    }
    if (rc != TM_OK) {
        tm_batch_destroy(b);
        return rc;
    }
    *out = b;
    return TM_OK;
}

int64_t tm_batch_total_elems(const tm_batch* b) { return b ? b->total : -1; }
int64_t tm_batch_instance_offset(const tm_batch* b, int k) { return (b && k >= 0 && k < b->n_inst) ? b->off[k] : -1; }
int64_t tm_batch_field_stride(const tm_batch* b, int k) { return (b && k >= 0 && k < b->n_inst) ? b->fstride[k] : -1; }
int tm_batch_num_fields(const tm_batch* b) { return b ? b->nf : -1; }
int tm_batch_obs_width(const tm_batch* b) { return b ? obs_w(b) : -1; }
int64_t tm_batch_step(const tm_batch* b) { return b ? b->step : -1; }

// After an upload: step counter, extinction flags, and the status bits of the
// uploaded state itself (NaN/Inf, negative values).
static int reset_after_upload(tm_batch* b, int64_t step)
{
    b->step = step;
    cudaStream_t s = b->ctx->stream;
    std::vector<int> ones(b->n_inst, 1);
    TM_CUDA(cudaMemcpyAsync(b->d_alive, ones.data(), b->n_inst * sizeof(int), cudaMemcpyHostToDevice, s));
    TM_CUDA(cudaMemsetAsync(b->d_status, 0, b->n_inst * sizeof(unsigned), s));
    InstTables it = b->tables();
    const int grid = warp_grid(b, b->n_tasks);
    TM_CUDA(b->precision == TM_FP64
                ? launch_validate<double>((const double*)b->buf[b->cur], it, b->d_tasks, b->n_tasks, b->nf, grid, s)
                : launch_validate<float>((const float*)b->buf[b->cur], it, b->d_tasks, b->n_tasks, b->nf, grid, s));
    TM_CUDA(cudaStreamSynchronize(s));
    return TM_OK;
}

int tm_batch_upload(tm_batch* b, const void* host, int64_t step)
{
    if (!b || !host || step < 0) return TM_ERR_INVALID;
    TM_CUDA(cudaSetDevice(b->ctx->device));
    const size_t bytes = (size_t)b->total * b->esize;
    // page-locked host memory mapped into the device's address space: read by a copy
    // kernel; any other host memory: through the copy engines
    const void* mapped = nullptr;
    cudaPointerAttributes pa{};
    if (cudaPointerGetAttributes(&pa, host) == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer)
        mapped = pa.devicePointer;
    (void)cudaGetLastError();
    if (mapped && ((uintptr_t)mapped & 15u) == 0 && (bytes & 15u) == 0)
        TM_CUDA(launch_copy_in(mapped, b->buf[b->cur], bytes, b->ctx->num_sms * 4, b->ctx->stream));
    else
        TM_CUDA(cudaMemcpyAsync(b->buf[b->cur], host, bytes, cudaMemcpyHostToDevice, b->ctx->stream));
    return reset_after_upload(b, step);
}

int tm_batch_upload_device(tm_batch* b, const void* dev, int64_t step)
{
    if (!b || !dev || step < 0) return TM_ERR_INVALID;
    TM_CUDA(cudaSetDevice(b->ctx->device));
    TM_CUDA(cudaMemcpyAsync(b->buf[b->cur], dev, (size_t)b->total * b->esize, cudaMemcpyDeviceToDevice,
                            b->ctx->stream));
    return reset_after_upload(b, step);
}

static int zero_extinct_host(tm_batch* b, void* host)
{
    if (b->model != 0) return TM_OK;
    std::vector<int> alive(b->n_inst);
    TM_CUDA(cudaMemcpy(alive.data(), b->d_alive, b->n_inst * sizeof(int), cudaMemcpyDeviceToHost));
    for (int k = 0; k < b->n_inst; ++k)
        if (!alive[k])
            std::memset((char*)host + (size_t)b->off[k] * b->esize, 0, (size_t)b->nf * b->fstride[k] * b->esize);
    return TM_OK;
}

int tm_batch_download(tm_batch* b, void* host)
{
    if (!b || !host) return TM_ERR_INVALID;
    TM_CUDA(cudaSetDevice(b->ctx->device));
    TM_CUDA(cudaMemcpyAsync(host, b->buf[b->cur], (size_t)b->total * b->esize, cudaMemcpyDeviceToHost, b->ctx->stream));
    TM_CUDA(cudaStreamSynchronize(b->ctx->stream));
    return zero_extinct_host(b, host);
}

int tm_batch_download_device(tm_batch* b, void* dev)
{
    if (!b || !dev) return TM_ERR_INVALID;
    TM_CUDA(cudaSetDevice(b->ctx->device));
    TM_CUDA(cudaMemcpyAsync(dev, b->buf[b->cur], (size_t)b->total * b->esize, cudaMemcpyDeviceToDevice,
                            b->ctx->stream));
    TM_CUDA(cudaStreamSynchronize(b->ctx->stream));
    if (b->model == 0) {
        std::vector<int> alive(b->n_inst);
        TM_CUDA(cudaMemcpy(alive.data(), b->d_alive, b->n_inst * sizeof(int), cudaMemcpyDeviceToHost));
        for (int k = 0; k < b->n_inst; ++k)
            if (!alive[k])
                TM_CUDA(cudaMemset((char*)dev + (size_t)b->off[k] * b->esize, 0,
                                   (size_t)b->nf * b->fstride[k] * b->esize));
    }
    return TM_OK;
}

int tm_batch_snapshot(tm_batch* b, int k, void* host_out)
{
    if (!b || !host_out || k < 0 || k >= b->n_inst) return TM_ERR_INVALID;
    TM_CUDA(cudaSetDevice(b->ctx->device));
    const size_t n = (size_t)b->inst[k].L * b->inst[k].L;
    int alive = 1;
    if (b->model == 0) TM_CUDA(cudaMemcpy(&alive, b->d_alive + k, sizeof(int), cudaMemcpyDeviceToHost));
    for (int f = 0; f < b->nf; ++f) {
        char* dst = (char*)host_out + f * n * b->esize;
        if (!alive) {
            std::memset(dst, 0, n * b->esize);
            continue;
        }
        TM_CUDA(cudaMemcpyAsync(dst, (char*)b->buf[b->cur] + (size_t)(b->off[k] + f * b->fstride[k]) * b->esize,
                                n * b->esize, cudaMemcpyDeviceToHost, b->ctx->stream));
    }
    TM_CUDA(cudaStreamSynchronize(b->ctx->stream));
    return TM_OK;
}

int tm_batch_advance(tm_batch* b, int64_t n_steps, const int64_t* meas, int n_meas, double* obs, uint32_t* status)
{
    if (!b || n_steps < 0 || n_meas < 0 || (n_meas > 0 && (!meas || !obs))) return TM_ERR_INVALID;
    const int64_t s0 = b->step, end = s0 + n_steps;
    for (int j = 0; j < n_meas; ++j) {
        if (meas[j] < s0 || meas[j] > end) return TM_ERR_INVALID;
        if (j > 0 && meas[j] < meas[j - 1]) return TM_ERR_INVALID;
    }
    TM_CUDA(cudaSetDevice(b->ctx->device));
    int rc = obs_reserve(b, n_meas);
    if (rc) return rc;
    if (b->spreading) {  // the border check of the state about to be measured and stepped
        cudaError_t e = b->precision == TM_FP64
                            ? launch_border_stop<double>((const double*)b->buf[b->cur], b->tables(), b->n_inst,
                                                         b->ctx->stream)
                            : launch_border_stop<float>((const float*)b->buf[b->cur], b->tables(), b->n_inst,
                                                        b->ctx->stream);
        TM_CUDA(e);
    }
    int j = 0;
    while (true) {
        while (j < n_meas && meas[j] == b->step) {
            rc = measure_into(b, j);
            if (rc) return rc;
            ++j;
        }
        if (b->step == end) break;
        const int64_t target = (j < n_meas) ? meas[j] : end;
        rc = run_steps(b, target - b->step);
        if (rc) return rc;
    }
    const int W = obs_w(b);
    if (n_meas > 0)
        TM_CUDA(cudaMemcpyAsync(obs, b->d_obs, (size_t)n_meas * b->n_inst * W * sizeof(double),
                                cudaMemcpyDeviceToHost, b->ctx->stream));
    std::vector<uint32_t> st_local;
    uint32_t* st = status;
    if (!st) {
        st_local.resize(b->n_inst);
        st = st_local.data();
    }
    TM_CUDA(cudaMemcpyAsync(st, b->d_status, b->n_inst * sizeof(unsigned), cudaMemcpyDeviceToHost, b->ctx->stream));
    TM_CUDA(cudaStreamSynchronize(b->ctx->stream));
    for (int k = 0; k < b->n_inst; ++k)
        if (st[k] & TM_STATUS_WAIT_TIMEOUT) return TM_ERR_TIMEOUT;
    return TM_OK;
}

int tm_batch_enqueue_steps(tm_batch* b, int64_t n_steps)
{
    if (!b || n_steps < 0) return TM_ERR_INVALID;
    TM_CUDA(cudaSetDevice(b->ctx->device));
    return run_steps(b, n_steps);
}

int tm_batch_set_launch(tm_batch* b, int rows, int ctas)
{
    if (!b || rows < 0 || ctas < 0 || rows > kMaxRowsPerTask || ctas > 64) return TM_ERR_INVALID;
    TM_CUDA(cudaSetDevice(b->ctx->device));
    TM_CUDA(cudaStreamSynchronize(b->ctx->stream));
    bool rebuild = false;
    if (rows > 0 && rows != b->rows_per_task) { b->rows_per_task = rows; rebuild = true; }
    if (ctas > 0 && ctas != b->ctas_per_sm) { b->ctas_per_sm = ctas; free_graphs(b); }
    return rebuild ? build_tasks(b) : TM_OK;
}

int tm_batch_get_launch(const tm_batch* b, int* rows, int* ctas)
{
    if (!b) return TM_ERR_INVALID;
    if (rows) *rows = b->rows_per_task;
    if (ctas) *ctas = b->ctas_per_sm;
    return TM_OK;
}

int tm_batch_autotune(tm_batch* b, int steps_per_trial)
{
    if (!b || steps_per_trial < 1) return TM_ERR_INVALID;
    TM_CUDA(cudaSetDevice(b->ctx->device));
    cudaStream_t s = b->ctx->stream;
    // save state, counters and flags so the trials leave no trace
    void* save = nullptr;
    TM_CUDA(cudaMalloc(&save, (size_t)b->total * b->esize));
    std::vector<int> alive(b->n_inst);
    std::vector<unsigned> status(b->n_inst);
    TM_CUDA(cudaMemcpyAsync(save, b->buf[b->cur], (size_t)b->total * b->esize, cudaMemcpyDeviceToDevice, s));
    TM_CUDA(cudaMemcpyAsync(alive.data(), b->d_alive, b->n_inst * sizeof(int), cudaMemcpyDeviceToHost, s));
    TM_CUDA(cudaMemcpyAsync(status.data(), b->d_status, b->n_inst * sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    TM_CUDA(cudaStreamSynchronize(s));
    const int64_t step0 = b->step;
    const int cur0 = b->cur;
    const int rows_c[] = {1, 2, 4, 8, 16};
    const int ctas_c[] = {1, 2, 3, 4};
    int best_r = b->rows_per_task, best_c = b->ctas_per_sm;
    float best = 1e30f;
    cudaEvent_t e0, e1;
    TM_CUDA(cudaEventCreate(&e0));
    TM_CUDA(cudaEventCreate(&e1));
    int rc = TM_OK;
    for (int r : rows_c) {
        for (int c : ctas_c) {
            rc = tm_batch_set_launch(b, r, c);
            if (rc) break;
            b->step = step0; b->cur = cur0;
            rc = run_steps(b, 1);  // warm-up (also builds nothing: single step)
            if (rc) break;
            cudaEventRecord(e0, s);
            rc = run_steps(b, steps_per_trial);
            if (rc) break;
            cudaEventRecord(e1, s);
            if (!cuda_ok(cudaEventSynchronize(e1))) { rc = TM_ERR_CUDA; break; }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) { best = ms; best_r = r; best_c = c; }
            // restore
            b->cur = cur0;
            cudaMemcpyAsync(b->buf[b->cur], save, (size_t)b->total * b->esize, cudaMemcpyDeviceToDevice, s);
            cudaMemcpyAsync(b->d_alive, alive.data(), b->n_inst * sizeof(int), cudaMemcpyHostToDevice, s);
            cudaStreamSynchronize(s);
        }
        if (rc) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->step = step0; b->cur = cur0;
    cudaMemcpyAsync(b->buf[b->cur], save, (size_t)b->total * b->esize, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(b->d_alive, alive.data(), b->n_inst * sizeof(int), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(b->d_status, status.data(), b->n_inst * sizeof(unsigned), cudaMemcpyHostToDevice, s);
    cudaStreamSynchronize(s);
    cudaFree(save);
    if (rc) return rc;
    return tm_batch_set_launch(b, best_r, best_c);
}

int tm_batch_set_spreading(tm_batch* b, int enable, int cx, int cy)
{
    if (!b || b->model != 0 || b->dpm.deterministic || cx < -1 || cy < -1) return TM_ERR_INVALID;
    for (int k = 0; k < b->n_inst; ++k)
        if (cx >= b->inst[k].L || cy >= b->inst[k].L) return TM_ERR_INVALID;
    TM_CUDA(cudaSetDevice(b->ctx->device));
    TM_CUDA(cudaStreamSynchronize(b->ctx->stream));
    b->spreading = enable ? 1 : 0;
    b->spread_cx = cx;
    b->spread_cy = cy;
    free_graphs(b);
    cudaFree(b->d_obs);   // the measurement width changed
    b->d_obs = nullptr;
    b->obs_cap = 0;
    return TM_OK;
}

int tm_batch_set_site_coeff(tm_batch* b, const void* host_coeff)
{
    if (!b || b->model != 0 || b->dpm.deterministic) return TM_ERR_INVALID;
    TM_CUDA(cudaSetDevice(b->ctx->device));
    TM_CUDA(cudaStreamSynchronize(b->ctx->stream));
    if (!host_coeff) {
        cudaFree(b->site_b);
        b->site_b = nullptr;
    } else {
        if (!b->site_b && !cuda_ok(cudaMalloc(&b->site_b, (size_t)b->total * b->esize))) return TM_ERR_NOMEM;
        TM_CUDA(cudaMemcpy(b->site_b, host_coeff, (size_t)b->total * b->esize, cudaMemcpyHostToDevice));
    }
    free_graphs(b);
    return TM_OK;
}

int tm_batch_box_means(tm_batch* b, int k, int field, int box, double* out)
{
    if (!b || !out || k < 0 || k >= b->n_inst || field < 0 || field >= b->nf || box < 1) return TM_ERR_INVALID;
    const int L = b->inst[k].L;
    if (L % box != 0) return TM_ERR_INVALID;
    TM_CUDA(cudaSetDevice(b->ctx->device));
    const size_t nb = (size_t)(L / box) * (L / box);
    int alive = 1;
    if (b->model == 0) TM_CUDA(cudaMemcpy(&alive, b->d_alive + k, sizeof(int), cudaMemcpyDeviceToHost));
    if (!alive) {
        for (size_t i = 0; i < nb; ++i) out[i] = 0.0;
        return TM_OK;
    }
    double* d = nullptr;
    TM_CUDA(cudaMalloc(&d, nb * sizeof(double)));
    const char* base = (const char*)b->buf[b->cur] + (size_t)(b->off[k] + field * b->fstride[k]) * b->esize;
    cudaError_t e = b->precision == TM_FP64
                        ? launch_box_means<double>((const double*)base, L, box, d, b->ctx->stream)
                        : launch_box_means<float>((const float*)base, L, box, d, b->ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d, nb * sizeof(double), cudaMemcpyDeviceToHost, b->ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->ctx->stream);
    cudaFree(d);
    TM_CUDA(e);
    return TM_OK;
}

int tm_batch_power_spectrum(tm_batch* b, int k, int field, double binwidth, double* kvals, double* power,
                            int max_bins, int* n_bins)
{
    if (!b || k < 0 || k >= b->n_inst || field < 0 || field >= b->nf) return TM_ERR_INVALID;
    TM_CUDA(cudaSetDevice(b->ctx->device));
    int alive = 1;
    if (b->model == 0) TM_CUDA(cudaMemcpy(&alive, b->d_alive + k, sizeof(int), cudaMemcpyDeviceToHost));
    if (!alive) {  // an extinct instance is all zeros: no power at any k
        const int L = b->inst[k].L;
        int rc = tm_power_spectrum_device(b->buf[b->cur], b->precision, L, binwidth, b->ctx->stream, kvals, power,
                                          max_bins, n_bins);
        if (rc == TM_OK)
            for (int i = 0; i < *n_bins; ++i) power[i] = 0.0;
        return rc;
    }
    const char* base = (const char*)b->buf[b->cur] + (size_t)(b->off[k] + field * b->fstride[k]) * b->esize;
    return tm_power_spectrum_device(base, b->precision, b->inst[k].L, binwidth, b->ctx->stream, kvals, power,
                                    max_bins, n_bins);
}

static int run_common(tm_batch* b, const void* init, int64_t n_steps, const int64_t* meas, int n_meas, double* obs,
                      uint32_t* status, void* fin)
{
    int rc = tm_batch_upload(b, init, 0);
    if (rc == TM_OK) rc = tm_batch_advance(b, n_steps, meas, n_meas, obs, status);
    if (rc == TM_OK && fin) rc = tm_batch_download(b, fin);
    return rc;
}

int tm_run_dp(tm_ctx* c, const tm_dp_model* m, const tm_instance* inst, int n_inst, int precision, const void* init,
              int64_t n_steps, const int64_t* meas, int n_meas, double* obs, uint32_t* status, void* fin)
{
    if (!init) return TM_ERR_INVALID;
    tm_batch* b = nullptr;
    int rc = tm_batch_create_dp(c, m, inst, n_inst, precision, &b);
    if (rc) return rc;
    rc = run_common(b, init, n_steps, meas, n_meas, obs, status, fin);
    tm_batch_destroy(b);
    return rc;
}

int tm_run_rietkerk(tm_ctx* c, const tm_rietkerk_model* m, const tm_instance* inst, int n_inst, int precision,
                    const void* init, int64_t n_steps, const int64_t* meas, int n_meas, double* obs,
                    uint32_t* status, void* fin)
{
    if (!init) return TM_ERR_INVALID;
    tm_batch* b = nullptr;
    int rc = tm_batch_create_rietkerk(c, m, inst, n_inst, precision, &b);
    if (rc) return rc;
    rc = run_common(b, init, n_steps, meas, n_meas, obs, status, fin);
    tm_batch_destroy(b);
    return rc;
}

}  // extern "C"
