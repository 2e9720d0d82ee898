// tm_noalloc.cu -- observables of caller-owned device lattices without any
// device allocation (tm_observe_noalloc in include/tm.h).
//
// Who needs this: a host application that has already handed the GPU's memory
// to its own pool (a framework with a fixed device arena, a JVM or Go process
// that pre-reserves memory at start-up), or a latency-sensitive loop that must
// not pay cudaMalloc's implicit device synchronisation, cannot let a library
// call cudaMalloc behind its back.  The batch API allocates its state and its
// reduction scratch; this entry point only reads the caller's fields and
// writes the caller's output buffer.
//
// It is the observable reduction of tm_measure.cu (per-task FP64 partial sums
// in a fixed order, then one warp per instance), with its scratch -- the
// instance table, the task table and the per-task partials -- in the
// file-scope array below.  The array is TM_NOALLOC_SCRATCH_BYTES long and is
// part of the library image: every GPU that loads libtm.so holds it until the
// process exits.  Its device address is looked up once per device with
// cudaGetSymbolAddress (the host-side symbol is only a stand-in for it).
#include "../../include/tm.h"

#include <cuda_runtime.h>
#include <mutex>
#include <stdint.h>

namespace {

constexpr size_t kScratchBytes = TM_NOALLOC_SCRATCH_BYTES;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

// Scratch layout (each region 256-byte aligned):
//   int64 off[n_inst] | int32 L[n_inst] | int32 begin[n_inst + 1] | int2 task[n_tasks] | double2 partial[n_tasks]
struct Layout {
    size_t off, L, begin, task, partial, end;
};
__host__ __device__ inline size_t al256(size_t v) { return (v + 255) / 256 * 256; }
__host__ __device__ inline Layout layout_of(int n_inst, long long n_tasks)
{
    Layout y;
    y.off = 0;
    y.L = al256(y.off + (size_t)n_inst * 8);
    y.begin = al256(y.L + (size_t)n_inst * 4);
    y.task = al256(y.begin + (size_t)(n_inst + 1) * 4);
    y.partial = al256(y.task + (size_t)n_tasks * sizeof(int2));
    y.end = y.partial + (size_t)n_tasks * sizeof(double2);
    return y;
}

// Device address of the scratch on the current device (first call per device
// looks it up; later calls reuse it).
int scratch_on_current_device(unsigned char** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        (void)cudaGetLastError();
        return TM_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            (void)cudaGetLastError();
            return TM_ERR_CUDA;
        }
        g_scratch_ptr[dev] = (unsigned char*)p;
    }
    *out = g_scratch_ptr[dev];
    return TM_OK;
}

__global__ void na_tasks_kernel(unsigned char* scratch, int n_inst, long long n_tasks)
{
    // one thread lays out the column-strip tasks (n_inst is small); every
    // begin[] and task[] entry is rewritten on each call
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const Layout y = layout_of(n_inst, n_tasks);
    const int* L = (const int*)(scratch + y.L);
    int* begin = (int*)(scratch + y.begin);
    int2* tasks = (int2*)(scratch + y.task);
    int t = 0;
    for (int k = 0; k < n_inst; ++k) {
        begin[k] = t;
        for (int x0 = 0; x0 < L[k]; x0 += 32) tasks[t++] = make_int2(k, x0);
    }
    begin[n_inst] = t;
}

__device__ __forceinline__ double na_warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <typename T>
__global__ void __launch_bounds__(256) na_measure_kernel(const T* fields, unsigned char* scratch, int n_inst,
                                                         int n_tasks)
{
    const Layout y = layout_of(n_inst, n_tasks);
    const long long* off = (const long long*)(scratch + y.off);
    const int* Ls = (const int*)(scratch + y.L);
    const int2* tasks = (const int2*)(scratch + y.task);
    double2* partial = (double2*)(scratch + y.partial);
    const int lane = threadIdx.x & 31;
    const int gw = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int nw = (int)((gridDim.x * blockDim.x) >> 5);
    for (int t = gw; t < n_tasks; t += nw) {
        const int2 tk = tasks[t];
        const int L = Ls[tk.x];
        const int x = tk.y + lane;
        double s = 0.0, a = 0.0;
        if (x < L) {
            const T* base = fields + off[tk.x];
            for (int r = 0; r < L; ++r) {
                const T v = base[(long long)r * L + x];
                s += (double)v;
                if (v > T(0)) a += 1.0;
            }
        }
        s = na_warp_sum(s);
        a = na_warp_sum(a);
        if (lane == 0) partial[t] = make_double2(s, a);  // every partial is written before it is read
    }
}

__global__ void na_finalize_kernel(const unsigned char* scratch, int n_inst, int n_tasks, double* out)
{
    const Layout y = layout_of(n_inst, n_tasks);
    const int* Ls = (const int*)(scratch + y.L);
    const int* begin = (const int*)(scratch + y.begin);
    const double2* partial = (const double2*)(scratch + y.partial);
    const int lane = threadIdx.x & 31;
    const int k = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (k >= n_inst) return;
    double s = 0.0, a = 0.0;
    for (int t = begin[k] + lane; t < begin[k + 1]; t += 32) {
        s += partial[t].x;
        a += partial[t].y;
    }
    s = na_warp_sum(s);
    a = na_warp_sum(a);
    if (lane == 0) {
        const double n = (double)Ls[k] * (double)Ls[k];
        out[2LL * k + 0] = s / n;
        out[2LL * k + 1] = a;
    }
}

}  // namespace

extern "C" int tm_observe_noalloc(const void* dev_fields, int precision, const int32_t* L, const int64_t* offsets,
                                  int n_inst, double* dev_out, void* stream)
{
    if (!dev_fields || !L || !offsets || !dev_out || n_inst <= 0) return TM_ERR_INVALID;
    if (precision != TM_FP64 && precision != TM_FP32) return TM_ERR_INVALID;
    long long n_tasks = 0;
    for (int k = 0; k < n_inst; ++k) {
        if (L[k] < 1 || L[k] > 65535 || offsets[k] < 0) return TM_ERR_INVALID;
        n_tasks += (L[k] + 31) / 32;
    }
    const Layout y = layout_of(n_inst, n_tasks);
    if (y.end > kScratchBytes || n_tasks > 0x7fffffffLL) return TM_ERR_INVALID;  // beyond the built-in scratch
    unsigned char* scratch = nullptr;
    int rc = scratch_on_current_device(&scratch);
    if (rc != TM_OK) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    // instance tables straight from the caller's host arrays into the scratch
    if (cudaMemcpyAsync(scratch + y.off, offsets, (size_t)n_inst * 8, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(scratch + y.L, L, (size_t)n_inst * 4, cudaMemcpyHostToDevice, s) != cudaSuccess) {
        (void)cudaGetLastError();
        return TM_ERR_CUDA;
    }
    na_tasks_kernel<<<1, 1, 0, s>>>(scratch, n_inst, n_tasks);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long warps_needed = n_tasks;
    long long grid = (warps_needed + 7) / 8;
    const long long cap = (long long)(sms > 0 ? sms : 1) * 8;
    if (grid > cap) grid = cap;
    if (precision == TM_FP64)
        na_measure_kernel<double><<<(int)grid, 256, 0, s>>>((const double*)dev_fields, scratch, n_inst, (int)n_tasks);
    else
        na_measure_kernel<float><<<(int)grid, 256, 0, s>>>((const float*)dev_fields, scratch, n_inst, (int)n_tasks);
    na_finalize_kernel<<<(n_inst * 32 + 255) / 256, 256, 0, s>>>(scratch, n_inst, (int)n_tasks, dev_out);
    if (cudaGetLastError() != cudaSuccess) return TM_ERR_CUDA;
    return TM_OK;
}
