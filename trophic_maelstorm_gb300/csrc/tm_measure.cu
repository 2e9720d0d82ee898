// tm_measure.cu -- observables in FP64 with a fixed reduction order.
//
// mean_of_vector / occupied_sites_of_vector (stochasticSPDP.cpp:123-154) for
// every instance of a batch: one warp per task sums its strip (lanes own
// columns, rows in order), a butterfly of shuffles combines the lanes, and
// the per-task partials are summed per instance by one warp in task order.
// No atomics, so a given state always gives the same bits.
//
// GB300's FP64 rate is a small fraction of its FP32 rate, so the per-site work
// avoids FP64: active sites are counted with ballots, and an FP32 lane keeps
// the sum of its column's values (at most 16) as an unevaluated pair hi + lo
// by Knuth's TwoSum, which is exact up to the rounding of lo (relative 2^-48).
// The lanes' pairs are combined the same way through the shuffle butterfly
// (the values are non-negative, so nothing cancels), and lane 0 converts the
// task's pair to FP64.
#include "tm_device.cuh"
#include "tm_kernels.cuh"

namespace tmg {

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// hi + lo += v with hi the rounded sum and its error carried in lo (TwoSum; the
// kernels are built without contraction of multiply-adds, so every step rounds)
__device__ __forceinline__ void two_sum_add(float& hi, float& lo, float v)
{
    const float s = hi + v;
    const float bp = s - hi;
    const float e = (hi - (s - bp)) + (v - bp);
    hi = s;
    lo = lo + e;
}

template <typename T>
struct ColSum {
    T s = T(0);
    __device__ __forceinline__ void add(T v) { s += v; }
    __device__ __forceinline__ double warp_total() const { return warp_sum((double)s); }
};
template <>
struct ColSum<float> {
    float hi = 0.0f, lo = 0.0f;
    __device__ __forceinline__ void add(float v) { two_sum_add(hi, lo, v); }
    // sum over the warp, valid in lane 0
    __device__ __forceinline__ double warp_total() const
    {
        float h = hi, l = lo;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float ho = __shfl_down_sync(0xffffffffu, h, o);
            const float lo2 = __shfl_down_sync(0xffffffffu, l, o);
            two_sum_add(h, l, ho);
            l = l + lo2;
        }
        return (double)h + (double)l;
    }
};

// partial[t*4 + f]: f = 0..nf-1 field sums, 3 = sites with field 0 > 0.  With
// spread (DP), f = 1 is the sum over occupied sites of the squared distance
// (row - cy)^2 + (col - cx)^2 from the seed site (meansq_spread_of_vector,
// stochasticSPDP.cpp:156-170), summed as integers; cx, cy < 0 mean L/2.
constexpr int kChunk = 8;   // rows whose loads a warp issues together

template <typename T>
__global__ void __launch_bounds__(256) measure_kernel(const T* state, const InstTables it, const int4* tasks,
                                                      int n_tasks, int nf, double* partial, int spread, int scx,
                                                      int scy)
{
    const int lane = threadIdx.x & 31;
    const int gw = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int nw = (int)((gridDim.x * blockDim.x) >> 5);
    for (int t = gw; t < n_tasks; t += nw) {
        const int4 tk = tasks[t];
        const int k = tk.x;
        const int L = it.L[k];
        const int x = tk.y + lane;
        ColSum<T> c0, c1, c2;
        int ac = 0;
        long long sq = 0;
        const bool on = it.alive == nullptr || it.alive[k] != 0;   // warp-uniform
        if (on) {
            const T* base = state + it.off[k];
            const long long fs = it.fstride[k];
            const bool in = x < L;
            const long long cx = scx < 0 ? L / 2 : scx, cy = scy < 0 ? L / 2 : scy;
            // rows in chunks of kChunk: every load of a chunk is issued before the
            // sums use them (the state streams from HBM once; the sums keep row order)
            for (int r0 = 0; r0 < tk.w; r0 += kChunk) {
                T v0[kChunk], v1[kChunk], v2[kChunk];
#pragma unroll
                for (int j = 0; j < kChunk; ++j) {
                    const bool ok = in && r0 + j < tk.w;
                    const long long i = (long long)(tk.z + r0 + j) * L + x;
                    v0[j] = ok ? base[i] : T(0);
                    v1[j] = (nf == 3 && ok) ? base[i + fs] : T(0);
                    v2[j] = (nf == 3 && ok) ? base[i + 2 * fs] : T(0);
                }
#pragma unroll
                for (int j = 0; j < kChunk; ++j) {
                    if (r0 + j >= tk.w) break;
                    c0.add(v0[j]);
                    ac += __popc(__ballot_sync(0xffffffffu, v0[j] > T(0)));
                    if (spread && v0[j] > T(0)) {
                        const long long dy = (long long)(tk.z + r0 + j) - cy, dx = (long long)x - cx;
                        sq += dy * dy + dx * dx;
                    }
                    if (nf == 3 && in) {
                        c1.add(v1[j]);
                        c2.add(v2[j]);
                    }
                }
            }
        }
        const double s0 = c0.warp_total();
        double s1 = 0.0, s2 = 0.0;
        if (nf == 3) { s1 = c1.warp_total(); s2 = c2.warp_total(); }
        if (spread) s1 = warp_sum((double)sq);   // integers below 2^53: exact in any order
        if (lane == 0) {
            partial[4LL * t + 0] = s0;
            partial[4LL * t + 1] = s1;
            partial[4LL * t + 2] = s2;
            partial[4LL * t + 3] = (double)ac;
        }
    }
}

template <typename T>
cudaError_t launch_measure(const T* state, const InstTables& it, const int4* tasks, int n_tasks, int nf,
                           double* partial, int grid, int block, cudaStream_t s, int spread, int cx, int cy)
{
    if (n_tasks <= 0) return cudaSuccess;
    measure_kernel<T><<<grid, block, 0, s>>>(state, it, tasks, n_tasks, nf, partial, spread, cx, cy);
    return cudaGetLastError();
}
template cudaError_t launch_measure<float>(const float*, const InstTables&, const int4*, int, int, double*, int, int,
                                           cudaStream_t, int, int, int);
template cudaError_t launch_measure<double>(const double*, const InstTables&, const int4*, int, int, double*, int,
                                            int, cudaStream_t, int, int, int);

// Spreading runs stop once activity reaches the lattice's edge (theborderwall,
// stochasticSPDP.cpp:380-390, checked before every step at :1206-1213): one warp
// per live instance scans its four border rows/columns and marks it stopped
// (alive = 0, so later steps skip it and its later measurements are 0).
template <typename T>
__global__ void border_stop_kernel(const T* state, const InstTables it, int n_inst)
{
    const int lane = threadIdx.x & 31;
    const int k = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (k >= n_inst || it.alive[k] == 0) return;
    const int L = it.L[k];
    const T* base = state + it.off[k];
    bool hit = false;
    for (int i = lane; i < L; i += 32)
        hit = hit || base[i] > T(0) || base[(long long)i * L] > T(0) || base[(long long)(L - 1) * L + i] > T(0) ||
              base[(long long)i * L + L - 1] > T(0);
    if (__any_sync(0xffffffffu, hit) && lane == 0) it.alive[k] = 0;
}

template <typename T>
cudaError_t launch_border_stop(const T* state, const InstTables& it, int n_inst, cudaStream_t s)
{
    if (n_inst <= 0) return cudaSuccess;
    border_stop_kernel<T><<<(n_inst * 32 + 255) / 256, 256, 0, s>>>(state, it, n_inst);
    return cudaGetLastError();
}
template cudaError_t launch_border_stop<float>(const float*, const InstTables&, int, cudaStream_t);
template cudaError_t launch_border_stop<double>(const double*, const InstTables&, int, cudaStream_t);

// Status bits of an uploaded state, per instance: TM_STATUS_NAN_BIT for a NaN or
// Inf and TM_STATUS_NEG_BIT for a negative value in any field -- the checks the
// reference runs on every new state (multiSPDP.cpp:2949-2955, 3237-3255;
// rietkerk_bjork_FKE.cpp:4352-4370), applied to the state a caller uploads.
template <typename T>
__global__ void __launch_bounds__(256) validate_kernel(const T* state, const InstTables it, const int4* tasks,
                                                       int n_tasks, int nf)
{
    const int lane = threadIdx.x & 31;
    const int gw = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int nw = (int)((gridDim.x * blockDim.x) >> 5);
    for (int t = gw; t < n_tasks; t += nw) {
        const int4 tk = tasks[t];
        const int k = tk.x;
        const int L = it.L[k];
        const int x = tk.y + lane;
        unsigned st = 0;
        if (x < L) {
            const T* base = state + it.off[k];
            const long long fs = it.fstride[k];
            for (int f = 0; f < nf; ++f)
                for (int r0 = 0; r0 < tk.w; r0 += kChunk) {
                    T v[kChunk];
#pragma unroll
                    for (int j = 0; j < kChunk; ++j)
                        v[j] = r0 + j < tk.w ? base[f * fs + (long long)(tk.z + r0 + j) * L + x] : T(0);
#pragma unroll
                    for (int j = 0; j < kChunk; ++j) st |= value_status(v[j]);
                }
        }
        st = __reduce_or_sync(0xffffffffu, st);
        if (lane == 0 && st) atomicOr(it.status + k, st);
    }
}

template <typename T>
cudaError_t launch_validate(const T* state, const InstTables& it, const int4* tasks, int n_tasks, int nf, int grid,
                            cudaStream_t s)
{
    if (n_tasks <= 0) return cudaSuccess;
    validate_kernel<T><<<grid, 256, 0, s>>>(state, it, tasks, n_tasks, nf);
    return cudaGetLastError();
}
template cudaError_t launch_validate<float>(const float*, const InstTables&, const int4*, int, int, int, cudaStream_t);
template cudaError_t launch_validate<double>(const double*, const InstTables&, const int4*, int, int, int,
                                             cudaStream_t);

// Upload of a state from page-locked host memory: the device reads it over the host
// link, 16 bytes per load, grid-stride.  On GB300 machines the copy engines' host-to-device
// rate dropped from 211 to 18-30 GB/s in some copies after compute phases, while these
// loads of the same buffer held 212 GB/s.
__global__ void __launch_bounds__(512) copy_in_kernel(const uint4* __restrict__ src, uint4* __restrict__ dst,
                                                      long long n16)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += stride) dst[i] = src[i];
}

cudaError_t launch_copy_in(const void* src, void* dst, size_t bytes, int grid, cudaStream_t s)
{
    if (bytes == 0) return cudaSuccess;
    if (((uintptr_t)src | (uintptr_t)dst | (uintptr_t)bytes) & 15u) return cudaErrorInvalidValue;
    copy_in_kernel<<<grid, 512, 0, s>>>((const uint4*)src, (uint4*)dst, (long long)(bytes / 16));
    return cudaGetLastError();
}

// One warp per instance: obs_row[k*W + f], W = 2 (DP: mean, active), 3 (DP
// spreading: mean, active, summed squared distance) or 4 (Rietkerk: mean P, W, O,
// active P).  With dp_extinction, an instance seen with no active site is marked
// extinct (stochasticSPDP.cpp:1021-1022).
__global__ void finalize_kernel(const double* partial, const int* task_begin, const InstTables it, int n_inst, int nf,
                                int dp_extinction, int spread, double* obs_row)
{
    const int lane = threadIdx.x & 31;
    const int k = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (k >= n_inst) return;
    const int t0 = task_begin[k], t1 = task_begin[k + 1];
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, ac = 0.0;
    for (int t = t0 + lane; t < t1; t += 32) {
        s0 += partial[4LL * t + 0];
        s1 += partial[4LL * t + 1];
        s2 += partial[4LL * t + 2];
        ac += partial[4LL * t + 3];
    }
    s0 = warp_sum(s0); s1 = warp_sum(s1); s2 = warp_sum(s2); ac = warp_sum(ac);
    if (lane == 0) {
        const bool dead = it.alive != nullptr && it.alive[k] == 0;
        const double n = (double)it.L[k] * (double)it.L[k];
        if (nf == 1 && spread) {
            obs_row[3LL * k + 0] = dead ? 0.0 : s0 / n;
            obs_row[3LL * k + 1] = dead ? 0.0 : ac;
            obs_row[3LL * k + 2] = dead ? 0.0 : s1;
        } else if (nf == 1) {
            obs_row[2LL * k + 0] = dead ? 0.0 : s0 / n;
            obs_row[2LL * k + 1] = dead ? 0.0 : ac;
        } else {
            obs_row[4LL * k + 0] = s0 / n;
            obs_row[4LL * k + 1] = s1 / n;
            obs_row[4LL * k + 2] = s2 / n;
            obs_row[4LL * k + 3] = ac;
        }
        if (dp_extinction && it.alive != nullptr && ac == 0.0) it.alive[k] = 0;
    }
}

cudaError_t launch_finalize(const double* partial, const int* task_begin, const InstTables& it, int n_inst, int nf,
                            int dp_extinction, int spread, double* obs_row, cudaStream_t s)
{
    if (n_inst <= 0) return cudaSuccess;
    const int threads = 256;
    const int grid = (n_inst * 32 + threads - 1) / threads;
    finalize_kernel<<<grid, threads, 0, s>>>(partial, task_begin, it, n_inst, nf, dp_extinction, spread, obs_row);
    return cudaGetLastError();
}

}  // namespace tmg
