// tm_fke.cu -- FKE advection-diffusion of a consumer field, as a gather.
//
// The reference moves its consumer species with advdiff_FKE_MultiSp
// (simulations/Rietkerk_FPE/rietkerk_bjork_FKE.cpp:3614-3695) and, on the GPU,
// with updateMovement (kernel_advdiff_FKE2D.cu:92-180): every source site with
// rho >= eps scatters its mass through four separable Gaussian kernels
// (diffusion around the site, advection around the site shifted by
// round(v * pref), and the two mixed products), the reference kernel with FP64
// atomicAdd.  Here each target site gathers instead: for every source within
// reach it multiplies the row and column stencil sums over all periodic images
// of the target, so there are no atomics and the result does not depend on
// scheduling.  Reach = max(RD, RV + largest |shift|), the shift bound taken
// from the velocity field on the device.
#include "tm_kernels.cuh"
#include "../../include/tm.h"

#include <cuda_runtime.h>

namespace {

__device__ __forceinline__ int pmod(int p, int L)
{
    const int r = p % L;
    return r < 0 ? r + L : r;
}

// sum of g[|d + k L|] over the images k with |d + k L| <= R
template <typename T>
__device__ __forceinline__ T image_sum(const T* g, int R, int d, int L)
{
    T s = T(0);
    int k0 = -((R + d) / L) - 1;
    for (int k = k0; d + k * L <= R; ++k) {
        const int e = d + k * L;
        if (e >= -R) s = s + g[e < 0 ? -e : e];
    }
    return s;
}

template <typename T>
__global__ void fke_prep_kernel(const T* rho, const T* vx, const T* vy, int L, T pref, T eps, T* w, int* mux, int* muy,
                                int* smax)
{
    const int n = L * L;
    int local = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int ci = i / L, cj = i - ci * L;
        w[i] = (rho[i] < eps) ? T(0) : rho[i];
        const int sx = (int)round((T)ci + vx[i] * pref) - ci;
        const int sy = (int)round((T)cj + vy[i] * pref) - cj;
        mux[i] = pmod(ci + sx, L);
        muy[i] = pmod(cj + sy, L);
        local = max(local, max(abs(sx), abs(sy)));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) local = max(local, __shfl_xor_sync(0xffffffffu, local, o));
    if ((threadIdx.x & 31) == 0) atomicMax(smax, local);
}

template <typename T>
__global__ void fke_gather_kernel(const T* w, const T* gam, const int* mux, const int* muy, const int* smax, int L,
                                  const T* gD, int RD, const T* gV, int RV, T* out)
{
    __shared__ T sD[64], sV[64];
    for (int i = threadIdx.x; i <= RD; i += blockDim.x) sD[i] = gD[i];
    for (int i = threadIdx.x; i <= RV; i += blockDim.x) sV[i] = gV[i];
    __syncthreads();
    const int n = L * L;
    const int W = max(RD, RV + *smax);
    const bool all = 2 * W + 1 >= L;
    const int lo = all ? 0 : -W, hi = all ? L - 1 : W;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int ty = t / L, tx = t - ty * L;
        T acc = T(0);
        for (int oy = lo; oy <= hi; ++oy) {
            const int sy = all ? oy : pmod(ty - oy, L);
            for (int ox = lo; ox <= hi; ++ox) {
                const int sx = all ? ox : pmod(tx - ox, L);
                const int j = sy * L + sx;
                const T r = w[j];
                if (r == T(0)) continue;
                const T g = gam[j];
                const T g2 = g * g;
                const T SDr = image_sum(sD, RD, ty - sy, L), SDc = image_sum(sD, RD, tx - sx, L);
                const T SVr = image_sum(sV, RV, ty - mux[j], L), SVc = image_sum(sV, RV, tx - muy[j], L);
                const T wDV = (g - g2) * r;
                acc = acc + (g2 * r) * (SDr * SDc) + wDV * (SDr * SVc) + wDV * (SVr * SDc) +
                      (((T(1) - g) * (T(1) - g)) * r) * (SVr * SVc);
            }
        }
        out[t] = acc;
    }
}

template <typename T>
int run(const void* rho, const void* gam, const void* vx, const void* vy, int L, double pref, double eps,
        const double* gD, int RD, const double* gV, int RV, void* out, cudaStream_t s)
{
    const size_t n = (size_t)L * L;
    T *w = nullptr, *dgD = nullptr, *dgV = nullptr;
    int *mx = nullptr, *my = nullptr, *smax = nullptr;
    T hD[64], hV[64];
    for (int i = 0; i <= RD; ++i) hD[i] = (T)gD[i];
    for (int i = 0; i <= RV; ++i) hV[i] = (T)gV[i];
    int rc = TM_OK;
    if (cudaMalloc(&w, n * sizeof(T)) != cudaSuccess || cudaMalloc(&mx, n * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&my, n * sizeof(int)) != cudaSuccess || cudaMalloc(&smax, sizeof(int)) != cudaSuccess ||
        cudaMalloc(&dgD, 64 * sizeof(T)) != cudaSuccess || cudaMalloc(&dgV, 64 * sizeof(T)) != cudaSuccess) {
        rc = TM_ERR_NOMEM;
    } else {
        cudaMemsetAsync(smax, 0, sizeof(int), s);
        cudaMemcpyAsync(dgD, hD, (RD + 1) * sizeof(T), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(dgV, hV, (RV + 1) * sizeof(T), cudaMemcpyHostToDevice, s);
        const int grid = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
        fke_prep_kernel<T><<<grid, 256, 0, s>>>((const T*)rho, (const T*)vx, (const T*)vy, L, (T)pref, (T)eps, w, mx, my,
                                                smax);
        fke_gather_kernel<T><<<grid, 256, 0, s>>>(w, (const T*)gam, mx, my, smax, L, dgD, RD, dgV, RV, (T*)out);
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) rc = TM_ERR_CUDA;
    }
    cudaFree(w); cudaFree(mx); cudaFree(my); cudaFree(smax); cudaFree(dgD); cudaFree(dgV);
    (void)cudaGetLastError();
    return rc;
}

}  // namespace

extern "C" int tm_fke_advdiff_device(const void* dev_rho, const void* dev_gamma, const void* dev_vx,
                                     const void* dev_vy, int precision, int L, double pref, double eps,
                                     const double* gD, int RD, const double* gV, int RV, void* dev_out, void* stream)
{
    if (!dev_rho || !dev_gamma || !dev_vx || !dev_vy || !dev_out || !gD || !gV || L < 1 || L > 46340 || RD < 0 || RV < 0 ||
        RD > 63 || RV > 63)
        return TM_ERR_INVALID;
    if (precision == TM_FP64)
        return run<double>(dev_rho, dev_gamma, dev_vx, dev_vy, L, pref, eps, gD, RD, gV, RV, dev_out,
                           (cudaStream_t)stream);
    if (precision == TM_FP32)
        return run<float>(dev_rho, dev_gamma, dev_vx, dev_vy, L, pref, eps, gD, RD, gV, RV, dev_out,
                          (cudaStream_t)stream);
    return TM_ERR_INVALID;
}
