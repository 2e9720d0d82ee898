// fke_scatter_ref.cu -- TEST INFRASTRUCTURE ONLY: the reference's GPU design of the
// consumer movement, restated for a same-box comparison with the library's gather.
//
// The reference moves a consumer field on the GPU with updateMovement
// (simulations/Rietkerk_FPE/kernel_advdiff_FKE2D.cu:92-180, launched with 256-thread
// blocks and one thread per site at :226-235): each source site with rho >= eps
// adds its mass, split by gamma into the diffusion/advection products, to every
// site under the four separable stencil products, with FP64 atomicAdd.  This file
// restates that scatter for one species (the reference loops over species with
// per-species offsets into the stencils), with its periodic wrap written as a
// proper modulo.  Only tests/ and oracle/time_fke_scatter.py load it; the library
// never links it.
#include <cuda_runtime.h>

namespace {

__device__ __forceinline__ int wrap(int p, int L)
{
    const int r = p % L;
    return r < 0 ? r + L : r;
}

__global__ void fke_scatter_kernel(const double* rho, const double* gam, const double* vx, const double* vy, int L,
                                   double pref, double eps, const double* gD, int RD, const double* gV, int RV,
                                   double* out)
{
    const int n = L * L;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double m = rho[i];
        if (m < eps) continue;
        const int ci = i / L, cj = i % L;
        const double g = gam[i];
        const double wdd = g * g * m, wdv = g * (1.0 - g) * m, wvv = (1.0 - g) * (1.0 - g) * m;
        const int mx = wrap((int)round(ci + vx[i] * pref), L);
        const int my = wrap((int)round(cj + vy[i] * pref), L);
        // rows around the site: diffusion x diffusion, then diffusion x advection
        for (int p = ci - RD; p <= ci + RD; ++p) {
            const double gx = gD[abs(p - ci)];
            const int row = wrap(p, L) * L;
            for (int q = cj - RD; q <= cj + RD; ++q) atomicAdd(out + row + wrap(q, L), wdd * (gx * gD[abs(q - cj)]));
            for (int q = my - RV; q <= my + RV; ++q) atomicAdd(out + row + wrap(q, L), wdv * (gx * gV[abs(q - my)]));
        }
        // rows around the shifted site: advection x diffusion, then advection x advection
        for (int p = mx - RV; p <= mx + RV; ++p) {
            const double gx = gV[abs(p - mx)];
            const int row = wrap(p, L) * L;
            for (int q = cj - RD; q <= cj + RD; ++q) atomicAdd(out + row + wrap(q, L), wdv * (gx * gD[abs(q - cj)]));
            for (int q = my - RV; q <= my + RV; ++q) atomicAdd(out + row + wrap(q, L), wvv * (gx * gV[abs(q - my)]));
        }
    }
}

}  // namespace

// out (device, L*L) is zeroed and then receives the moved field; gD, gV are device
// arrays of RD + 1 and RV + 1 values.  Queues work on `stream` and returns the
// launch status.
extern "C" int tmo_fke_scatter_f64(const double* rho, const double* gam, const double* vx, const double* vy, int L,
                                   double pref, double eps, const double* gD, int RD, const double* gV, int RV,
                                   double* out, void* stream)
{
    if (L < 1 || RD < 0 || RV < 0) return -1;
    cudaStream_t s = (cudaStream_t)stream;
    if (cudaMemsetAsync(out, 0, (size_t)L * L * sizeof(double), s) != cudaSuccess) return -2;
    const int threads = 256;
    const int blocks = (L * L + threads - 1) / threads;
    fke_scatter_kernel<<<blocks, threads, 0, s>>>(rho, gam, vx, vy, L, pref, eps, gD, RD, gV, RV, out);
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}
