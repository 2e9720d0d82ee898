// tm_spectrum.cu -- radially averaged power spectrum of a lattice on the GPU.
//
// Semantics of gen_FFT_PowerSpectra (simulations/Utilities/glow_up.py:752-827),
// the reference's pattern-wavelength estimator: the field is divided by its
// maximum (unless that is 0), transformed by a 2-D FFT in double precision,
// |F(k)|^2 is averaged over annuli k in [e_b, e_{b+1}) with e_b = 1 - w/2 + b w
// (the last bin closed, as numpy.histogram), and each bin mean is multiplied by
// the annulus area pi (e_{b+1}^2 - e_b^2).  Empty bins are 0 (the reference
// turns them into NaN afterwards).  The wavelength is L / k at the peak.
//
// The FFT is cuFFT's D2Z (half spectrum); columns with a mirror image count
// twice.  The bins depend only on L, so the elements of each bin are listed
// once on the host (CSR) and each bin is summed by one warp in list order:
// the result does not depend on scheduling.
#include "tm_kernels.cuh"
#include "../../include/tm.h"

#include <cuda_runtime.h>
#include <cufft.h>
#include <cmath>
#include <vector>

namespace {

__device__ __forceinline__ double wsum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <typename T>
__global__ void max_partial_kernel(const T* f, long long n, double* part)
{
    __shared__ double red[32];
    double m = -INFINITY;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        m = fmax(m, (double)f[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : -INFINITY;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0) part[blockIdx.x] = m;
    }
}

__global__ void max_final_kernel(double* part, int n)
{
    double m = -INFINITY;
    for (int i = threadIdx.x; i < n; i += 32) m = fmax(m, part[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) part[0] = (m != 0.0) ? m : 1.0;
}

template <typename T>
__global__ void normalise_kernel(const T* f, long long n, const double* mx, double* out)
{
    const double m = *mx;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = (double)f[i] / m;
}

// one warp per bin: sum of w * |F|^2 over the bin's listed elements, in list order
__global__ void bin_kernel(const cufftDoubleComplex* F, const int* ptr, const int* idx, const unsigned char* w,
                           int nbins, const double* area, double* power)
{
    const int lane = threadIdx.x & 31;
    const int b = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (b >= nbins) return;
    double s = 0.0, c = 0.0;
    for (int j = ptr[b] + lane; j < ptr[b + 1]; j += 32) {
        const cufftDoubleComplex z = F[idx[j]];
        const double p = z.x * z.x + z.y * z.y;
        s += (double)w[j] * p;
        c += (double)w[j];
    }
    s = wsum(s);
    c = wsum(c);
    if (lane == 0) power[b] = (c != 0.0) ? (s / c) * area[b] : 0.0;
}

struct Plan {
    int L = 0;
    double bw = 0;
    int nbins = 0;
    std::vector<double> kvals, area;
    std::vector<int> ptr, idx;
    std::vector<unsigned char> w;
};

void make_plan(int L, double bw, Plan& p)
{
    p.L = L;
    p.bw = bw;
    // edges: numpy.arange(1 - bw/2, L//2 + 1, bw)
    std::vector<double> e;
    const double start = 1.0 - bw / 2.0, stop = (double)(L / 2 + 1);
    const long long ne = (long long)std::ceil((stop - start) / bw);
    for (long long i = 0; i < ne; ++i) e.push_back(start + (double)i * bw);
    p.nbins = e.size() > 1 ? (int)e.size() - 1 : 0;
    p.kvals.resize(p.nbins);
    p.area.resize(p.nbins);
    for (int b = 0; b < p.nbins; ++b) {
        p.kvals[b] = 0.5 * (e[b + 1] + e[b]);
        p.area[b] = M_PI * (e[b + 1] * e[b + 1] - e[b] * e[b]);
    }
    const int nx = L / 2 + 1;
    std::vector<std::vector<int>> per(p.nbins);
    std::vector<std::vector<unsigned char>> pw(p.nbins);
    for (int ky = 0; ky < L; ++ky) {
        const long long fy = (ky <= (L - 1) / 2) ? ky : ky - L;
        for (int kx = 0; kx < nx; ++kx) {
            const double k = std::sqrt((double)(kx * (long long)kx + fy * fy));
            if (p.nbins == 0 || k < e[0] || k > e[p.nbins]) continue;
            int b = (int)((k - e[0]) / bw);
            if (b >= p.nbins) b = p.nbins - 1;
            while (b > 0 && k < e[b]) --b;
            while (b < p.nbins - 1 && k >= e[b + 1]) ++b;
            const bool mirrored = kx >= 1 && kx <= (L - 1) / 2;
            per[b].push_back(ky * nx + kx);
            pw[b].push_back(mirrored ? 2 : 1);
        }
    }
    p.ptr.assign(p.nbins + 1, 0);
    for (int b = 0; b < p.nbins; ++b) p.ptr[b + 1] = p.ptr[b] + (int)per[b].size();
    p.idx.clear();
    p.w.clear();
    for (int b = 0; b < p.nbins; ++b) {
        p.idx.insert(p.idx.end(), per[b].begin(), per[b].end());
        p.w.insert(p.w.end(), pw[b].begin(), pw[b].end());
    }
}

}  // namespace

extern "C" int tm_power_spectrum_device(const void* dev_field, int precision, int L, double binwidth, void* stream,
                                        double* kvals, double* power, int max_bins, int* n_bins)
{
    if (!dev_field || L < 2 || !(binwidth > 0) || !kvals || !power || !n_bins || max_bins < 0) return TM_ERR_INVALID;
    if (precision != TM_FP64 && precision != TM_FP32) return TM_ERR_INVALID;
    Plan p;
    make_plan(L, binwidth, p);
    *n_bins = p.nbins;
    if (p.nbins > max_bins) return TM_ERR_INVALID;
    if (p.nbins == 0) return TM_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const long long n = (long long)L * L;
    const int nx = L / 2 + 1;
    double* img = nullptr;
    cufftDoubleComplex* F = nullptr;
    double *part = nullptr, *d_area = nullptr, *d_pow = nullptr;
    int *d_ptr = nullptr, *d_idx = nullptr;
    unsigned char* d_w = nullptr;
    int rc = TM_OK;
    cufftHandle plan = 0;
    bool have_plan = false;
    const int nblk = 304;
    auto ok = [&](cudaError_t e) { if (e != cudaSuccess && rc == TM_OK) rc = TM_ERR_CUDA; return rc == TM_OK; };
    if (ok(cudaMalloc(&img, n * sizeof(double))) && ok(cudaMalloc(&F, (size_t)L * nx * sizeof(cufftDoubleComplex))) &&
        ok(cudaMalloc(&part, nblk * sizeof(double))) && ok(cudaMalloc(&d_area, p.nbins * sizeof(double))) &&
        ok(cudaMalloc(&d_pow, p.nbins * sizeof(double))) && ok(cudaMalloc(&d_ptr, (p.nbins + 1) * sizeof(int))) &&
        ok(cudaMalloc(&d_idx, p.idx.size() * sizeof(int) + 4)) && ok(cudaMalloc(&d_w, p.w.size() + 4)) &&
        ok(cudaMemcpyAsync(d_area, p.area.data(), p.nbins * sizeof(double), cudaMemcpyHostToDevice, s)) &&
        ok(cudaMemcpyAsync(d_ptr, p.ptr.data(), (p.nbins + 1) * sizeof(int), cudaMemcpyHostToDevice, s)) &&
        ok(cudaMemcpyAsync(d_idx, p.idx.data(), p.idx.size() * sizeof(int), cudaMemcpyHostToDevice, s)) &&
        ok(cudaMemcpyAsync(d_w, p.w.data(), p.w.size(), cudaMemcpyHostToDevice, s))) {
        if (precision == TM_FP64) {
            max_partial_kernel<double><<<nblk, 256, 0, s>>>((const double*)dev_field, n, part);
            max_final_kernel<<<1, 32, 0, s>>>(part, nblk);
            normalise_kernel<double><<<nblk, 256, 0, s>>>((const double*)dev_field, n, part, img);
        } else {
            max_partial_kernel<float><<<nblk, 256, 0, s>>>((const float*)dev_field, n, part);
            max_final_kernel<<<1, 32, 0, s>>>(part, nblk);
            normalise_kernel<float><<<nblk, 256, 0, s>>>((const float*)dev_field, n, part, img);
        }
        ok(cudaGetLastError());
        if (rc == TM_OK && cufftPlan2d(&plan, L, L, CUFFT_D2Z) == CUFFT_SUCCESS) {
            have_plan = true;
            if (cufftSetStream(plan, s) != CUFFT_SUCCESS || cufftExecD2Z(plan, img, F) != CUFFT_SUCCESS) rc = TM_ERR_CUDA;
        } else if (rc == TM_OK) {
            rc = TM_ERR_CUDA;
        }
        if (rc == TM_OK) {
            bin_kernel<<<(p.nbins * 32 + 255) / 256, 256, 0, s>>>(F, d_ptr, d_idx, d_w, p.nbins, d_area, d_pow);
            ok(cudaGetLastError());
            ok(cudaMemcpyAsync(power, d_pow, p.nbins * sizeof(double), cudaMemcpyDeviceToHost, s));
            ok(cudaStreamSynchronize(s));
            for (int b = 0; b < p.nbins; ++b) kvals[b] = p.kvals[b];
        }
    }
    if (have_plan) cufftDestroy(plan);
    cudaFree(img); cudaFree(F); cudaFree(part); cudaFree(d_area); cudaFree(d_pow);
    cudaFree(d_ptr); cudaFree(d_idx); cudaFree(d_w);
    (void)cudaGetLastError();
    return rc;
}
