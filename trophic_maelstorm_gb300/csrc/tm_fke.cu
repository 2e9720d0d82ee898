// tm_fke.cu -- FKE advection-diffusion of a consumer field, as separable gathers.
//
// The reference moves its consumer species with advdiff_FKE_MultiSp
// (simulations/Rietkerk_FPE/rietkerk_bjork_FKE.cpp:3614-3695) and, on the GPU,
// with updateMovement (kernel_advdiff_FKE2D.cu:92-180): every source site with
// rho >= eps scatters its mass through four separable Gaussian stencils
// (diffusion around the site, advection around the site shifted by
// round(v * pref), and the two mixed products), the reference kernel with FP64
// atomicAdd.  Here the four terms are grouped by their row stencil and
// gathered in two passes, with no atomics (the result does not depend on
// scheduling):
//   pass 1, along rows:  A_D[r][q] = sum over the sources of row r of
//                                    wDD gD(q - cj) + wDV gV(q - muy)
//                        A_V[r][q] = the same sum over the sources whose
//                                    shifted row mux is r, of wDV gD(q - cj) + wVV gV(q - muy)
//   pass 2, down columns: out[p][q] = sum_r gD(p - r) A_D[r][q] + gV(p - r) A_V[r][q]
// with wDD = gamma^2 rho, wDV = gamma (1 - gamma) rho, wVV = (1 - gamma)^2 rho,
// and gD, gV the stencils wrapped onto the periodic lattice (summed over
// every image, so lattices narrower than a stencil are exact).  A site then
// costs about (2W + 1)(2 + 2(2S + 1)) + 2RD + 2RV + 2 multiply-adds, W the
// source window max(RD, RV + S) and S the largest shift, against the
// (2W + 1)^2 sources a direct gather visits.
#include "tm_kernels.cuh"
#include "../../include/tm.h"

#include <cuda_runtime.h>

#include <stdint.h>
#include <vector>

namespace {

__device__ __forceinline__ int pmod(int p, int L)
{
    const int r = p % L;
    return r < 0 ? r + L : r;
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

// offsets o of a window [-R, R] taken mod L: each residue once (all of them when 2R+1 >= L)
__device__ __forceinline__ void window(int R, int L, int& lo, int& hi)
{
    if (2 * R + 1 >= L) { lo = 0; hi = L - 1; }
    else { lo = -R; hi = R; }
}

// pass 1: A_D and A_V of one (row r, column q)
template <typename T>
__global__ void fke_rows_kernel(const T* w, const T* gam, const int* mux, const int* muy, const int* smax, int L,
                                const T* gDw, const T* gVw, int RD, int RV, T* AD, T* AV)
{
    const int n = L * L;
    const int S = *smax;
    int wlo, whi, slo, shi;
    window(max(RD, RV + S), L, wlo, whi);
    window(S, L, slo, shi);
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int r = t / L, q = t - r * L;
        T ad = T(0), av = T(0);
        for (int o = wlo; o <= whi; ++o) {
            const int cj = pmod(q - o, L);
            const int j = r * L + cj;
            const T rv = w[j];
            if (rv == T(0)) continue;
            const T g = gam[j];
            const T g2 = g * g;
            ad = ad + (g2 * rv) * gDw[pmod(q - cj, L)] + ((g - g2) * rv) * gVw[pmod(q - muy[j], L)];
        }
        for (int so = slo; so <= shi; ++so) {
            const int ci = pmod(r - so, L);
            for (int o = wlo; o <= whi; ++o) {
                const int cj = pmod(q - o, L);
                const int j = ci * L + cj;
                if (mux[j] != r) continue;
                const T rv = w[j];
                if (rv == T(0)) continue;
                const T g = gam[j];
                av = av + ((g - g * g) * rv) * gDw[pmod(q - cj, L)] +
                     (((T(1) - g) * (T(1) - g)) * rv) * gVw[pmod(q - muy[j], L)];
            }
        }
        AD[t] = ad;
        AV[t] = av;
    }
}

// pass 2: out[p][q] = sum_d gD(d) A_D[p - d][q] + gV(d) A_V[p - d][q]
template <typename T>
__global__ void fke_cols_kernel(const T* AD, const T* AV, int L, const T* gDw, const T* gVw, int RD, int RV, T* out)
{
    const int n = L * L;
    int dlo, dhi, vlo, vhi;
    window(RD, L, dlo, dhi);
    window(RV, L, vlo, vhi);
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int p = t / L, q = t - p * L;
        T acc = T(0);
        for (int d = dlo; d <= dhi; ++d) acc = acc + gDw[pmod(d, L)] * AD[pmod(p - d, L) * L + q];
        for (int d = vlo; d <= vhi; ++d) acc = acc + gVw[pmod(d, L)] * AV[pmod(p - d, L) * L + q];
        out[t] = acc;
    }
}

// Workspace of one call (each region 256-byte aligned): w, A_D, A_V (T, L^2 each),
// mux, muy (int, L^2 each), the wrapped stencils gDw, gVw (T, L each), smax (int).
struct FkeLayout {
    size_t w, AD, AV, mx, my, gD, gV, smax, end;
};
inline size_t al256(size_t v) { return (v + 255) / 256 * 256; }
inline FkeLayout fke_layout(size_t esize, int L)
{
    const size_t n = (size_t)L * L;
    FkeLayout y;
    y.w = 0;
    y.AD = al256(y.w + n * esize);
    y.AV = al256(y.AD + n * esize);
    y.mx = al256(y.AV + n * esize);
    y.my = al256(y.mx + n * sizeof(int));
    y.gD = al256(y.my + n * sizeof(int));
    y.gV = al256(y.gD + (size_t)L * esize);
    y.smax = al256(y.gV + (size_t)L * esize);
    y.end = y.smax + 256;
    return y;
}

// Stencils passed by value (the workspace entry point copies nothing from the host).
struct FkeStencils {
    double gD[TM_FKE_WS_MAX_RADIUS + 1];
    double gV[TM_FKE_WS_MAX_RADIUS + 1];
    int RD, RV;
};

// The stencils wrapped onto the lattice: residue i gets every g[|d|] with
// d = i (mod L), |d| <= R, added in increasing d in FP64 and rounded once --
// the same sums the host forms for the allocating entry point.
template <typename T>
__global__ void fke_wrap_kernel(const FkeStencils st, int L, T* gDw, T* gVw)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < L; i += gridDim.x * blockDim.x) {
        double sd = 0.0, sv = 0.0;
        for (int d = -st.RD; d <= st.RD; ++d)
            if (pmod(d, L) == i) sd += st.gD[d < 0 ? -d : d];
        for (int d = -st.RV; d <= st.RV; ++d)
            if (pmod(d, L) == i) sv += st.gV[d < 0 ? -d : d];
        gDw[i] = (T)sd;
        gVw[i] = (T)sv;
    }
}

// The three passes on a caller-sized workspace whose wrapped stencils are already
// set (or queued) on stream s; nothing is allocated and nothing waits.
template <typename T>
cudaError_t enqueue_passes(const void* rho, const void* gam, const void* vx, const void* vy, int L, double pref,
                           double eps, int RD, int RV, void* out, unsigned char* ws, cudaStream_t s)
{
    const FkeLayout y = fke_layout(sizeof(T), L);
    T* w = (T*)(ws + y.w);
    T* AD = (T*)(ws + y.AD);
    T* AV = (T*)(ws + y.AV);
    int* mx = (int*)(ws + y.mx);
    int* my = (int*)(ws + y.my);
    const T* dgD = (const T*)(ws + y.gD);
    const T* dgV = (const T*)(ws + y.gV);
    int* smax = (int*)(ws + y.smax);
    const size_t n = (size_t)L * L;
    cudaError_t e = cudaMemsetAsync(smax, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    const int grid = (int)((n + 255) / 256 < 8192 ? (n + 255) / 256 : 8192);
    fke_prep_kernel<T><<<grid, 256, 0, s>>>((const T*)rho, (const T*)vx, (const T*)vy, L, (T)pref, (T)eps, w, mx, my,
                                            smax);
    fke_rows_kernel<T><<<grid, 256, 0, s>>>(w, (const T*)gam, mx, my, smax, L, dgD, dgV, RD, RV, AD, AV);
    fke_cols_kernel<T><<<grid, 256, 0, s>>>(AD, AV, L, dgD, dgV, RD, RV, (T*)out);
    return cudaGetLastError();
}

template <typename T>
int run(const void* rho, const void* gam, const void* vx, const void* vy, int L, double pref, double eps,
        const double* gD, int RD, const double* gV, int RV, void* out, cudaStream_t s)
{
    // the stencils wrapped onto the lattice: every image d = delta (mod L) of |d| <= R summed
    std::vector<double> wd(L, 0.0), wv(L, 0.0);
    for (int d = -RD; d <= RD; ++d) wd[((d % L) + L) % L] += gD[d < 0 ? -d : d];
    for (int d = -RV; d <= RV; ++d) wv[((d % L) + L) % L] += gV[d < 0 ? -d : d];
    std::vector<T> hd(wd.begin(), wd.end()), hv(wv.begin(), wv.end());
    const FkeLayout y = fke_layout(sizeof(T), L);
    unsigned char* ws = nullptr;
    int rc = TM_OK;
    if (cudaMalloc(&ws, y.end) != cudaSuccess) {
        rc = TM_ERR_NOMEM;
    } else if (cudaMemcpyAsync(ws + y.gD, hd.data(), L * sizeof(T), cudaMemcpyHostToDevice, s) != cudaSuccess ||
               cudaMemcpyAsync(ws + y.gV, hv.data(), L * sizeof(T), cudaMemcpyHostToDevice, s) != cudaSuccess ||
               enqueue_passes<T>(rho, gam, vx, vy, L, pref, eps, RD, RV, out, ws, s) != cudaSuccess ||
               cudaStreamSynchronize(s) != cudaSuccess) {
        rc = TM_ERR_CUDA;
    }
    cudaFree(ws);
    (void)cudaGetLastError();
    return rc;
}

template <typename T>
int run_ws(const void* rho, const void* gam, const void* vx, const void* vy, int L, double pref, double eps,
           const double* gD, int RD, const double* gV, int RV, void* out, void* ws, cudaStream_t s)
{
    FkeStencils st;
    for (int d = 0; d <= TM_FKE_WS_MAX_RADIUS; ++d) {
        st.gD[d] = d <= RD ? gD[d] : 0.0;
        st.gV[d] = d <= RV ? gV[d] : 0.0;
    }
    st.RD = RD;
    st.RV = RV;
    const FkeLayout y = fke_layout(sizeof(T), L);
    unsigned char* b = (unsigned char*)ws;
    fke_wrap_kernel<T><<<(L + 255) / 256, 256, 0, s>>>(st, L, (T*)(b + y.gD), (T*)(b + y.gV));
    if (enqueue_passes<T>(rho, gam, vx, vy, L, pref, eps, RD, RV, out, b, s) != cudaSuccess) {
        (void)cudaGetLastError();
        return TM_ERR_CUDA;
    }
    return TM_OK;
}

}  // namespace

extern "C" size_t tm_fke_workspace_bytes(int precision, int L)
{
    if ((precision != TM_FP64 && precision != TM_FP32) || L < 1 || L > 46340) return 0;
    return fke_layout(precision == TM_FP64 ? 8 : 4, L).end;
}

extern "C" int tm_fke_advdiff_device_ws(const void* dev_rho, const void* dev_gamma, const void* dev_vx,
                                        const void* dev_vy, int precision, int L, double pref, double eps,
                                        const double* gD, int RD, const double* gV, int RV, void* dev_out,
                                        void* dev_workspace, size_t workspace_bytes, void* stream)
{
    if (!dev_rho || !dev_gamma || !dev_vx || !dev_vy || !dev_out || !dev_workspace || !gD || !gV || L < 1 ||
        L > 46340 || RD < 0 || RV < 0 || RD > TM_FKE_WS_MAX_RADIUS || RV > TM_FKE_WS_MAX_RADIUS ||
        ((uintptr_t)dev_workspace & 255u) != 0)
        return TM_ERR_INVALID;
    const size_t need = tm_fke_workspace_bytes(precision, L);
    if (need == 0 || workspace_bytes < need) return TM_ERR_INVALID;
    if (precision == TM_FP64)
        return run_ws<double>(dev_rho, dev_gamma, dev_vx, dev_vy, L, pref, eps, gD, RD, gV, RV, dev_out, dev_workspace,
                              (cudaStream_t)stream);
    return run_ws<float>(dev_rho, dev_gamma, dev_vx, dev_vy, L, pref, eps, gD, RD, gV, RV, dev_out, dev_workspace,
                         (cudaStream_t)stream);
}

extern "C" int tm_fke_advdiff_device(const void* dev_rho, const void* dev_gamma, const void* dev_vx,
                                     const void* dev_vy, int precision, int L, double pref, double eps,
                                     const double* gD, int RD, const double* gV, int RV, void* dev_out, void* stream)
{
    if (!dev_rho || !dev_gamma || !dev_vx || !dev_vy || !dev_out || !gD || !gV || L < 1 || L > 46340 || RD < 0 ||
        RV < 0 || RD > (1 << 20) || RV > (1 << 20))
        return TM_ERR_INVALID;
    if (precision == TM_FP64)
        return run<double>(dev_rho, dev_gamma, dev_vx, dev_vy, L, pref, eps, gD, RD, gV, RV, dev_out,
                           (cudaStream_t)stream);
    if (precision == TM_FP32)
        return run<float>(dev_rho, dev_gamma, dev_vx, dev_vy, L, pref, eps, gD, RD, gV, RV, dev_out,
                          (cudaStream_t)stream);
    return TM_ERR_INVALID;
}
