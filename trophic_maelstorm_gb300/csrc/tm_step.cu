// tm_step.cu -- the fused Dornic step for sm_103a.
//
// One warp owns a strip of 32 columns x R rows of one instance ("task") and
// walks down it with a three-row register window (north, centre, south);
// east/west neighbours come from warp shuffles, the two strip-edge columns
// from global memory.  Each lattice value is read from HBM once per step and
// written once (8 B per site-update in FP32).  Per site it fuses:
//   alpha_i  = (D/dx^2) * sum of the 4 neighbours       stochasticSPDP.cpp:1037-1038
//   skip     if alpha_i == 0 and rho_i == 0             :1049-1052
//   rho*     = Gamma(2 alpha_i/sigma^2 + Poisson(lambda e^{beta dt} rho_i)) / lambda   :1053-1059
//   remainder: rho*/(1 + b rho* dt) (:1064-1068) or RK4 of -b rho^2 - c rho^3
//            (multiSPDP.cpp:1821-1898, stochasticSPDP.cpp:1775-1805) or none
//   clamp    clamp_lo <= rho < clamp_eps -> 0           multiSPDP.cpp:3256-3259
// The same kernel with remainder "none" produces P* of the Rietkerk step
// (rietkerk_bjork_FKE.cpp:4154-4211).  Random draws come from the counter
// stream of (instance seed, site, step), so no generator state is stored.
// The task loop is persistent (grid-stride over tasks of all instances of a
// ragged batch); extinct DP instances are skipped without touching memory.
#include "tm_device.cuh"
#include "tm_kernels.cuh"

namespace tmg {

template <typename T>
__device__ __forceinline__ T rem_f(T x, T b, T c, int cubic)
{
    T f = ((-b) * x) * x;
    if (cubic) f = f - ((c * x) * x) * x;
    return f;
}

template <typename T, int REM>
__global__ void __launch_bounds__(256) dornic_step_kernel(const DornicArgs<T> A)
{
    const int lane = threadIdx.x & 31;
    const int gw = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int nw = (int)((gridDim.x * blockDim.x) >> 5);
    const long long step = (A.step_base ? *A.step_base : 0LL) + A.step_off;
    for (int t = gw; t < A.n_tasks; t += nw) {
        const int4 tk = A.tasks[t];
        const int k = tk.x;
        if (A.it.alive != nullptr && A.it.alive[k] == 0) continue;
        const int L = A.it.L[k];
        const T* __restrict__ src = A.in + A.it.off[k];
        T* __restrict__ dst = A.out + A.it.off[k];
        const Dc4 cs = A.it.consts[k];
        const T pm = (T)cs.x, inv_lambda = (T)cs.y, a1 = (T)cs.z, a2 = (T)cs.w;
        const unsigned long long seed = A.it.seed[k];
        const int x0 = tk.y, y0 = tk.z, rows = tk.w;
        const int w = min(32, L - x0);
        const int x = x0 + lane;
        const bool act = lane < w;
        const int xw = (x0 == 0) ? L - 1 : x0 - 1;
        const int xe = (x0 + w == L) ? 0 : x0 + w;
        const int yn = (y0 == 0) ? L - 1 : y0 - 1;
        T north = act ? src[(long long)yn * L + x] : T(0);
        T cur = act ? src[(long long)y0 * L + x] : T(0);
        unsigned st = 0;
        for (int r = 0; r < rows; ++r) {
            const int y = y0 + r;
            const int ys = (y == L - 1) ? 0 : y + 1;
            const T south = act ? src[(long long)ys * L + x] : T(0);
            T west = __shfl_up_sync(0xffffffffu, cur, 1);
            T east = __shfl_down_sync(0xffffffffu, cur, 1);
            if (lane == 0) west = src[(long long)y * L + xw];
            if (lane == w - 1) east = src[(long long)y * L + xe];
            if (act) {
                const T nsum = ((north + south) + west) + east;
                const T alpha = A.dcoef * nsum;
                T rs;
                if (alpha == T(0) && cur == T(0)) {
                    rs = T(0);
                } else if (A.sampler == 2) {
                    rs = a1 * cur + a2 * alpha;
                } else {
                    Stream<T> g;
                    g.init(seed, (uint32_t)(y * L + x), step);
                    rs = dornic_draw(g, pm * cur, alpha * A.two_s2, inv_lambda, A.sampler);
                    st |= g.status;
                }
                T res;
                if (REM == 0) {
                    res = rs / (T(1) + (A.b * rs) * A.dt);
                } else if (REM == 1) {
                    const T k1 = rem_f(rs, A.b, A.c, A.cubic);
                    const T k2 = rem_f(rs + A.dt2 * k1, A.b, A.c, A.cubic);
                    const T k3 = rem_f(rs + A.dt2 * k2, A.b, A.c, A.cubic);
                    const T k4 = rem_f(rs + A.dt * k3, A.b, A.c, A.cubic);
                    res = rs + A.dt6 * (((k1 + T(2) * k2) + T(2) * k3) + k4);
                } else {
                    res = rs;
                }
                if (REM != 2) {
                    if (res < A.ceps && res >= A.clo) res = T(0);
                    st |= value_status(res);
                }
                dst[(long long)y * L + x] = res;
            }
            north = cur;
            cur = south;
        }
        if (st) atomicOr(A.it.status + k, st);
    }
}

template <typename T>
cudaError_t launch_dornic(const DornicArgs<T>& a, int rem, int grid, int block, cudaStream_t s)
{
    if (a.n_tasks <= 0) return cudaSuccess;
    if (rem == 0) dornic_step_kernel<T, 0><<<grid, block, 0, s>>>(a);
    else if (rem == 1) dornic_step_kernel<T, 1><<<grid, block, 0, s>>>(a);
    else dornic_step_kernel<T, 2><<<grid, block, 0, s>>>(a);
    return cudaGetLastError();
}
template cudaError_t launch_dornic<float>(const DornicArgs<float>&, int, int, int, cudaStream_t);
template cudaError_t launch_dornic<double>(const DornicArgs<double>&, int, int, int, cudaStream_t);

// Dornic constants per instance for the step about to run (stochasticSPDP.cpp:952-954):
// beta = a - 4D/dx^2, lambda = 2 beta / (sigma^2 (e^{beta dt} - 1)); the beta == 0
// limit is lambda = 2/(sigma^2 dt).  a(s) = a0 + astep * s (a ramp when astep != 0).
__global__ void consts_kernel(const double* a0, const double* astep, int n, double diff4, double sigma2, double dt,
                              const long long* step_base, long long step_off, Dc4* out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const long long step = (step_base ? *step_base : 0LL) + step_off;
    const double a = a0[k] + astep[k] * (double)step;
    const double beta = a - diff4;
    const double e = tm_exp(beta * dt);
    double lambda, m2;
    if (beta == 0.0) {
        lambda = 2.0 / (sigma2 * dt);
        m2 = dt;
    } else {
        lambda = (2.0 * beta) / (sigma2 * (e - 1.0));
        m2 = (e - 1.0) / beta;
    }
    out[k] = Dc4{lambda * e, 1.0 / lambda, e, m2};
}

cudaError_t launch_consts(const double* a0, const double* astep, int n, double diff4, double sigma2, double dt,
                          const long long* step_base, long long step_off, Dc4* out, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    consts_kernel<<<(n + 127) / 128, 128, 0, s>>>(a0, astep, n, diff4, sigma2, dt, step_base, step_off, out);
    return cudaGetLastError();
}

__global__ void set_step_kernel(long long* d, long long v) { *d = v; }

cudaError_t launch_set_step(long long* d_step, long long v, cudaStream_t s)
{
    set_step_kernel<<<1, 1, 0, s>>>(d_step, v);
    return cudaGetLastError();
}

}  // namespace tmg
