// tm_rk4.cu -- RK4 of the Rietkerk three-field right-hand side, fused in one
// pass over a shared-memory tile, and the noise-off DP stage kernels.
//
// Rietkerk (rietkerk_bjork_FKE.cpp:2363-2444 stochastic remainder f_2Dor,
// :1760-1856 noise-off f_2D): the W and O tendencies carry 5-point
// Laplacians, so stage s needs stage s-1 values one site further out.  A CTA
// loads a (64+8) x (32+8) region of [P*, W, O] (halo 4, periodic wrap) into
// shared memory and runs all four stages there, stage s only on the region
// inset by s+1 cells, so the 64 x 32 interior comes out exact after stage 4
// with 1.15 stage evaluations per cell and stage.
// The state is read and written once per step (plus the halo re-read, which
// hits L2); the K1..K4 temporaries the reference keeps as full lattices
// never leave the SM.
#include "tm_device.cuh"
#include "tm_kernels.cuh"

namespace tmg {

// c + s * x for a power of two s: s * x is exact, so the fused form rounds once,
// as the separate multiply and add do -- the same bits in one instruction.
template <typename T>
__device__ __forceinline__ T add_pow2_times(T c, T s, T x)
{
    return Tr<T>::fma_(s, x, c);
}

// Right-hand side at region cell c of S (f_2Dor, or f_2D when DET); R per instance.
template <typename T, bool DET>
__device__ __forceinline__ void rk_rhs_cell(const RK4Args<T>& A, const T* S, int c, T R, T& fP, T& fW, T& fO)
{
    const int cn = c - RK_RX, cs = c + RK_RX, cw = c - 1, ce = c + 1;
    const T* SP = S;
    const T* SW = S + RK_RN;
    const T* SO = S + 2 * RK_RN;
    const T Pc = SP[c], Wc = SW[c], Oc = SO[c];
    const T upt_num = (A.gmax * Wc) * Pc;
    const T wk = Wc + A.k1;
    T infil, upt;
    if constexpr (sizeof(T) == 8) {
        // the reference's own expressions
        infil = ((A.alpha * (Pc + A.k2W0)) / (Pc + A.k2)) * Oc;
        fP = ((A.cgmax * Wc) * Pc) / wk;
        upt = upt_num / wk;
    } else {
        // FP32: two correctly rounded reciprocals instead of three divisions
        const T iwk = __frcp_rn(wk);
        infil = ((A.alpha * (Pc + A.k2W0)) * __frcp_rn(Pc + A.k2)) * Oc;
        fP = ((A.cgmax * Wc) * Pc) * iwk;
        upt = upt_num * iwk;
    }
    const T lapW = add_pow2_times(((SW[cn] + SW[cs]) + SW[cw]) + SW[ce], T(-4), Wc);
    const T lapO = add_pow2_times(((SO[cn] + SO[cs]) + SO[cw]) + SO[ce], T(-4), Oc);
    if (DET) {
        const T lapP = add_pow2_times(((SP[cn] + SP[cs]) + SP[cw]) + SP[ce], T(-4), Pc);
        fP = (fP - A.d * Pc) + A.DPx * lapP;
    }
    fW = ((infil - upt) - A.rW * Wc) + A.DWx * lapW;
    fO = (R - infil) + A.DOx * lapO;
}

// One CTA per tile (persistent over tiles).  Stage s (0..3) is evaluated on
// the region inset by s+1 cells -- exactly the cells whose stage-s value an
// interior cell depends on -- so the interior is exact after stage 3.  Stage
// inputs ping-pong between two shared buffers, so each stage needs one barrier
// and no value is held in registers across it.
// Tile rows by bulk copy: for a tile that does not wrap in x on a lattice with
// L % 4 == 0, each of the 3 x RK_RY halo rows is a contiguous RK_RX-float segment
// starting on a 16-byte boundary (instance offsets and field strides are
// multiples of 32 elements), so one thread issues them as cp.async.bulk copies
// completing on an mbarrier instead of 256 threads loading 5184 values.
// Every wait on the copies is bounded (RK4Args::wait_limit polls, about 0.3 s at
// the default): a CTA whose copies do not complete marks the instances of its
// current and remaining tiles with TM_STATUS_WAIT_BIT (their fields are invalid
// after this step, and the host call returns TM_ERR_TIMEOUT), waits once more,
// again bounded, for copies still in flight into its shared memory, and exits.
// Under TM_PROBE_TILE_WAIT the CTA issues no copy and arms nothing, so the
// first wait runs out with nothing in flight (the test of this path).

__device__ __forceinline__ uint32_t rk_saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool rk_bar_wait(uint32_t bar, uint32_t parity, int limit)
{
    for (int i = 0; i < limit; ++i) {
        uint32_t ok;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}\n"
                     : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
        if (ok) return true;
        if (i > 16) __nanosleep(32);
    }
    return false;
}

template <typename T, bool DET>
__global__ void __launch_bounds__(RK_THREADS, (sizeof(T) == 4 ? RK_CTAS : 1)) rk4_tile_kernel(const RK4Args<T> A)
{
    extern __shared__ __align__(16) unsigned char rk_smem[];
    __shared__ __align__(8) uint64_t tile_bar;
    __shared__ int tile_bulk;
    T* const X0 = reinterpret_cast<T*>(rk_smem);          // [3][RK_RN] stage-0 input
    T* const MA = X0 + 3 * RK_RN;                           // [3][RK_RN] stage inputs (ping)
    T* const MB = MA + 3 * RK_RN;                           // [3][RK_RN] (pong)
    constexpr int kPer = RK_TX * RK_TY / RK_THREADS;        // interior cells per thread
    static_assert(RK_TX * RK_TY % RK_THREADS == 0, "interior cells per thread");
    const int tid = threadIdx.x;
    const uint32_t bar = rk_saddr(&tile_bar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    uint32_t phase = 0;
    for (int t = blockIdx.x; t < A.n_tasks; t += gridDim.x) {
        const int4 tk = A.tasks[t];
        const int k = tk.x;
        const int L = A.it.L[k];
        const long long off = A.it.off[k];
        const long long fs = A.it.fstride[k];
        const T R = (T)A.it.R[k];
        const int x0 = tk.y, y0 = tk.z;
        const T* __restrict__ P0 = (DET ? A.in : A.pstar) + off;
        const T* __restrict__ W0 = A.in + off + fs;
        const T* __restrict__ O0 = A.in + off + 2 * fs;
        __syncthreads();  // previous tile done with shared memory
        // halo coordinates lie within RK_H of [0, L + tile), so one wrap is enough
        // once L covers the tile and its halo; smaller lattices take the modulo
        const bool one_wrap = L >= RK_RY && L >= RK_RX;
        {
            // one halo row per thread (3 x RK_RY rows): the block takes the bulk path
            // only if every row start is 16-byte aligned
            constexpr int kRows = 3 * RK_RY;
            const bool shape = (sizeof(T) == 4 && one_wrap && (L & 3) == 0 && x0 >= RK_H && x0 + RK_TX + RK_H <= L) ||
                               A.probe_no_copy;
            const T* src = nullptr;
            bool aligned = true;
            if (shape && !A.probe_no_copy && tid < kRows) {
                const int f = tid / RK_RY, ry = tid - f * RK_RY;
                int gy = y0 - RK_H + ry;
                gy = gy < 0 ? gy + L : (gy >= L ? gy - L : gy);
                src = (f == 0 ? P0 : (f == 1 ? W0 : O0)) + (long long)gy * L + (x0 - RK_H);
                aligned = ((uintptr_t)src & 15u) == 0;
            }
            const bool bulk = shape && __syncthreads_and(aligned);
            if (bulk && !A.probe_no_copy) {
                constexpr uint32_t row_bytes = RK_RX * sizeof(T);
                static_assert((RK_RX * sizeof(float)) % 16 == 0 && (RK_RN * sizeof(float)) % 16 == 0, "bulk rows");
                if (tid == 0)
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                                 :: "r"(bar), "r"((uint32_t)kRows * row_bytes) : "memory");
                __syncthreads();
                if (tid < kRows) {
                    const int f = tid / RK_RY, ry = tid - f * RK_RY;
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
                                 "[%0], [%1], %2, [%3];"
                                 :: "r"(rk_saddr(X0 + f * RK_RN + ry * RK_RX)), "l"(src), "r"(row_bytes), "r"(bar)
                                 : "memory");
                }
            }
            if (tid == 0) tile_bulk = bulk ? 1 : 0;
        }
        __syncthreads();
        if (tile_bulk) {
            const bool ok = rk_bar_wait(bar, phase, A.wait_limit);
            phase ^= 1u;
            if (__syncthreads_or(!ok)) {
                // copies did not complete: flag this tile's and every later tile's
                // instance, give copies still in flight one more bounded wait, stop
                for (int t2 = t + tid * (int)gridDim.x; t2 < A.n_tasks; t2 += RK_THREADS * (int)gridDim.x)
                    atomicOr(A.it.status + A.tasks[t2].x, TM_STATUS_WAIT_BIT);
                (void)rk_bar_wait(bar, phase ^ 1u, A.wait_limit);
                return;
            }
        } else
        for (int c = tid; c < RK_RN; c += RK_THREADS) {
            const int ry = c / RK_RX, rx = c - ry * RK_RX;
            int gy = y0 - RK_H + ry, gx = x0 - RK_H + rx;
            if (one_wrap) {
                gy = gy < 0 ? gy + L : (gy >= L ? gy - L : gy);
                gx = gx < 0 ? gx + L : (gx >= L ? gx - L : gx);
            } else {
                gy %= L; if (gy < 0) gy += L;
                gx %= L; if (gx < 0) gx += L;
            }
            const long long gi = (long long)gy * L + gx;
            X0[c] = P0[gi];
            X0[RK_RN + c] = W0[gi];
            X0[2 * RK_RN + c] = O0[gi];
        }
        __syncthreads();
        // Stage s on the region inset by s+1: the 64 x 32 interior with a fixed
        // thread mapping (kPer cells per thread, whose weighted sums of K stay in
        // registers), then the ring between the inset and the interior.
        T acc[3][kPer];
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            const T* S = (s == 0) ? X0 : ((s & 1) ? MA : MB);
            T* D = (s & 1) ? MB : MA;
            const T coef = (s == 2) ? A.dt : A.dt2;
#pragma unroll
            for (int j = 0; j < kPer; ++j) {
                const int a = tid + j * RK_THREADS;
                const int c = ((a / RK_TX) + RK_H) * RK_RX + (a % RK_TX) + RK_H;
                T k0, k1, k2;
                rk_rhs_cell<T, DET>(A, S, c, R, k0, k1, k2);
                if (s == 0) {
                    acc[0][j] = k0; acc[1][j] = k1; acc[2][j] = k2;
                } else if (s == 3) {
                    acc[0][j] = acc[0][j] + k0; acc[1][j] = acc[1][j] + k1; acc[2][j] = acc[2][j] + k2;
                } else {
                    acc[0][j] = add_pow2_times(acc[0][j], T(2), k0);
                    acc[1][j] = add_pow2_times(acc[1][j], T(2), k1);
                    acc[2][j] = add_pow2_times(acc[2][j], T(2), k2);
                }
                if (s < 3) {
                    D[c] = X0[c] + coef * k0;
                    D[RK_RN + c] = X0[RK_RN + c] + coef * k1;
                    D[2 * RK_RN + c] = X0[2 * RK_RN + c] + coef * k2;
                }
            }
            if (s < 3) {
                // ring of thickness t = 3 - s: top and bottom bands (t rows of the
                // inset's width w), then left and right bands (RK_TY rows, t columns)
                const int in = s + 1, t = 3 - s, w = RK_RX - 2 * in;
                const int nband = t * w, nside = RK_TY * t;
                for (int q = tid; q < 2 * nband + 2 * nside; q += RK_THREADS) {
                    int ry, rx;
                    if (q < 2 * nband) {
                        const int qb = q < nband ? q : q - nband;
                        ry = (q < nband ? in : RK_H + RK_TY) + qb / w;
                        rx = in + qb % w;
                    } else {
                        const int qs = q - 2 * nband;
                        const int qq = qs < nside ? qs : qs - nside;
                        ry = RK_H + qq / t;
                        rx = (qs < nside ? in : RK_H + RK_TX) + qq % t;
                    }
                    const int c = ry * RK_RX + rx;
                    T k0, k1, k2;
                    rk_rhs_cell<T, DET>(A, S, c, R, k0, k1, k2);
                    D[c] = X0[c] + coef * k0;
                    D[RK_RN + c] = X0[RK_RN + c] + coef * k1;
                    D[2 * RK_RN + c] = X0[2 * RK_RN + c] + coef * k2;
                }
            }
            __syncthreads();
        }
        unsigned st = 0;
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            const int a = tid + j * RK_THREADS;
            const int ly = a / RK_TX, lx = a % RK_TX;
            const int gy = y0 + ly, gx = x0 + lx;
            if (gy < L && gx < L) {
                const int c = (ly + RK_H) * RK_RX + lx + RK_H;
                const long long gi = off + (long long)gy * L + gx;
#pragma unroll
                for (int f = 0; f < 3; ++f) {
                    T v = X0[f * RK_RN + c] + A.dt6 * acc[f][j];
                    if (v < A.ceps && v >= A.clo) v = T(0);
                    st |= value_status(v);
                    A.out[gi + f * fs] = v;
                }
            }
        }
        if (st) atomicOr(A.it.status + k, st);
    }
}

template <typename T>
cudaError_t launch_rk4(const RK4Args<T>& a, bool det, int grid, cudaStream_t s)
{
    if (a.n_tasks <= 0) return cudaSuccess;
    const size_t smem = 9 * (size_t)RK_RN * sizeof(T);
    static bool attr[2] = {false, false};
    cudaError_t e = cudaSuccess;
    if (!attr[det ? 1 : 0]) {
        e = det ? cudaFuncSetAttribute(rk4_tile_kernel<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                : cudaFuncSetAttribute(rk4_tile_kernel<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr[det ? 1 : 0] = true;
    }
    if (det) rk4_tile_kernel<T, true><<<grid, RK_THREADS, smem, s>>>(a);
    else rk4_tile_kernel<T, false><<<grid, RK_THREADS, smem, s>>>(a);
    return cudaGetLastError();
}
template cudaError_t launch_rk4<float>(const RK4Args<float>&, bool, int, cudaStream_t);
template cudaError_t launch_rk4<double>(const RK4Args<double>&, bool, int, cudaStream_t);

// ---- noise-off DP: drho/dt = a rho - b rho^2 - c rho^3 + D Lap(rho) ---------------
// percNoDiff_2D (stochasticSPDP.cpp:549-662) with the 5-point Laplacian or the
// 4th-order cross of fP_2D (:516-529), written as f = react - D/(12 dx^2)
// (o2 - 16 o1 + 60 rho).  One CTA per 64 x 32 tile (persistent over the tiles of
// every instance), all stages in shared memory as in rk4_tile_kernel: a stencil of
// radius RAD makes stage s need stage s-1 values RAD sites further out, so the tile
// loads a halo of NST * RAD sites and evaluates stage s on the region inset by
// (s+1) RAD.  The reference keeps K1..K4 and the stage input as full lattices
// (:594-626); here they never leave the SM, and one launch per step covers the
// whole batch.
template <typename T, int RAD>
__device__ __forceinline__ T dp_det_rhs(const DetTileArgs<T>& A, const T* S, int c, int rx, T a)
{
    const T r = S[c];
    T f = (a * r) - ((A.b * r) * r);
    if (A.cubic) f = f - ((A.c * r) * r) * r;
    if constexpr (RAD == 1) {
        const T lap = add_pow2_times(((S[c - rx] + S[c + rx]) + S[c - 1]) + S[c + 1], T(-4), r);
        f = f + A.dlap * lap;
    } else {
        const T o2 = ((S[c - 2 * rx] + S[c + 2 * rx]) + S[c - 2]) + S[c + 2];
        const T o1 = ((S[c - rx] + S[c + rx]) + S[c - 1]) + S[c + 1];
        const T sm = add_pow2_times(o2, T(-16), o1) + T(60) * r;
        f = f - A.dk12 * sm;
    }
    return f;
}

template <typename T, int RAD, int NST>
__global__ void __launch_bounds__(RK_THREADS, 1) dp_det_tile_kernel(const DetTileArgs<T> A)
{
    constexpr int H = RAD * NST, RX = RK_TX + 2 * H, RY = RK_TY + 2 * H, RN = RX * RY;
    constexpr int kPer = RK_TX * RK_TY / RK_THREADS;
    extern __shared__ __align__(16) unsigned char det_smem[];
    T* const X0 = reinterpret_cast<T*>(det_smem);
    T* const MA = X0 + RN;
    T* const MB = MA + RN;
    const int tid = threadIdx.x;
    for (int t = blockIdx.x; t < A.n_tasks; t += gridDim.x) {
        const int4 tk = A.tasks[t];
        const int k = tk.x;
        const int L = A.it.L[k];
        const long long off = A.it.off[k];
        const T a = (T)A.it.R[k];
        const int x0 = tk.y, y0 = tk.z;
        const T* __restrict__ src = A.in + off;
        __syncthreads();  // previous tile done with shared memory
        const bool one_wrap = L >= RY && L >= RX;
        for (int c = tid; c < RN; c += RK_THREADS) {
            const int ry = c / RX, rx = c - ry * RX;
            int gy = y0 - H + ry, gx = x0 - H + rx;
            if (one_wrap) {
                gy = gy < 0 ? gy + L : (gy >= L ? gy - L : gy);
                gx = gx < 0 ? gx + L : (gx >= L ? gx - L : gx);
            } else {
                gy %= L; if (gy < 0) gy += L;
                gx %= L; if (gx < 0) gx += L;
            }
            X0[c] = src[(long long)gy * L + gx];
        }
        __syncthreads();
        T acc[kPer];
#pragma unroll
        for (int s = 0; s < NST; ++s) {
            const T* S = (s == 0) ? X0 : ((s & 1) ? MA : MB);
            T* D = (s & 1) ? MB : MA;
            const T coef = (s == 2) ? A.dt : A.dt2;
#pragma unroll
            for (int j = 0; j < kPer; ++j) {
                const int q = tid + j * RK_THREADS;
                const int c = ((q / RK_TX) + H) * RX + (q % RK_TX) + H;
                const T kv = dp_det_rhs<T, RAD>(A, S, c, RX, a);
                if (s == 0) acc[j] = kv;
                else if (s == NST - 1) acc[j] = acc[j] + kv;
                else acc[j] = add_pow2_times(acc[j], T(2), kv);
                if (s < NST - 1) D[c] = X0[c] + coef * kv;
            }
            if (s < NST - 1) {
                // ring between the region inset by (s+1) RAD and the interior: top and
                // bottom bands (tt rows of the inset's width w), left and right bands
                const int in = (s + 1) * RAD, tt = H - in, w = RX - 2 * in;
                const int nband = tt * w, nside = RK_TY * tt;
                for (int q = tid; q < 2 * nband + 2 * nside; q += RK_THREADS) {
                    int ry, rx;
                    if (q < 2 * nband) {
                        const int qb = q < nband ? q : q - nband;
                        ry = (q < nband ? in : H + RK_TY) + qb / w;
                        rx = in + qb % w;
                    } else {
                        const int qs = q - 2 * nband;
                        const int qq = qs < nside ? qs : qs - nside;
                        ry = H + qq / tt;
                        rx = (qs < nside ? in : H + RK_TX) + qq % tt;
                    }
                    const int c = ry * RX + rx;
                    D[c] = X0[c] + coef * dp_det_rhs<T, RAD>(A, S, c, RX, a);
                }
            }
            __syncthreads();
        }
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            const int q = tid + j * RK_THREADS;
            const int ly = q / RK_TX, lx = q % RK_TX;
            const int gy = y0 + ly, gx = x0 + lx;
            if (gy < L && gx < L) {
                const int c = (ly + H) * RX + lx + H;
                const T v = (NST == 4) ? X0[c] + A.dt6 * acc[j] : X0[c] + acc[j] * A.dt;
                A.out[off + (long long)gy * L + gx] = v;
            }
        }
    }
}

template <typename T, int RAD, int NST>
cudaError_t launch_det_t(const DetTileArgs<T>& a, int grid, cudaStream_t s)
{
    constexpr int H = RAD * NST;
    const size_t smem = 3 * (size_t)(RK_TX + 2 * H) * (RK_TY + 2 * H) * sizeof(T);
    static bool attr = false;
    if (!attr) {
        const cudaError_t e =
            cudaFuncSetAttribute(dp_det_tile_kernel<T, RAD, NST>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    dp_det_tile_kernel<T, RAD, NST><<<grid, RK_THREADS, smem, s>>>(a);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_dp_det(const DetTileArgs<T>& a, int stencil, int rk4, int grid, cudaStream_t s)
{
    if (a.n_tasks <= 0) return cudaSuccess;
    if (stencil == 5) return rk4 ? launch_det_t<T, 1, 4>(a, grid, s) : launch_det_t<T, 1, 1>(a, grid, s);
    if (stencil == 9) return rk4 ? launch_det_t<T, 2, 4>(a, grid, s) : launch_det_t<T, 2, 1>(a, grid, s);
    return cudaErrorInvalidValue;
}
template cudaError_t launch_dp_det<float>(const DetTileArgs<float>&, int, int, int, cudaStream_t);
template cudaError_t launch_dp_det<double>(const DetTileArgs<double>&, int, int, int, cudaStream_t);

}  // namespace tmg
