// tm_mlp.cu -- the sweep surrogate: a 3-128-128-128-2 GELU network with BF16
// weights, trained and evaluated on the 5th-generation tensor cores.
//
// The reference has no learned part; the network, its rounding points and its
// optimiser are specified in include/tm.h (tm_mlp_*).  One CTA owns a tile of
// 128 samples (sample t = TMEM lane t) and runs the whole forward and backward
// pass of that tile with 16 warps: warp w reads TMEM lane quarter w % 4 (the
// quarter a warp may access) and handles column slice w / 4, so a thread does
// 32 of the 128 columns of its sample and the 128-sample column sums are split
// four ways:
//   * the two 128x128 layers and the four GEMMs of their backward pass are
//     tcgen05.mma (kind::f16, BF16 x BF16 -> FP32, M = N = K = 128), issued by
//     one thread, with both operands in shared memory in the K-major
//     no-swizzle core-matrix layout and the accumulators in TMEM;
//   * the 3-wide input layer, the 2-wide output layer, GELU and its derivative
//     run on the CUDA cores between the MMAs, reading accumulators back with
//     tcgen05.ld;
//   * each CTA writes its partial gradient; a second kernel sums the partials
//     in tile order (no atomics: the result does not depend on scheduling) and
//     applies Adam to the FP32 master weights, refreshing their BF16 copies.
// Every wait on an MMA completion is bounded: on timeout the CTA records an
// error, waits once more (again bounded) for the MMAs it issued, frees its
// TMEM and returns; the update kernel then leaves the parameters unchanged.
#include "tm_kernels.cuh"
#include "../../include/tm.h"

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <new>

namespace {

constexpr int TS = 128;              // samples per tile = TMEM lanes
constexpr int NT = 512;              // threads per CTA: 4 column slices x 128 samples
constexpr int NS = NT / TS;          // column slices (32 columns each)
constexpr int OFF_W1 = 0, OFF_B1 = 384, OFF_W2 = 512, OFF_B2 = 16896, OFF_W3 = 17024, OFF_B3 = 33408,
              OFF_W4 = 33536, OFF_B4 = 33792, NP = 33794;
static_assert(NP == TM_MLP_NPARAMS, "parameter layout");
constexpr int PS = 33808;            // per-tile stride of the partial gradients (16-byte aligned rows)

// shared memory map
constexpr int BUF = 32768;           // one 128 x 128 BF16 operand tile
constexpr int SM_W1 = 6 * BUF;
constexpr int SM_B = SM_W1 + 1536;   // b1 | b2 | b3
constexpr int SM_W4 = SM_B + 1536;
constexpr int SM_B4 = SM_W4 + 1024;
constexpr int SM_X = SM_B4 + 16;
constexpr int SM_DY = SM_X + 1536;
constexpr int SM_LOSS = SM_DY + 1024;
constexpr int SM_RED = SM_LOSS + 512;       // [NS][128][3] FP32 partial sums
constexpr int SM_BAR = SM_RED + NS * TS * 3 * 4;
constexpr int SM_TMEM = SM_BAR + 8;
constexpr int SM_TOTAL = SM_TMEM + 8;
constexpr int FPAD = 129;            // row stride (floats) of the FP32 column-sum scratch over buffers 0-2
static_assert(TS * FPAD * 4 <= 3 * BUF, "scratch fits buffers 0-2");
static_assert(SM_BAR % 8 == 0, "mbarrier alignment");

constexpr int kWaitLimit = 1 << 22;  // polls of an MMA completion before the CTA gives up (~0.3 s)
constexpr int kProbeWaitLimit = 1 << 16;  // the same under TM_PROBE_MLP_WAIT (nothing in flight)

// byte offset of element (row r, k) of a 128-row operand in the K-major,
// no-swizzle canonical layout: 8 x 16-byte core matrices, 128 B apart along K
// (leading byte offset) and 2048 B apart along the rows (stride byte offset)
__device__ __forceinline__ uint32_t cm(int r, int k)
{
    return (uint32_t)((r >> 3) * 2048 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start >> 4, LBO = 128 B, SBO = 2048 B,
// fixed 0b001 at bits 46-48, no swizzle
__device__ __forceinline__ uint64_t desc_kmajor(uint32_t a)
{
    return (uint64_t)((a & 0x3FFFFu) >> 4) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(2048 >> 4) << 32) |
           (1ull << 46);
}

// instruction descriptor, kind::f16: D FP32 (bits 4-5 = 1), A and B BF16 (bits 7-9, 10-12 = 1),
// both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(128 >> 3) << 17) |
                            ((uint32_t)(128 >> 4) << 24);

// D[128 x 128] (TMEM columns d..d+127) = A[128 x 128] * B[128 x 128]^T, both K-major in shared memory
__device__ __forceinline__ void mma_128(uint32_t d, uint32_t a, uint32_t b)
{
#pragma unroll
    for (int kk = 0; kk < 8; ++kk) {
        const uint64_t da = desc_kmajor(a + kk * 256), db = desc_kmajor(b + kk * 256);
        const uint32_t acc = kk > 0 ? 1u : 0u;
        asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                     "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
                     :: "r"(d), "l"(da), "l"(db), "r"(kIdesc), "r"(acc));
    }
}

__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(bar)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity, int limit)
{
    for (int i = 0; i < limit; ++i) {
        uint32_t ok;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}\n"
                     : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
        if (ok) return true;
        if (i > 32) __nanosleep(64);
    }
    return false;
}

// 32 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v)
{
    uint32_t r[32];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                 "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                   "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                   "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

constexpr float kGeluC = 0.7978845608028654f;   // sqrt(2/pi)
constexpr float kGeluK = 0.044715f;

__device__ __forceinline__ float gelu(float a)
{
    const float th = tanhf(kGeluC * (a + kGeluK * (a * a * a)));
    return 0.5f * a * (1.0f + th);
}

__device__ __forceinline__ float gelu_grad(float a)
{
    const float th = tanhf(kGeluC * (a + kGeluK * (a * a * a)));
    return 0.5f * (1.0f + th) + 0.5f * a * (1.0f - th * th) * kGeluC * (1.0f + 3.0f * kGeluK * (a * a));
}

// 128 x 128 BF16 row-major matrix (global) -> K-major core-matrix tile (shared)
__device__ __forceinline__ void load_tile(unsigned char* dst, const __nv_bfloat16* src)
{
    const uint4* s = reinterpret_cast<const uint4*>(src);
    for (int c = threadIdx.x; c < 2048; c += NT) *reinterpret_cast<uint4*>(dst + cm(c >> 4, (c & 15) * 8)) = s[c];
}

// sum over k in [32 p, 32 p + 32) of row r of a K-major BF16 tile, k ascending
__device__ __forceinline__ float row_sum_part(const unsigned char* buf, int r, int p)
{
    float s = 0.0f;
    for (int g = 4 * p; g < 4 * p + 4; ++g) {
        const uint4 q = *reinterpret_cast<const uint4*>(buf + cm(r, g * 8));
        const __nv_bfloat16* h = reinterpret_cast<const __nv_bfloat16*>(&q);
#pragma unroll
        for (int i = 0; i < 8; ++i) s = s + __bfloat162float(h[i]);
    }
    return s;
}

__device__ __forceinline__ void store8(unsigned char* buf, int r, int k0, const __nv_bfloat16* h)
{
    *reinterpret_cast<uint4*>(buf + cm(r, k0)) = *reinterpret_cast<const uint4*>(h);
}

__device__ __forceinline__ void store1(unsigned char* buf, int r, int k, __nv_bfloat16 h)
{
    *reinterpret_cast<__nv_bfloat16*>(buf + cm(r, k)) = h;
}

struct MlpArgs {
    const float* x;                  // n x 3 features
    const float* y;                  // n x 2 targets (training)
    const float* w;                  // n x 2 loss weights (training)
    int n;
    float inv_norm;
    const float* p;                  // FP32 master parameters
    const __nv_bfloat16 *W2, *W2T, *W3, *W3T;   // BF16 copies, [out][in] and transposed
    float* grad_part;                // [tiles][PS] partial gradients (training)
    float* loss_part;                // [tiles] partial losses (training)
    float* y_out;                    // n x 2 outputs (inference)
    int* err;                        // set to 1 when an MMA wait ran out
    int wait_limit;                  // polls of one MMA completion
    int probe_no_mma;                // TM_PROBE_MLP_WAIT: the first GEMM is not issued, so its wait runs out
};

template <bool TRAIN>
__global__ void __launch_bounds__(NT, 1) mlp_tile_kernel(MlpArgs a)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char* B0 = sm;
    unsigned char* B1 = sm + BUF;
    unsigned char* B2 = sm + 2 * BUF;
    unsigned char* B3 = sm + 3 * BUF;
    unsigned char* B4 = sm + 4 * BUF;
    unsigned char* B5 = sm + 5 * BUF;
    float* F = reinterpret_cast<float*>(sm);           // FP32 scratch [128][FPAD] over B0..B2
    float* W1s = reinterpret_cast<float*>(sm + SM_W1);
    float* bs = reinterpret_cast<float*>(sm + SM_B);
    float* W4s = reinterpret_cast<float*>(sm + SM_W4);
    float* b4s = reinterpret_cast<float*>(sm + SM_B4);
    float* xs = reinterpret_cast<float*>(sm + SM_X);
    float* dys = reinterpret_cast<float*>(sm + SM_DY);
    float* ls = reinterpret_cast<float*>(sm + SM_LOSS);
    float* red = reinterpret_cast<float*>(sm + SM_RED);    // [NS][TS][3]
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + SM_BAR);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + SM_TMEM);

    const int tid = threadIdx.x, warp = tid >> 5;
    const int q = warp & 3, cs = warp >> 2;            // TMEM lane quarter, column slice
    const int t = q * 32 + (tid & 31);                 // this thread's sample (= TMEM lane)
    const int c0 = cs * 32;                            // first column of this thread's slice
    const int tile = blockIdx.x;
    const long long s = (long long)tile * TS + t;
    const bool valid = s < a.n;
    const uint32_t bar_a = saddr(bar);

    for (int i = tid; i < 384; i += NT) W1s[i] = bf16r(a.p[OFF_W1 + i]);
    for (int i = tid; i < 128; i += NT) {
        bs[i] = a.p[OFF_B1 + i];
        bs[128 + i] = a.p[OFF_B2 + i];
        bs[256 + i] = a.p[OFF_B3 + i];
    }
    for (int i = tid; i < 256; i += NT) W4s[i] = bf16r(a.p[OFF_W4 + i]);
    if (tid < 2) b4s[tid] = a.p[OFF_B4 + tid];
    float x0 = 0.0f, x1 = 0.0f, x2 = 0.0f;
    if (valid) {
        x0 = a.x[3 * s];
        x1 = a.x[3 * s + 1];
        x2 = a.x[3 * s + 2];
    }
    if (cs == 0) {
        xs[3 * t] = x0;
        xs[3 * t + 1] = x1;
        xs[3 * t + 2] = x2;
    }
    load_tile(B0, a.W2);
    load_tile(B1, a.W3);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(bar_a) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" :: "r"(saddr(tslot))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    const uint32_t lane = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0;   // this warp's lanes and slice
    float* gp = TRAIN ? a.grad_part + (size_t)tile * PS : nullptr;
    uint32_t phase = 0;
    bool failed = false;
    __align__(16) __nv_bfloat16 hb[8];
    float v[32];

    do {
        // ---- layer 1 (CUDA cores): h1 = bf16(gelu(W1 x + b1)) -> B2 (A operand); h1^T -> B3
#pragma unroll
        for (int g = 0; g < 4; ++g) {
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const int j = c0 + g * 8 + i;
                const float z = ((W1s[3 * j] * x0 + W1s[3 * j + 1] * x1) + W1s[3 * j + 2] * x2) + bs[j];
                hb[i] = __float2bfloat16_rn(gelu(z));
                if (TRAIN) store1(B3, j, t, hb[i]);
            }
            store8(B2, t, c0 + g * 8, hb);
        }
        fence_async_smem();
        __syncthreads();
        if (tid == 0 && !a.probe_no_mma) {
            tc_fence_after();
            mma_128(tmem + 0, saddr(B2), saddr(B0));          // a2 - b2 -> TMEM cols 0..127
            mma_commit(bar_a);
        }
        failed = __syncthreads_or(!bar_wait(bar_a, phase, a.wait_limit));
        phase ^= 1;
        if (failed) break;
        tc_fence_after();

        // ---- layer 2 epilogue: h2 = bf16(gelu(a2)) -> B2 (A operand); h2^T -> B4
        tmem_ld32(lane + 0, v);
#pragma unroll
        for (int g = 0; g < 4; ++g) {
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const int j = c0 + g * 8 + i;
                hb[i] = __float2bfloat16_rn(gelu(v[g * 8 + i] + bs[128 + j]));
                if (TRAIN) store1(B4, j, t, hb[i]);
            }
            store8(B2, t, c0 + g * 8, hb);
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            mma_128(tmem + 128, saddr(B2), saddr(B1));        // a3 - b3 -> TMEM cols 128..255
            mma_commit(bar_a);
        }
        failed = __syncthreads_or(!bar_wait(bar_a, phase, a.wait_limit));
        phase ^= 1;
        if (failed) break;
        tc_fence_after();

        // ---- layer 3 epilogue and output layer: y = W4 gelu(a3) + b4, slice partials summed in
        //      slice order (h3 kept FP32 in F for dW4)
        {
            float y0 = 0.0f, y1 = 0.0f;
            tmem_ld32(lane + 128, v);
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                const int j = c0 + i;
                const float h = gelu(v[i] + bs[256 + j]);
                y0 = y0 + W4s[j] * h;
                y1 = y1 + W4s[128 + j] * h;
                if (TRAIN) F[j * FPAD + t] = h;
            }
            red[(cs * TS + t) * 3] = y0;
            red[(cs * TS + t) * 3 + 1] = y1;
        }
        __syncthreads();
        float dy0 = 0.0f, dy1 = 0.0f;
        if (cs == 0) {
            float y0 = 0.0f, y1 = 0.0f;
            for (int p = 0; p < NS; ++p) {
                y0 = y0 + red[(p * TS + t) * 3];
                y1 = y1 + red[(p * TS + t) * 3 + 1];
            }
            y0 = y0 + b4s[0];
            y1 = y1 + b4s[1];
            if (!TRAIN) {
                if (valid) {
                    a.y_out[2 * s] = y0;
                    a.y_out[2 * s + 1] = y1;
                }
            } else {
                // loss and output-layer gradient of this sample
                float e0 = 0.0f, e1 = 0.0f, w0 = 0.0f, w1 = 0.0f;
                if (valid) {
                    e0 = y0 - a.y[2 * s];
                    e1 = y1 - a.y[2 * s + 1];
                    w0 = a.w[2 * s];
                    w1 = a.w[2 * s + 1];
                }
                ls[t] = w0 * e0 * e0 + w1 * e1 * e1;
                dys[2 * t] = ((2.0f * w0) * e0) * a.inv_norm;
                dys[2 * t + 1] = ((2.0f * w1) * e1) * a.inv_norm;
            }
        }
        if (!TRAIN) break;
        __syncthreads();
        dy0 = dys[2 * t];
        dy1 = dys[2 * t + 1];
        {
            // gW4[o][j] = sum_u dy_o[u] h3[u][j]: thread (j = tid & 127, part p = tid >> 7) sums 32 samples
            const int j = tid & 127, p = tid >> 7;
            float g0 = 0.0f, g1 = 0.0f;
            for (int u = 32 * p; u < 32 * p + 32; ++u) {
                const float h = F[j * FPAD + u];
                g0 = g0 + dys[2 * u] * h;
                g1 = g1 + dys[2 * u + 1] * h;
            }
            red[(p * TS + j) * 3] = g0;
            red[(p * TS + j) * 3 + 1] = g1;
        }
        __syncthreads();
        if (tid < 128) {
            float g0 = 0.0f, g1 = 0.0f;
            for (int p = 0; p < NS; ++p) {
                g0 = g0 + red[(p * TS + tid) * 3];
                g1 = g1 + red[(p * TS + tid) * 3 + 1];
            }
            gp[OFF_W4 + tid] = g0;
            gp[OFF_W4 + 128 + tid] = g1;
        }
        if (tid == 0) {
            float s0 = 0.0f, s1 = 0.0f, sl = 0.0f;
            for (int u = 0; u < TS; ++u) {
                s0 = s0 + dys[2 * u];
                s1 = s1 + dys[2 * u + 1];
                sl = sl + ls[u];
            }
            gp[OFF_B4] = s0;
            gp[OFF_B4 + 1] = s1;
            a.loss_part[tile] = sl * a.inv_norm;
        }
        __syncthreads();                                      // F (B0..B2) and red free again

        // ---- dz3 = bf16((dy W4) * gelu'(a3)) -> B2 (A operand of dH2); dz3^T -> B5 (A operand of dW3)
        load_tile(B1, a.W3T);
        tmem_ld32(lane + 128, v);
#pragma unroll
        for (int g = 0; g < 4; ++g) {
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const int j = c0 + g * 8 + i;
                const float dh = dy0 * W4s[j] + dy1 * W4s[128 + j];
                hb[i] = __float2bfloat16_rn(dh * gelu_grad(v[g * 8 + i] + bs[256 + j]));
                store1(B5, j, t, hb[i]);
            }
            store8(B2, t, c0 + g * 8, hb);
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            mma_128(tmem + 256, saddr(B2), saddr(B1));        // dH2 = dz3 W3      -> cols 256..383
            mma_128(tmem + 384, saddr(B5), saddr(B4));        // gW3 = dz3^T h2    -> cols 384..511
            mma_commit(bar_a);
        }
        red[(cs * TS + t) * 3 + 2] = row_sum_part(B5, t, cs);   // gb3 partial: row t of dz3^T, samples 32 cs..
        failed = __syncthreads_or(!bar_wait(bar_a, phase, a.wait_limit));
        phase ^= 1;
        if (failed) break;
        tc_fence_after();
        if (tid < 128) {
            float sb = 0.0f;
            for (int p = 0; p < NS; ++p) sb = sb + red[(p * TS + tid) * 3 + 2];
            gp[OFF_B3 + tid] = sb;
        }

        // ---- gW3 rows; dz2 = bf16(dH2 * gelu'(a2)) -> B2; dz2^T -> B5
        load_tile(B0, a.W2T);
        tmem_ld32(lane + 384, v);
        {
            float4* dst = reinterpret_cast<float4*>(gp + OFF_W3 + t * 128 + c0);
#pragma unroll
            for (int i = 0; i < 8; ++i) dst[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
        }
        {
            float z[32];
            tmem_ld32(lane + 256, v);
            tmem_ld32(lane + 0, z);
    #pragma unroll
        for (int g = 0; g < 4; ++g) {
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const int j = c0 + g * 8 + i;
                    hb[i] = __float2bfloat16_rn(v[g * 8 + i] * gelu_grad(z[g * 8 + i] + bs[128 + j]));
                    store1(B5, j, t, hb[i]);
                }
                store8(B2, t, c0 + g * 8, hb);
            }
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();                                      // also: every gb3 read of red is done
        if (tid == 0) {
            tc_fence_after();
            mma_128(tmem + 128, saddr(B2), saddr(B0));        // dH1 = dz2 W2      -> cols 128..255
            mma_128(tmem + 0, saddr(B5), saddr(B3));          // gW2 = dz2^T h1    -> cols 0..127
            mma_commit(bar_a);
        }
        red[(cs * TS + t) * 3 + 2] = row_sum_part(B5, t, cs);   // gb2 partial
        failed = __syncthreads_or(!bar_wait(bar_a, phase, a.wait_limit));
        phase ^= 1;
        if (failed) break;
        tc_fence_after();
        if (tid < 128) {
            float sb = 0.0f;
            for (int p = 0; p < NS; ++p) sb = sb + red[(p * TS + tid) * 3 + 2];
            gp[OFF_B2 + tid] = sb;
        }

        // ---- gW2 rows; dz1 = dH1 * gelu'(z1) (FP32) -> F; gW1, gb1 by column sums
        tmem_ld32(lane + 0, v);
        {
            float4* dst = reinterpret_cast<float4*>(gp + OFF_W2 + t * 128 + c0);
#pragma unroll
            for (int i = 0; i < 8; ++i) dst[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
        }
        tmem_ld32(lane + 128, v);
#pragma unroll
        for (int i = 0; i < 32; ++i) {
            const int j = c0 + i;
            const float z = ((W1s[3 * j] * x0 + W1s[3 * j + 1] * x1) + W1s[3 * j + 2] * x2) + bs[j];
            F[j * FPAD + t] = v[i] * gelu_grad(z);
        }
        __syncthreads();                                      // F complete; every gb2 read of red is done
        {
            const int j = tid & 127, p = tid >> 7;
            float g0 = 0.0f, g1 = 0.0f, g2 = 0.0f;
            for (int u = 32 * p; u < 32 * p + 32; ++u) {
                const float d = F[j * FPAD + u];
                g0 = g0 + d * xs[3 * u];
                g1 = g1 + d * xs[3 * u + 1];
                g2 = g2 + d * xs[3 * u + 2];
            }
            red[(p * TS + j) * 3] = g0;
            red[(p * TS + j) * 3 + 1] = g1;
            red[(p * TS + j) * 3 + 2] = g2;
        }
        __syncthreads();
        if (tid < 128) {
            float g0 = 0.0f, g1 = 0.0f, g2 = 0.0f, gb = 0.0f;
            for (int p = 0; p < NS; ++p) {
                g0 = g0 + red[(p * TS + tid) * 3];
                g1 = g1 + red[(p * TS + tid) * 3 + 1];
                g2 = g2 + red[(p * TS + tid) * 3 + 2];
            }
            for (int u = 0; u < TS; ++u) gb = gb + F[tid * FPAD + u];
            gp[OFF_W1 + 3 * tid] = g0;
            gp[OFF_W1 + 3 * tid + 1] = g1;
            gp[OFF_W1 + 3 * tid + 2] = g2;
            gp[OFF_B1 + tid] = gb;
        }
    } while (false);

    if (failed) {
        // the wait on the phase just toggled past ran out: give the MMAs issued
        // for it one more bounded wait before their TMEM is freed
        if (tid == 0) atomicExch(a.err, 1);
        (void)bar_wait(bar_a, phase ^ 1u, a.wait_limit);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" :: "r"(tmem) : "memory");
}

// Sum the partial gradients in tile order, optionally apply Adam, and refresh
// the BF16 copies of W2 and W3 (row-major and transposed).
struct AdamArgs {
    const float* part;
    int n_tiles;
    const float* loss_part;
    double* loss_out;                // sum of the partial losses (may be null)
    float* p;
    float* m;
    float* v;
    float* grad_out;                 // summed gradient (may be null)
    int update;
    float lr, b1, b2, eps, c1, c2;
    __nv_bfloat16 *W2, *W2T, *W3, *W3T;
    const int* err;                  // a tile kernel's wait ran out: the partials are invalid, change nothing
};

__global__ void mlp_adam_kernel(AdamArgs a)
{
    if (a.err != nullptr && *a.err != 0) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NP; i += gridDim.x * blockDim.x) {
        float pv = a.p[i];
        if (a.n_tiles > 0) {
            float g = 0.0f;
            for (int k = 0; k < a.n_tiles; ++k) g = g + a.part[(size_t)k * PS + i];
            if (a.grad_out) a.grad_out[i] = g;
            if (a.update) {
                const float mv = a.b1 * a.m[i] + (1.0f - a.b1) * g;
                const float vv = a.b2 * a.v[i] + (1.0f - a.b2) * (g * g);
                pv = pv - a.lr * (mv * a.c1) / (sqrtf(vv * a.c2) + a.eps);
                a.m[i] = mv;
                a.v[i] = vv;
                a.p[i] = pv;
            }
        }
        if (i >= OFF_W2 && i < OFF_W2 + 16384) {
            const int r = (i - OFF_W2) >> 7, c = (i - OFF_W2) & 127;
            const __nv_bfloat16 h = __float2bfloat16_rn(pv);
            a.W2[r * 128 + c] = h;
            a.W2T[c * 128 + r] = h;
        } else if (i >= OFF_W3 && i < OFF_W3 + 16384) {
            const int r = (i - OFF_W3) >> 7, c = (i - OFF_W3) & 127;
            const __nv_bfloat16 h = __float2bfloat16_rn(pv);
            a.W3[r * 128 + c] = h;
            a.W3T[c * 128 + r] = h;
        }
    }
    if (a.loss_out && blockIdx.x == 0 && threadIdx.x == 0) {
        double sl = 0.0;
        for (int k = 0; k < a.n_tiles; ++k) sl += (double)a.loss_part[k];
        *a.loss_out = sl;
    }
}

template <typename P>
cudaError_t dalloc(P** p, size_t n)
{
    *p = nullptr;
    return cudaMalloc(reinterpret_cast<void**>(p), n * sizeof(P));
}

}  // namespace

struct tm_mlp {
    tm_ctx* ctx = nullptr;
    float *p = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr;
    __nv_bfloat16 *W2 = nullptr, *W2T = nullptr, *W3 = nullptr, *W3T = nullptr;
    float *x = nullptr, *y = nullptr, *w = nullptr;   // training set
    int n = 0;
    float* part = nullptr;                             // [tiles][PS]
    float* loss_part = nullptr;
    int tiles_cap = 0;
    double* loss_dev = nullptr;
    int loss_cap = 0;
    float *px = nullptr, *py = nullptr;                // prediction buffers
    int pcap = 0;
    int* err = nullptr;
    long long step = 0;
};

namespace {

#define MLP_CUDA(call)                     \
    do {                                   \
        cudaError_t e__ = (call);          \
        if (e__ != cudaSuccess) {          \
            (void)cudaGetLastError();      \
            return TM_ERR_CUDA;            \
        }                                  \
    } while (0)

int grow_tiles(tm_mlp* m, int tiles)
{
    if (tiles <= m->tiles_cap) return TM_OK;
    cudaFree(m->part);
    cudaFree(m->loss_part);
    m->part = nullptr;
    m->loss_part = nullptr;
    m->tiles_cap = 0;
    if (dalloc(&m->part, (size_t)tiles * PS) != cudaSuccess || dalloc(&m->loss_part, (size_t)tiles) != cudaSuccess) {
        (void)cudaGetLastError();
        return TM_ERR_NOMEM;
    }
    m->tiles_cap = tiles;
    return TM_OK;
}

cudaError_t set_smem_attr()
{
    cudaError_t e = cudaFuncSetAttribute(mlp_tile_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, SM_TOTAL);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(mlp_tile_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, SM_TOTAL);
}

AdamArgs adam_args(tm_mlp* m, int n_tiles, double* loss_out, float* grad_out, int update, float lr, float b1,
                   float b2, float eps, float c1, float c2)
{
    AdamArgs a;
    a.part = m->part;
    a.n_tiles = n_tiles;
    a.loss_part = m->loss_part;
    a.loss_out = loss_out;
    a.p = m->p;
    a.m = m->m;
    a.v = m->v;
    a.grad_out = grad_out;
    a.update = update;
    a.lr = lr;
    a.b1 = b1;
    a.b2 = b2;
    a.eps = eps;
    a.c1 = c1;
    a.c2 = c2;
    a.W2 = m->W2;
    a.W2T = m->W2T;
    a.W3 = m->W3;
    a.W3T = m->W3T;
    a.err = m->err;
    return a;
}

MlpArgs tile_args(tm_mlp* m, const float* x, int n, float inv_norm, float* y_out)
{
    MlpArgs a;
    a.x = x;
    a.y = m->y;
    a.w = m->w;
    a.n = n;
    a.inv_norm = inv_norm;
    a.p = m->p;
    a.W2 = m->W2;
    a.W2T = m->W2T;
    a.W3 = m->W3;
    a.W3T = m->W3T;
    a.grad_part = m->part;
    a.loss_part = m->loss_part;
    a.y_out = y_out;
    a.err = m->err;
    a.probe_no_mma = (m->ctx->probe & TM_PROBE_MLP_WAIT) ? 1 : 0;
    a.wait_limit = a.probe_no_mma ? kProbeWaitLimit : kWaitLimit;
    return a;
}

int finish(tm_mlp* m)
{
    int herr = 0;
    MLP_CUDA(cudaGetLastError());
    MLP_CUDA(cudaMemcpyAsync(&herr, m->err, sizeof(int), cudaMemcpyDeviceToHost, m->ctx->stream));
    MLP_CUDA(cudaStreamSynchronize(m->ctx->stream));
    if (herr) {
        (void)cudaMemsetAsync(m->err, 0, sizeof(int), m->ctx->stream);
        (void)cudaStreamSynchronize(m->ctx->stream);
        return TM_ERR_TIMEOUT;
    }
    return TM_OK;
}

int upload_params(tm_mlp* m, const float* params)
{
    cudaStream_t s = m->ctx->stream;
    MLP_CUDA(cudaMemcpyAsync(m->p, params, NP * sizeof(float), cudaMemcpyHostToDevice, s));
    MLP_CUDA(cudaMemsetAsync(m->m, 0, NP * sizeof(float), s));
    MLP_CUDA(cudaMemsetAsync(m->v, 0, NP * sizeof(float), s));
    AdamArgs a = adam_args(m, 0, nullptr, nullptr, 0, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f);
    mlp_adam_kernel<<<(NP + 255) / 256, 256, 0, s>>>(a);
    m->step = 0;
    return finish(m);
}

}  // namespace

extern "C" {

int tm_mlp_create(tm_ctx* ctx, const float* params, tm_mlp** out)
{
    if (!ctx || !params || !out) return TM_ERR_INVALID;
    *out = nullptr;
    tm_mlp* m = new (std::nothrow) tm_mlp();
    if (!m) return TM_ERR_NOMEM;
    m->ctx = ctx;
    if (cudaSetDevice(ctx->device) != cudaSuccess || set_smem_attr() != cudaSuccess) {
        (void)cudaGetLastError();
        delete m;
        return TM_ERR_CUDA;
    }
    if (dalloc(&m->p, NP) != cudaSuccess || dalloc(&m->m, NP) != cudaSuccess || dalloc(&m->v, NP) != cudaSuccess ||
        dalloc(&m->grad, NP) != cudaSuccess || dalloc(&m->W2, 16384) != cudaSuccess ||
        dalloc(&m->W2T, 16384) != cudaSuccess || dalloc(&m->W3, 16384) != cudaSuccess ||
        dalloc(&m->W3T, 16384) != cudaSuccess || dalloc(&m->err, 1) != cudaSuccess ||
        cudaMemset(m->err, 0, sizeof(int)) != cudaSuccess) {
        (void)cudaGetLastError();
        tm_mlp_destroy(m);
        return TM_ERR_NOMEM;
    }
    const int rc = upload_params(m, params);
    if (rc != TM_OK) {
        tm_mlp_destroy(m);
        return rc;
    }
    *out = m;
    return TM_OK;
}

int tm_mlp_destroy(tm_mlp* m)
{
    if (!m) return TM_ERR_INVALID;
    if (m->ctx) cudaSetDevice(m->ctx->device);
    void* ptrs[] = {m->p, m->m, m->v, m->grad, m->W2, m->W2T, m->W3, m->W3T, m->x, m->y, m->w,
                    m->part, m->loss_part, m->loss_dev, m->px, m->py, m->err};
    for (void* q : ptrs) cudaFree(q);
    (void)cudaGetLastError();
    delete m;
    return TM_OK;
}

int tm_mlp_set_params(tm_mlp* m, const float* params)
{
    if (!m || !params) return TM_ERR_INVALID;
    MLP_CUDA(cudaSetDevice(m->ctx->device));
    return upload_params(m, params);
}

int tm_mlp_get_params(tm_mlp* m, float* params)
{
    if (!m || !params) return TM_ERR_INVALID;
    MLP_CUDA(cudaSetDevice(m->ctx->device));
    MLP_CUDA(cudaMemcpyAsync(params, m->p, NP * sizeof(float), cudaMemcpyDeviceToHost, m->ctx->stream));
    MLP_CUDA(cudaStreamSynchronize(m->ctx->stream));
    return TM_OK;
}

int tm_mlp_set_data(tm_mlp* m, const float* x, const float* y, const float* w, int n)
{
    if (!m || !x || !y || !w || n < 1) return TM_ERR_INVALID;
    MLP_CUDA(cudaSetDevice(m->ctx->device));
    if (n > m->n) {
        cudaFree(m->x);
        cudaFree(m->y);
        cudaFree(m->w);
        m->x = m->y = m->w = nullptr;
        m->n = 0;
        if (dalloc(&m->x, (size_t)n * 3) != cudaSuccess || dalloc(&m->y, (size_t)n * 2) != cudaSuccess ||
            dalloc(&m->w, (size_t)n * 2) != cudaSuccess) {
            (void)cudaGetLastError();
            return TM_ERR_NOMEM;
        }
    }
    const int rc = grow_tiles(m, (n + TS - 1) / TS);
    if (rc != TM_OK) return rc;
    cudaStream_t s = m->ctx->stream;
    MLP_CUDA(cudaMemcpyAsync(m->x, x, (size_t)n * 3 * sizeof(float), cudaMemcpyHostToDevice, s));
    MLP_CUDA(cudaMemcpyAsync(m->y, y, (size_t)n * 2 * sizeof(float), cudaMemcpyHostToDevice, s));
    MLP_CUDA(cudaMemcpyAsync(m->w, w, (size_t)n * 2 * sizeof(float), cudaMemcpyHostToDevice, s));
    MLP_CUDA(cudaStreamSynchronize(s));
    m->n = n;
    return TM_OK;
}

int tm_mlp_loss_grad(tm_mlp* m, float inv_norm, double* loss, float* grad)
{
    if (!m || m->n < 1) return !m ? TM_ERR_INVALID : TM_ERR_STATE;
    MLP_CUDA(cudaSetDevice(m->ctx->device));
    if (m->loss_cap < 1) {
        if (dalloc(&m->loss_dev, 64) != cudaSuccess) return TM_ERR_NOMEM;
        m->loss_cap = 64;
    }
    cudaStream_t s = m->ctx->stream;
    const int tiles = (m->n + TS - 1) / TS;
    mlp_tile_kernel<true><<<tiles, NT, SM_TOTAL, s>>>(tile_args(m, m->x, m->n, inv_norm, nullptr));
    AdamArgs a = adam_args(m, tiles, m->loss_dev, m->grad, 0, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f);
    mlp_adam_kernel<<<(NP + 255) / 256, 256, 0, s>>>(a);
    const int rc = finish(m);
    if (rc != TM_OK) return rc;
    if (grad) MLP_CUDA(cudaMemcpy(grad, m->grad, NP * sizeof(float), cudaMemcpyDeviceToHost));
    if (loss) MLP_CUDA(cudaMemcpy(loss, m->loss_dev, sizeof(double), cudaMemcpyDeviceToHost));
    return TM_OK;
}

int tm_mlp_train(tm_mlp* m, int steps, float lr, float beta1, float beta2, float eps, float inv_norm,
                 double* loss_hist)
{
    if (!m || steps < 0 || !(lr >= 0.f) || !(beta1 >= 0.f && beta1 < 1.f) || !(beta2 >= 0.f && beta2 < 1.f))
        return TM_ERR_INVALID;
    if (m->n < 1) return TM_ERR_STATE;
    MLP_CUDA(cudaSetDevice(m->ctx->device));
    if (steps > m->loss_cap) {
        cudaFree(m->loss_dev);
        m->loss_dev = nullptr;
        m->loss_cap = 0;
        if (dalloc(&m->loss_dev, (size_t)steps) != cudaSuccess) return TM_ERR_NOMEM;
        m->loss_cap = steps;
    }
    cudaStream_t s = m->ctx->stream;
    const int tiles = (m->n + TS - 1) / TS;
    for (int k = 0; k < steps; ++k) {
        const long long st = m->step + 1 + k;
        const float c1 = (float)(1.0 / (1.0 - std::pow((double)beta1, (double)st)));
        const float c2 = (float)(1.0 / (1.0 - std::pow((double)beta2, (double)st)));
        mlp_tile_kernel<true><<<tiles, NT, SM_TOTAL, s>>>(tile_args(m, m->x, m->n, inv_norm, nullptr));
        AdamArgs a = adam_args(m, tiles, m->loss_dev + k, nullptr, 1, lr, beta1, beta2, eps, c1, c2);
        mlp_adam_kernel<<<(NP + 255) / 256, 256, 0, s>>>(a);
    }
    const int rc = finish(m);
    if (rc != TM_OK) return rc;
    m->step += steps;
    if (loss_hist && steps > 0)
        MLP_CUDA(cudaMemcpy(loss_hist, m->loss_dev, (size_t)steps * sizeof(double), cudaMemcpyDeviceToHost));
    return TM_OK;
}

int tm_mlp_predict(tm_mlp* m, const float* x, int n, float* y)
{
    if (!m || !x || !y || n < 0) return TM_ERR_INVALID;
    if (n == 0) return TM_OK;
    MLP_CUDA(cudaSetDevice(m->ctx->device));
    if (n > m->pcap) {
        cudaFree(m->px);
        cudaFree(m->py);
        m->px = m->py = nullptr;
        m->pcap = 0;
        if (dalloc(&m->px, (size_t)n * 3) != cudaSuccess || dalloc(&m->py, (size_t)n * 2) != cudaSuccess) {
            (void)cudaGetLastError();
            return TM_ERR_NOMEM;
        }
        m->pcap = n;
    }
    cudaStream_t s = m->ctx->stream;
    MLP_CUDA(cudaMemcpyAsync(m->px, x, (size_t)n * 3 * sizeof(float), cudaMemcpyHostToDevice, s));
    mlp_tile_kernel<false><<<(n + TS - 1) / TS, NT, SM_TOTAL, s>>>(tile_args(m, m->px, n, 0.f, m->py));
    const int rc = finish(m);
    if (rc != TM_OK) return rc;
    MLP_CUDA(cudaMemcpy(y, m->py, (size_t)n * 2 * sizeof(float), cudaMemcpyDeviceToHost));
    return TM_OK;
}

}  // extern "C"
