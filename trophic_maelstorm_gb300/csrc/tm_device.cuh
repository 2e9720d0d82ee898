// tm_device.cuh -- device-side arithmetic of the Dornic step for sm_103a.
//
// Counter-based random stream (Philox4x32-10), own elementary functions and
// the Poisson / Gamma / normal samplers used by the step kernels.  The
// specification is fixed operation by operation (compile with -fmad=false;
// every fused multiply-add is an explicit fma()), so a given
// (seed, site, step) produces the same variates on every GPU and matches the
// CPU restatement used by the tests bit for bit.
//
// Published methods implemented here:
//   Philox4x32-10  Salmon, Moraes, Dror, Shaw, SC'11 ("as easy as 1, 2, 3")
//   Poisson m>=32  Hormann 1993, PTRS (transformed rejection with squeeze)
//   Poisson m<32   inversion from the top of the tail with one 32-bit word
//   Gamma          Marsaglia & Tsang 2000, with the U^(1/k) boost for k<1 and
//                  the squeeze (1-u) 108 d min(1, 1+cx) > x^4: the acceptance
//                  bound is 3d h(cx), h(y) = log(1+y) - y + y^2/2 - y^3/3 >=
//                  -y^4 / (4 min(1, 1+y)), and log u <= u - 1
//   normal         ziggurat (Marsaglia & Tsang 2000), tables from oracle/gen_ziggurat.py
//   log / exp      Cody-Waite argument reduction + Taylor series
// The reference draws the same two distributions from libstdc++
// (stochasticSPDP.cpp:1054-1059, multiSPDP.cpp:2915-2943).
#pragma once
#include <stdint.h>
#include "tm_zig_table.cuh"

#define TM_STATUS_NAN_BIT 0x1u
#define TM_STATUS_NEG_BIT 0x2u
#define TM_STATUS_CAP_BIT 0x4u
#define TM_STATUS_WAIT_BIT 0x8u

namespace tmg {

// ---------------------------------------------------------------- Philox
struct U4 { uint32_t x, y, z, w; };

__device__ __forceinline__ U4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                            uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        const uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
        const uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
        const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    }
    return U4{c0, c1, c2, c3};
}

// ---------------------------------------------------------------- precision traits
template <typename T> struct Tr;
template <> struct Tr<double> {
    static __device__ __forceinline__ double fma_(double a, double b, double c) { return fma(a, b, c); }
    static __device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
    static __device__ __forceinline__ double inv_sqrt(double x) { return 1.0 / sqrt(x); }
    static __device__ __forceinline__ double floor_(double x) { return floor(x); }
    static __device__ __forceinline__ double trunc_(double x) { return trunc(x); }
    static __device__ __forceinline__ double rint_(double x) { return rint(x); }
    static __device__ __forceinline__ double fabs_(double x) { return fabs(x); }
};
template <> struct Tr<float> {
    static __device__ __forceinline__ float fma_(float a, float b, float c) { return fmaf(a, b, c); }
    static __device__ __forceinline__ float sqrt_(float x) { return sqrtf(x); }
    // correctly rounded 1/sqrt(x) (one rounding, where 1.0f / sqrtf(x) rounds twice)
    static __device__ __forceinline__ float inv_sqrt(float x) { return __frsqrt_rn(x); }
    static __device__ __forceinline__ float floor_(float x) { return floorf(x); }
    static __device__ __forceinline__ float trunc_(float x) { return truncf(x); }
    static __device__ __forceinline__ float rint_(float x) { return rintf(x); }
    static __device__ __forceinline__ float fabs_(float x) { return fabsf(x); }
};

// ---------------------------------------------------------------- elementary functions
// 2 atanh(s) = 2s + 2s z (1/3 + z/5 + ...), z = s^2, |s| <= 0.1716
__device__ __forceinline__ double atanh2_series(double s)
{
    const double z = s * s;
    double p = (double)(1.0 / 21.0);
    p = fma(z, p, (double)(1.0 / 19.0));
    p = fma(z, p, (double)(1.0 / 17.0));
    p = fma(z, p, (double)(1.0 / 15.0));
    p = fma(z, p, (double)(1.0 / 13.0));
    p = fma(z, p, (double)(1.0 / 11.0));
    p = fma(z, p, (double)(1.0 / 9.0));
    p = fma(z, p, (double)(1.0 / 7.0));
    p = fma(z, p, (double)(1.0 / 5.0));
    p = fma(z, p, (double)(1.0 / 3.0));
    p = p * z;
    const double t = s + s;
    return fma(t, p, t);
}
__device__ __forceinline__ float atanh2_series(float s)
{
    const float z = s * s;
    float p = (float)(1.0 / 11.0);
    p = fmaf(z, p, (float)(1.0 / 9.0));
    p = fmaf(z, p, (float)(1.0 / 7.0));
    p = fmaf(z, p, (float)(1.0 / 5.0));
    p = fmaf(z, p, (float)(1.0 / 3.0));
    p = p * z;
    const float t = s + s;
    return fmaf(t, p, t);
}

__device__ __forceinline__ double tm_log(double x)
{
    if (x != x) return x;
    if (x < 0.0) return __longlong_as_double(0x7ff8000000000000LL);
    if (x == 0.0) return -__longlong_as_double(0x7ff0000000000000LL);
    if (x == __longlong_as_double(0x7ff0000000000000LL)) return x;
    unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    int be = (int)((bits >> 52) & 0x7ff);
    int adj = 0;
    if (be == 0) {
        const double y = x * 0x1p54;
        bits = (unsigned long long)__double_as_longlong(y);
        be = (int)((bits >> 52) & 0x7ff);
        adj = 54;
    }
    int e = be - 1023 - adj;
    bits = (bits & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL;
    double m = __longlong_as_double((long long)bits);
    if (m > 0x1.6a09e667f3bcdp+0) { m = m * 0.5; e = e + 1; }
    const double f = m - 1.0;
    const double s = f / (2.0 + f);
    const double lm = atanh2_series(s);
    const double fe = (double)e;
    return fma(fe, 0x1.62e42fee00000p-1, fma(fe, 0x1.a39ef35793c76p-33, lm));
}
__device__ __forceinline__ float tm_log(float x)
{
    if (x != x) return x;
    if (x < 0.0f) return __int_as_float(0x7fc00000);
    if (x == 0.0f) return -__int_as_float(0x7f800000);
    if (x == __int_as_float(0x7f800000)) return x;
    uint32_t bits = __float_as_uint(x);
    int be = (int)((bits >> 23) & 0xff);
    int adj = 0;
    if (be == 0) {
        const float y = x * 0x1p25f;
        bits = __float_as_uint(y);
        be = (int)((bits >> 23) & 0xff);
        adj = 25;
    }
    int e = be - 127 - adj;
    bits = (bits & 0x007fffffu) | 0x3f800000u;
    float m = __uint_as_float(bits);
    if (m > 0x1.6a09e6p+0f) { m = m * 0.5f; e = e + 1; }
    const float f = m - 1.0f;
    const float s = f / (2.0f + f);
    const float lm = atanh2_series(s);
    const float fe = (float)e;
    return fmaf(fe, 0x1.62ep-1f, fmaf(fe, 0x1.0bfbe8p-15f, lm));
}

// log for arguments known to be positive, finite and normal (uniform
// variates, means, shapes): the same arithmetic as tm_log without the
// special-case branches, so it returns the same bits for such arguments.
__device__ __forceinline__ double tm_log_pos(double x)
{
    unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    int e = (int)((bits >> 52) & 0x7ff) - 1023;
    bits = (bits & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL;
    double m = __longlong_as_double((long long)bits);
    if (m > 0x1.6a09e667f3bcdp+0) { m = m * 0.5; e = e + 1; }
    const double f = m - 1.0;
    const double s = f / (2.0 + f);
    const double lm = atanh2_series(s);
    const double fe = (double)e;
    return fma(fe, 0x1.62e42fee00000p-1, fma(fe, 0x1.a39ef35793c76p-33, lm));
}
__device__ __forceinline__ float tm_log_pos(float x)
{
    uint32_t bits = __float_as_uint(x);
    int e = (int)((bits >> 23) & 0xff) - 127;
    bits = (bits & 0x007fffffu) | 0x3f800000u;
    float m = __uint_as_float(bits);
    if (m > 0x1.6a09e6p+0f) { m = m * 0.5f; e = e + 1; }
    const float f = m - 1.0f;
    const float s = f / (2.0f + f);
    const float lm = atanh2_series(s);
    const float fe = (float)e;
    return fmaf(fe, 0x1.62ep-1f, fmaf(fe, 0x1.0bfbe8p-15f, lm));
}

__device__ __forceinline__ double tm_log1p(double x)
{
    if (x > -0.29 && x < 0.41) return atanh2_series(x / (2.0 + x));
    return tm_log(1.0 + x);
}
__device__ __forceinline__ float tm_log1p(float x)
{
    if (x > (float)(-0.29) && x < (float)(0.41)) return atanh2_series(x / (2.0f + x));
    return tm_log(1.0f + x);
}

__device__ __forceinline__ double tm_exp(double x)
{
    if (x != x) return x;
    if (x > 709.782712893384) return __longlong_as_double(0x7ff0000000000000LL);
    if (x < -745.1332191019411) return 0.0;
    const double k = rint(x * 0x1.71547652b82fep+0);
    double r = fma(-k, 0x1.62e42fee00000p-1, x);
    r = fma(-k, 0x1.a39ef35793c76p-33, r);
    double p = (double)(1.0 / 6227020800.0);
    p = fma(r, p, (double)(1.0 / 479001600.0));
    p = fma(r, p, (double)(1.0 / 39916800.0));
    p = fma(r, p, (double)(1.0 / 3628800.0));
    p = fma(r, p, (double)(1.0 / 362880.0));
    p = fma(r, p, (double)(1.0 / 40320.0));
    p = fma(r, p, (double)(1.0 / 5040.0));
    p = fma(r, p, (double)(1.0 / 720.0));
    p = fma(r, p, (double)(1.0 / 120.0));
    p = fma(r, p, (double)(1.0 / 24.0));
    p = fma(r, p, (double)(1.0 / 6.0));
    p = fma(r, p, 0.5);
    p = fma(r, p, 1.0);
    p = fma(r, p, 1.0);
    const int ki = (int)k;
    const int k1 = ki / 2, k2 = ki - k1;
    const double s1 = __longlong_as_double((long long)((unsigned long long)(k1 + 1023) << 52));
    const double s2 = __longlong_as_double((long long)((unsigned long long)(k2 + 1023) << 52));
    return (p * s1) * s2;
}
__device__ __forceinline__ float tm_exp(float x)
{
    if (x != x) return x;
    if (x > 88.72283f) return __int_as_float(0x7f800000);
    if (x < -103.972084f) return 0.0f;
    const float k = rintf(x * 0x1.715476p+0f);
    float r = fmaf(-k, 0x1.62ep-1f, x);
    r = fmaf(-k, 0x1.0bfbe8p-15f, r);
    float p = (float)(1.0 / 5040.0);
    p = fmaf(r, p, (float)(1.0 / 720.0));
    p = fmaf(r, p, (float)(1.0 / 120.0));
    p = fmaf(r, p, (float)(1.0 / 24.0));
    p = fmaf(r, p, (float)(1.0 / 6.0));
    p = fmaf(r, p, 0.5f);
    p = fmaf(r, p, 1.0f);
    p = fmaf(r, p, 1.0f);
    const int ki = (int)k;
    const int k1 = ki / 2, k2 = ki - k1;
    const float s1 = __uint_as_float((uint32_t)(k1 + 127) << 23);
    const float s2 = __uint_as_float((uint32_t)(k2 + 127) << 23);
    return (p * s1) * s2;
}

// e^x for -32 < x <= 0 (the start e^-m of the Poisson search): tm_exp's
// arithmetic without its range checks and with one scale by 2^k.  On this range
// k >= -47 and the scaled value is a normal float, so the single scale is
// exact, as tm_exp's two half scales are: the same bits as tm_exp.
__device__ __forceinline__ float tm_exp_neg_small(float x)
{
    const float k = rintf(x * 0x1.715476p+0f);
    float r = fmaf(-k, 0x1.62ep-1f, x);
    r = fmaf(-k, 0x1.0bfbe8p-15f, r);
    float p = (float)(1.0 / 5040.0);
    p = fmaf(r, p, (float)(1.0 / 720.0));
    p = fmaf(r, p, (float)(1.0 / 120.0));
    p = fmaf(r, p, (float)(1.0 / 24.0));
    p = fmaf(r, p, (float)(1.0 / 6.0));
    p = fmaf(r, p, 0.5f);
    p = fmaf(r, p, 1.0f);
    p = fmaf(r, p, 1.0f);
    return p * __uint_as_float((uint32_t)((int)k + 127) << 23);
}

// 1 - e^-m for m >= 0 (alternating series below 0.25)
__device__ __forceinline__ double tm_negexpm1(double m)
{
    if (m < 0.25) {
        double p = (double)(1.0 / 6227020800.0);
        p = fma(m, p, (double)(-1.0 / 479001600.0));
        p = fma(m, p, (double)(1.0 / 39916800.0));
        p = fma(m, p, (double)(-1.0 / 3628800.0));
        p = fma(m, p, (double)(1.0 / 362880.0));
        p = fma(m, p, (double)(-1.0 / 40320.0));
        p = fma(m, p, (double)(1.0 / 5040.0));
        p = fma(m, p, (double)(-1.0 / 720.0));
        p = fma(m, p, (double)(1.0 / 120.0));
        p = fma(m, p, (double)(-1.0 / 24.0));
        p = fma(m, p, (double)(1.0 / 6.0));
        p = fma(m, p, -0.5);
        p = fma(m, p, 1.0);
        return m * p;
    }
    return 1.0 - tm_exp(-m);
}
__device__ __forceinline__ float tm_negexpm1(float m)
{
    if (m < 0.25f) {
        float p = (float)(-1.0 / 40320.0);
        p = fmaf(m, p, (float)(1.0 / 5040.0));
        p = fmaf(m, p, (float)(-1.0 / 720.0));
        p = fmaf(m, p, (float)(1.0 / 120.0));
        p = fmaf(m, p, (float)(-1.0 / 24.0));
        p = fmaf(m, p, (float)(1.0 / 6.0));
        p = fmaf(m, p, -0.5f);
        p = fmaf(m, p, 1.0f);
        return m * p;
    }
    return 1.0f - tm_exp(-m);
}

// ---------------------------------------------------------------- stream
// Counter (site, step_lo, call, step_hi), key (seed_lo, seed_hi).  Words are
// consumed in order; a shift register keeps them in registers.
template <typename T>
struct Stream {
    uint32_t k0, k1, site, slo, shi, call;
    uint32_t b0, b1, b2, b3;
    int avail;
    uint32_t status;

    __device__ __forceinline__ void init(uint64_t seed, uint32_t site_, int64_t step)
    {
        k0 = (uint32_t)seed; k1 = (uint32_t)(seed >> 32);
        site = site_; slo = (uint32_t)(uint64_t)step; shi = (uint32_t)((uint64_t)step >> 32);
        call = 0; avail = 0; status = 0;
        b0 = b1 = b2 = b3 = 0;
    }
    __device__ __forceinline__ uint32_t u32()
    {
        if (avail == 0) {
            const U4 r = philox4x32_10(site, slo, call, shi, k0, k1);
            b0 = r.x; b1 = r.y; b2 = r.z; b3 = r.w;
            call += 1u;
            avail = 4;
        }
        const uint32_t w = b0;
        b0 = b1; b1 = b2; b2 = b3;
        --avail;
        return w;
    }
    // uniform on (0,1)
    __device__ __forceinline__ T open();
    template <int CAP, class Tab>
    __device__ __forceinline__ T normal(const Tab& tb);
};

template <> __device__ __forceinline__ double Stream<double>::open()
{
    const uint32_t w1 = u32();
    const uint32_t w2 = u32();
    const unsigned long long x = ((unsigned long long)w1 << 21) | (unsigned long long)(w2 >> 11);
    return ((double)x + 0.5) * 0x1p-53;
}
template <> __device__ __forceinline__ float Stream<float>::open()
{
    const uint32_t w = u32();
    return ((float)(w >> 8) + 0.5f) * 0x1p-24f;
}

// Ziggurat word split: layer index (low kZigBits bits) and the signed value
// (the remaining bits, centred on 0).
__device__ __forceinline__ int zig_layer(uint32_t w) { return (int)(w & (uint32_t)(kZigN - 1)); }
__device__ __forceinline__ int32_t zig_value(uint32_t w)
{
    return (int32_t)(w >> kZigBits) - (int32_t)(1 << (31 - kZigBits));
}
static_assert(kZigN == (1 << kZigBits), "ziggurat layer count");

// Tables every sampler reads, staged in shared memory by the kernel:
// rcp[n] = 1/n (n <= 200) and the ziggurat (K: threshold and W: width of each
// layer, side by side so that one load reads both; F: f(x_i)).  For FP32, rcp[1]
// sits on a 16-byte boundary: the straight-line inversion reads rcp[it+1..it+4]
// with one vector load.
constexpr int kRcpTable = 201;
// Attempts of every rejection loop before TM_STATUS_CAP_BIT: the samplers take
// it as a template argument CAP, kSamplerCap everywhere but in the one kernel
// instantiation a test uses to make the cap path run (CAP = 1).
constexpr int kSamplerCap = 64;
template <typename T>
struct ZigLayer {
    uint32_t k;
    T w;
};
template <typename T>
struct __align__(16) SmemTab {
    T pad_[3];
    T rcp[kRcpTable];
    ZigLayer<T> zig[kZigN];
    T zf[kZigN + 1];
    __device__ __forceinline__ void fill()
    {
        for (int i = threadIdx.x; i < kRcpTable; i += blockDim.x) rcp[i] = (i == 0) ? T(0) : T(1) / (T)i;
        for (int i = threadIdx.x; i < kZigN; i += blockDim.x) zig[i] = ZigLayer<T>{kZigK[i], (T)kZigW[i]};
        for (int i = threadIdx.x; i <= kZigN; i += blockDim.x) zf[i] = (T)kZigF[i];
    }
};
static_assert(sizeof(ZigLayer<float>) == 8, "one 8-byte load per layer");

// standard normal by the ziggurat: one 32-bit word per attempt (layer index
// from the low kZigBits bits, signed value from the rest), wedge test or
// Marsaglia's tail method when the fast test fails.
template <typename T>
template <int CAP, class Tab>
__device__ __forceinline__ T Stream<T>::normal(const Tab& tb)
{
    for (int it = 0; it < CAP; ++it) {
        const uint32_t w = u32();
        const int iz = zig_layer(w);
        const int32_t hz = zig_value(w);
        const uint32_t az = (uint32_t)(hz < 0 ? -hz : hz);
        const ZigLayer<T> zl = tb.zig[iz];
        const T x = (T)hz * zl.w;
        if (az < zl.k) return x;
        if (iz == 0) {
            for (int jt = 0; jt < CAP; ++jt) {
                const T xt = -tm_log_pos(open()) * T(1.0 / kZigR);
                const T yt = -tm_log_pos(open());
                if (yt + yt >= xt * xt) {
                    const T r = T(kZigR) + xt;
                    return hz < 0 ? -r : r;
                }
            }
            break;
        }
        const T fb = tb.zf[iz], ft = tb.zf[iz + 1];
        if (fb + open() * (ft - fb) < tm_exp(T(-0.5) * (x * x))) return x;
    }
    status |= TM_STATUS_CAP_BIT;
    return T(0);
}

// log k!, k < 16
__device__ __forceinline__ double logfact_small(int k)
{
    switch (k) {
    case 2: return 0x1.62e42fefa39efp-1;
    case 3: return 0x1.cab0bfa2a2002p+0;
    case 4: return 0x1.96ca77c922cf9p+1;
    case 5: return 0x1.326643c4479c9p+2;
    case 6: return 0x1.a51273acf01cap+2;
    case 7: return 0x1.10ce1f32dcc30p+3;
    case 8: return 0x1.5358e82fcb70dp+3;
    case 9: return 0x1.99a8921a7f7cfp+3;
    case 10: return 0x1.e357590954d15p+3;
    case 11: return 0x1.180973f3a8d74p+4;
    case 12: return 0x1.3fcba16d50143p+4;
    case 13: return 0x1.68d5a9c3b32cep+4;
    case 14: return 0x1.930f3df162a42p+4;
    case 15: return 0x1.be636a63fd346p+4;
    default: return 0.0;
    }
}

// ---------------------------------------------------------------- samplers
template <int CAP, typename T>
__device__ __forceinline__ T poisson_exact(Stream<T>& g, T m, const SmemTab<T>& tb)
{
    if (!(m > T(0))) return T(0);
    if (m < T(32)) {
        const uint32_t w = g.u32();
        const T u = (T)w * T(0x1p-32);
        const bool small = m < T(0.25);                      // tm_negexpm1's own split
        T p = small ? T(0) : tm_exp(-m);
        T q = small ? tm_negexpm1(m) : T(1) - p;
        if (small && u < q) p = tm_exp(-m);                   // e^-m only when the search starts
        T n = T(0);
        int it = 0;
        while (u < q && it < 200) {
            ++it;
            n = n + T(1);
            p = (p * m) * tb.rcp[it];
            q = q - p;
        }
        return n;
    }
    const T slam = Tr<T>::sqrt_(m);
    const T loglam = tm_log_pos(m);
    const T b = T(0.931) + T(2.53) * slam;
    const T a = T(-0.059) + T(0.02483) * b;
    const T invalpha = T(1.1239) + T(1.1328) / (b - T(3.4));
    const T vr = T(0.9277) - T(3.6224) / (b - T(2));
    const T loginvalpha = tm_log_pos(invalpha);
    for (int it = 0; it < CAP; ++it) {
        const T U = g.open() - T(0.5);
        const T V = g.open();
        const T us = T(0.5) - Tr<T>::fabs_(U);
        const T k = Tr<T>::floor_((T(2) * a / us + b) * U + m + T(0.43));
        if (us >= T(0.07) && V <= vr) return k;
        if (k < T(0) || (us < T(0.013) && V > us)) continue;
        const T lhs = (tm_log_pos(V) + loginvalpha) - tm_log_pos(a / (us * us) + b);
        T rhs;
        if (k < T(16)) {
            rhs = (k * loglam - m) - (T)logfact_small((int)k);
        } else {
            const T z = k + T(1);
            const T d = z - m;
            const T iz = T(1) / z;
            const T iz2 = iz * iz;
            const T corr = iz * (T(1.0 / 12.0) - iz2 * (T(1.0 / 360.0) - iz2 * T(1.0 / 1260.0)));
            rhs = ((d - k * tm_log1p(d / m)) - T(0.5) * tm_log_pos(z)) - (T(0x1.d67f1c864beb4p-1) + corr);
        }
        if (lhs <= rhs) return k;
    }
    g.status |= TM_STATUS_CAP_BIT;
    return Tr<T>::floor_(m);
}

template <int CAP, typename T>
__device__ __forceinline__ T gamma_mt(Stream<T>& g, T k, const SmemTab<T>& tb)
{
    if (!(k > T(0))) return T(0);
    const T kk = (k < T(1)) ? k + T(1) : k;
    const T d = kk - T(1.0 / 3.0);
    const T c = Tr<T>::inv_sqrt(T(9) * d);
    T res = kk;
    bool done = false;
    for (int it = 0; it < CAP && !done; ++it) {
        T x = T(0), v = T(0);
        bool ok = false;
        for (int jt = 0; jt < CAP; ++jt) {
            x = g.template normal<CAP>(tb);
            v = T(1) + c * x;
            if (v > T(0)) { ok = true; break; }
        }
        if (!ok) break;
        const T mm = (v < T(1)) ? v : T(1);
        v = (v * v) * v;
        const T u = g.open();
        const T x2 = x * x;
        if ((T(1) - u) * ((T(108) * d) * mm) > x2 * x2) { res = d * v; done = true; break; }
        if (tm_log_pos(u) < T(0.5) * x2 + d * ((T(1) - v) + tm_log(v))) { res = d * v; done = true; break; }
    }
    if (!done) g.status |= TM_STATUS_CAP_BIT;
    if (k < T(1)) {
        const T u = g.open();
        res = res * tm_exp(tm_log_pos(u) / k);
    }
    return res;
}

// sampler: 0 exact, 1 Gaussian above 100 (multiSPDP.cpp:2915-2943)
template <int CAP, typename T>
__device__ __forceinline__ T poisson_draw(Stream<T>& g, T m, int sampler, const SmemTab<T>& tb)
{
    if (!(m > T(0))) return T(0);
    if (sampler == 1 && m > T(100)) {
        const T z = g.template normal<CAP>(tb);
        return Tr<T>::trunc_(z * Tr<T>::sqrt_(m) + m);
    }
    return poisson_exact<CAP>(g, m, tb);
}

template <int CAP, typename T>
__device__ __forceinline__ T gamma_draw(Stream<T>& g, T k, int sampler, const SmemTab<T>& tb)
{
    if (sampler == 1 && k > T(100)) {
        const T z = g.template normal<CAP>(tb);
        return z * Tr<T>::sqrt_(k) + k;
    }
    return gamma_mt<CAP>(g, k, tb);
}

// rho* = Gamma(mu1 + Poisson(m)) / lambda  (stochasticSPDP.cpp:1053-1059)
template <int CAP, typename T>
__device__ __forceinline__ T dornic_draw(Stream<T>& g, T m, T mu1, T inv_lambda, int sampler,
                                        const SmemTab<T>& tb)
{
    const T n = poisson_draw<CAP>(g, m, sampler, tb);
    const T k = mu1 + n;
    const T gv = gamma_draw<CAP>(g, k, sampler, tb);
    return gv * inv_lambda;
}

// Straight-line draw for the common case (FP32): one Philox block of four
// words, Poisson by inversion finishing within kFastInv steps, a ziggurat
// normal accepted by its fast test, one Marsaglia-Tsang attempt accepted by
// the squeeze and, for shape < 1, the U^(1/k) boost from the next word.  Every
// step consumes the counter stream exactly as dornic_draw does, so when it
// returns without deferring the value equals dornic_draw's bit for bit;
// otherwise (*deferred) the caller recomputes the site with dornic_draw.
constexpr int kFastInv = 32;
static_assert(kFastInv % 4 == 0, "the inversion takes four terms per trip");

__device__ __forceinline__ float dornic_draw_fast(uint64_t seed, uint32_t site, int64_t step, float m, float mu1,
                                                  float inv_lambda, int sampler, const SmemTab<float>& tb,
                                                  bool& deferred)
{
    deferred = false;
    const U4 r = philox4x32_10(site, (uint32_t)(uint64_t)step, 0u, (uint32_t)((uint64_t)step >> 32),
                               (uint32_t)seed, (uint32_t)(seed >> 32));
    float n = 0.0f;
    const bool draw = m > 0.0f;
    if (sampler == 1 && m > 100.0f) {
        // Gaussian approximations of both draws (multiSPDP.cpp:2922-2943): one
        // ziggurat word each
        const int i1 = zig_layer(r.x);
        const int32_t h1 = zig_value(r.x);
        const uint32_t a1 = (uint32_t)(h1 < 0 ? -h1 : h1);
        const ZigLayer<float> l1 = tb.zig[i1];
        if (!(a1 < l1.k)) { deferred = true; return 0.0f; }
        const float z1 = (float)h1 * l1.w;
        const float kk = mu1 + truncf(z1 * sqrtf(m) + m);
        if (!(kk > 100.0f)) { deferred = true; return 0.0f; }
        const int i2 = zig_layer(r.y);
        const int32_t h2 = zig_value(r.y);
        const uint32_t a2 = (uint32_t)(h2 < 0 ? -h2 : h2);
        const ZigLayer<float> l2 = tb.zig[i2];
        if (!(a2 < l2.k)) { deferred = true; return 0.0f; }
        const float z2 = (float)h2 * l2.w;
        return (z2 * sqrtf(kk) + kk) * inv_lambda;
    }
    if (draw) {
        if (!(m < 32.0f)) { deferred = true; return 0.0f; }
        const float u = (float)r.x * 0x1p-32f;
        // e^-m is only needed once u < q; below m = 0.25 q has its own series
        const bool small = m < 0.25f;
        float p = small ? 0.0f : tm_exp_neg_small(-m);
        float q = small ? tm_negexpm1(m) : 1.0f - p;
        if (small && u < q) p = tm_exp_neg_small(-m);
        // four terms per trip: the same products and differences as one term
        // per trip (kFastInv is a multiple of 4), tested after the second and
        // the fourth term.  q only decreases (p >= 0), so the terms with u < q
        // form a prefix, and a failed test counts the one term before it that
        // still had u < q -- the same count as testing every term, with half the
        // branches.
        int it = 0;
        while (u < q && it < kFastInv) {
            const float4 r4 = *reinterpret_cast<const float4*>(tb.rcp + it + 1);
            const float p1 = (p * m) * r4.x;
            const float q1 = q - p1;
            const float p2 = (p1 * m) * r4.y;
            const float q2 = q1 - p2;
            if (!(u < q2)) { it += 1 + (int)(u < q1); q = q2; break; }
            const float p3 = (p2 * m) * r4.z;
            const float q3 = q2 - p3;
            p = (p3 * m) * r4.w;
            q = q3 - p;
            if (!(u < q)) { it += 3 + (int)(u < q3); break; }
            it += 4;
        }
        if (u < q) { deferred = true; return 0.0f; }
        n = (float)it;
    }
    const float k = mu1 + n;
    if (!(k > 0.0f)) return 0.0f;  // Gamma(0) = 0, no draw
    if (sampler == 1 && k > 100.0f) { deferred = true; return 0.0f; }
    const uint32_t wz = draw ? r.y : r.x, wu = draw ? r.z : r.y, wb = draw ? r.w : r.z;
    const bool boost = k < 1.0f;            // Gamma(k) = Gamma(k+1) U^(1/k)
    const float kk = boost ? k + 1.0f : k;
    const float d = kk - (float)(1.0 / 3.0);
    const float c = Tr<float>::inv_sqrt(9.0f * d);
    const int iz = zig_layer(wz);
    const int32_t hz = zig_value(wz);
    const uint32_t az = (uint32_t)(hz < 0 ? -hz : hz);
    const ZigLayer<float> lz = tb.zig[iz];
    if (!(az < lz.k)) { deferred = true; return 0.0f; }
    const float x = (float)hz * lz.w;
    float v = 1.0f + c * x;
    if (!(v > 0.0f)) { deferred = true; return 0.0f; }
    const float mm = (v < 1.0f) ? v : 1.0f;
    v = (v * v) * v;
    const float u = ((float)(wu >> 8) + 0.5f) * 0x1p-24f;
    const float x2 = x * x;
    if (!((1.0f - u) * ((108.0f * d) * mm) > x2 * x2)) { deferred = true; return 0.0f; }
    float res = d * v;
    if (boost) {
        const float ub = ((float)(wb >> 8) + 0.5f) * 0x1p-24f;
        res = res * tm_exp(tm_log_pos(ub) / k);
    }
    return res * inv_lambda;
}

template <typename T>
__device__ __forceinline__ uint32_t value_status(T x)
{
    uint32_t s = 0;
    if (!(x == x) || Tr<T>::fabs_(x) == T(INFINITY)) s |= TM_STATUS_NAN_BIT;
    if (x < T(0)) s |= TM_STATUS_NEG_BIT;
    return s;
}

}  // namespace tmg
