// tm_step.cu -- the fused Dornic step for sm_103a.
//
// One warp owns a strip of 32 columns x R rows (R <= 16) of one instance
// ("task") and walks down it with a three-row register window (north,
// centre, south; the next row is read one row ahead); east/west neighbours
// come from warp shuffles, the two strip-edge columns from one read per task.
// Each lattice value is read from HBM once per step and written once (8 B per
// site-update in FP32).  Sites that need a random draw are compacted into a
// per-warp queue in shared memory so that every lane of the sampler loop works
// on a live site: absorbing sites never occupy a sampler lane.  FP32 draws take
// a straight-line path first; the few sites it defers (a few % of live sites)
// go to the warp's own segment of a batch-wide list (no atomics: the warp keeps
// the count) that a second kernel draws with the general sampler, so the step
// kernel's loop body holds no general-sampler code.  The FP32 DP step stores
// each site as soon as its value is known: absorbing sites while the rows
// stream in (pass 1), drawn sites right after their draw (pass 2).  The
// Rietkerk draw and FP64 keep a third pass that stores from shared memory.  FP64
// draws every live site with the general sampler, carried from task to task and
// drawn 32 at a time.  Per site it fuses:
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

// Per-warp shared scratch for one task of up to rows_cap rows: the Dornic draw
// of every site (res), the queue of live sites (Poisson mean, shape, index),
// the list of sites left to the general sampler, and up to 31 of those carried
// over from earlier tasks (instance, site, Poisson mean, shape).
constexpr int kWarps = 8;

template <typename T>
__host__ __device__ __forceinline__ size_t warp_scratch_bytes(int rows_cap)
{
    return (size_t)rows_cap * 32 * (3 * sizeof(T) + 2 * sizeof(unsigned short)) + 32 * (2 * sizeof(T) + 8);
}

__device__ __forceinline__ bool is_pos_zero(float x) { return __float_as_uint(x) == 0u; }

// Row-major site index y L + x, the Philox counter's site word: unsigned, so it is
// defined for every L the batches accept (L <= 65535 keeps L^2 below 2^32).
__device__ __forceinline__ uint32_t site_index(int y, int L, int x)
{
    return (uint32_t)y * (uint32_t)L + (uint32_t)x;
}
__device__ __forceinline__ bool is_pos_zero(double x) { return __double_as_longlong(x) == 0LL; }

// Remainder, clamp and status bits of one site after its Dornic draw.
template <typename T, int REM>
__device__ __forceinline__ T finish_site(const DornicArgs<T>& A, T rs, T bi, unsigned& st)
{
    T res;
    if (REM == 0) {
        res = rs / (T(1) + (bi * rs) * A.dt);
    } else if (REM == 1) {
        const T k1 = rem_f(rs, bi, A.c, A.cubic);
        const T k2 = rem_f(rs + A.dt2 * k1, bi, A.c, A.cubic);
        const T k3 = rem_f(rs + A.dt2 * k2, bi, A.c, A.cubic);
        const T k4 = rem_f(rs + A.dt * k3, bi, A.c, A.cubic);
        // (k1 + 2 k2) + 2 k3: the doubling is exact, so each fused add rounds once as
        // the separate multiply and add do (same bits, one instruction)
        res = rs + A.dt6 * (Tr<T>::fma_(T(2), k3, Tr<T>::fma_(T(2), k2, k1)) + k4);
    } else {
        res = rs;
    }
    if (REM != 2) {
        if (res < A.ceps && res >= A.clo) res = T(0);
        st |= value_status(res);
    }
    return res;
}

// One site through the general sampler, then finished and stored.  The draw
// depends only on (seed, site, step), so it may run in any later pass of the
// same warp.
template <typename T, int REM, int SAMP, int CAP>
__device__ __forceinline__ void draw_general_site(const DornicArgs<T>& A, const SmemTab<T>& tab, long long step,
                                                  int k, uint32_t site, T m, T mu1)
{
    Stream<T> g;
    g.init(A.it.seed[k], site, step);
    const T rs = dornic_draw<CAP>(g, m, mu1, (T)A.it.consts[k].y, SAMP, tab);
    const long long o = A.it.off[k] + (long long)site;
    unsigned st = g.status;
    A.out[o] = finish_site<T, REM>(A, rs, A.site_b ? A.site_b[o] : A.b, st);
    if (st) atomicOr(A.it.status + k, st);
}

// SAMP is the sampler (0 exact, 1 Gaussian above 100, 2 noise off) as a
// compile-time constant: each instantiation carries only its own sampler's
// code, which keeps the loop body small for the instruction cache.  CAP is the
// attempts of each rejection loop: kSamplerCap, or 1 in the instantiation that
// TM_PROBE_SAMPLER_CAP1 selects (the straight-line draw makes one attempt of
// each loop, so it is unchanged).
template <typename T, int REM, int SAMP, int CAP>
__global__ void __launch_bounds__(256, (sizeof(T) == 4 ? 4 : 2)) dornic_step_kernel(const DornicArgs<T> A)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ SmemTab<T> tab;
    __shared__ unsigned defer_rows[kWarps][32];
    tab.fill();
    __syncthreads();
    const int cap = A.rows_cap * 32;
    unsigned char* wbase = smem_raw + (threadIdx.x >> 5) * warp_scratch_bytes<T>(A.rows_cap);
    T* const Wres = reinterpret_cast<T*>(wbase);
    T* const Wqm = Wres + cap;
    T* const Wqmu = Wqm + cap;
    T* const Cm = Wqmu + cap;
    T* const Cmu = Cm + 32;
    int* const Ck = reinterpret_cast<int*>(Cmu + 32);
    uint32_t* const Cs = reinterpret_cast<uint32_t*>(Ck + 32);
    unsigned short* const Wqi = reinterpret_cast<unsigned short*>(Cs + 32);
    unsigned short* const Wdef = Wqi + cap;
    unsigned* const Wrows = defer_rows[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    const int gw = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int nw = (int)((gridDim.x * blockDim.x) >> 5);
    const long long step = (A.step_base ? *A.step_base : 0LL) + A.step_off;
    int nc = 0;  // entries carried in Ck/Cs/Cm/Cmu (FP64)
    int nseg = 0;  // entries in this warp's segment of the deferred-site list (FP32)
    // FP64: one more trip after the last task draws the carried entries; the
    // general sampler has a single call site, so its code is in the loop body once.
    for (int t = gw;; t += nw) {
        const bool more = t < A.n_tasks;
        int k = 0, L = 0, x0 = 0, y0 = 0, ndef = 0;
        if (more) k = A.tasks[t].x;
        if (more && (A.it.alive == nullptr || A.it.alive[k] != 0)) {
            const int4 tk = A.tasks[t];
            L = A.it.L[k];
            const T* __restrict__ src = A.in + A.it.off[k];
            T* __restrict__ dst = A.out + A.it.off[k];
            const Dc4 cs = A.it.consts[k];
            const T pm = (T)cs.x, inv_lambda = (T)cs.y, a1 = (T)cs.z, a2 = (T)cs.w;
            x0 = tk.y;
            y0 = tk.z;
            const int rows = tk.w;
            const int w = min(32, L - x0);
            const int x = x0 + lane;
            const bool act = lane < w;
            const int xw = (x0 == 0) ? L - 1 : x0 - 1;
            const int xe = (x0 + w == L) ? 0 : x0 + w;
            const int yn = (y0 == 0) ? L - 1 : y0 - 1;
            // pass 1: stream the rows, form alpha_i, resolve absorbing sites and the
            // noise-off mean directly, queue the live sites (row-major order)
            // the strip-edge columns of the task's rows, one row per lane; the
            // column itself is read one row ahead of its use
            const bool erow = lane < rows;
            const T wcol = erow ? src[(long long)(y0 + lane) * L + xw] : T(0);
            const T ecol = erow ? src[(long long)(y0 + lane) * L + xe] : T(0);
            T north = act ? src[(long long)yn * L + x] : T(0);
            T cur = act ? src[(long long)y0 * L + x] : T(0);
            T south = act ? src[(long long)((y0 == L - 1) ? 0 : y0 + 1) * L + x] : T(0);
            int nq = 0;
            unsigned drows = 0;  // rows of this lane's column left to the general sampler (FP64)
            unsigned st = 0;
            // The FP32 DP step finishes and stores every site where its value is known:
            // absorbing and noise-off sites in pass 1, drawn sites in pass 2, so it has no
            // pass 3 and no round trip of the draws through shared memory.  (For P* of the
            // Rietkerk step the compiler then spills; it keeps the three passes.)
            constexpr bool kStoreEarly = sizeof(T) == 4 && REM != 2;
            const T* __restrict__ sb = (kStoreEarly && A.site_b) ? A.site_b + A.it.off[k] : nullptr;
            if (!kStoreEarly) Wrows[lane] = 0u;
            for (int r = 0; r < rows; ++r) {
                const int y = y0 + r;
                T next = T(0);
                if (r + 1 < rows) {
                    int y2 = y + 2;
                    if (y2 >= L) y2 -= L;
                    if (y2 >= L) y2 -= L;
                    next = act ? src[(long long)y2 * L + x] : T(0);
                }
                T west = __shfl_up_sync(0xffffffffu, cur, 1);
                T east = __shfl_down_sync(0xffffffffu, cur, 1);
                const T wedge = __shfl_sync(0xffffffffu, wcol, r);
                const T eedge = __shfl_sync(0xffffffffu, ecol, r);
                if (lane == 0) west = wedge;
                if (lane == w - 1) east = eedge;
                const T nsum = ((north + south) + west) + east;
                const T alpha = A.dcoef * nsum;
                const bool live = act && !(alpha == T(0) && cur == T(0)) && SAMP != 2;
                const unsigned bal = __ballot_sync(0xffffffffu, live);
                if (!live) {
                    if constexpr (kStoreEarly) {
                        if (act) {
                            const T rs = (SAMP == 2) ? a1 * cur + a2 * alpha : T(0);
                            const long long o = (long long)y * L + x;
                            T res = rs;
                            if (!(A.zero_fixed && is_pos_zero(rs)))
                                res = finish_site<T, REM>(A, rs, sb ? sb[o] : A.b, st);
                            dst[o] = res;
                        }
                    } else {
                        Wres[r * 32 + lane] = (SAMP == 2 && act) ? a1 * cur + a2 * alpha : T(0);
                    }
                }
                if (sizeof(T) == 8 && live) drows |= 1u << r;
                if (live) {
                    const int pos = nq + __popc(bal & lt_mask);
                    Wqi[pos] = (unsigned short)(r * 32 + lane);
                    Wqm[pos] = pm * cur;
                    Wqmu[pos] = alpha * A.two_s2;
                }
                nq += __popc(bal);
                north = cur;
                cur = south;
                south = next;
            }
            __syncwarp();
            // pass 2: FP32 takes the straight-line common case for every queued
            // site and lists the rest for the general sampler (same stream, same
            // bits); FP64 lists every queued site.
            const unsigned long long seed = A.it.seed[k];
            if constexpr (sizeof(T) == 4) {
                for (int base = 0; base < nq; base += 32) {
                    const int j = base + lane;
                    const bool has = j < nq;
                    bool deferred = false;
                    if (has) {
                        const int li = Wqi[j];
                        const uint32_t site = site_index(y0 + (li >> 5), L, x0 + (li & 31));
                        const float v = dornic_draw_fast(seed, site, step, Wqm[j], Wqmu[j], inv_lambda, SAMP, tab,
                                                         deferred);
                        if constexpr (kStoreEarly) {
                            if (!deferred) {
                                const long long o = (long long)(y0 + (li >> 5)) * L + x0 + (li & 31);
                                T res = v;
                                if (!(A.zero_fixed && is_pos_zero(v)))
                                    res = finish_site<T, REM>(A, v, sb ? sb[o] : A.b, st);
                                dst[o] = res;
                            }
                        } else {
                            if (deferred) atomicOr(Wrows + (li & 31), 1u << (li >> 5));
                            else Wres[li] = v;
                        }
                    }
                    // deferred sites: appended to this warp's segment of the list
                    const unsigned bal = __ballot_sync(0xffffffffu, has && deferred);
                    if (has && deferred) {
                        const int li = Wqi[j];
                        A.dlist[(long long)gw * A.seg_cap + nseg + __popc(bal & lt_mask)] =
                            make_uint4((unsigned)k, site_index(y0 + (li >> 5), L, x0 + (li & 31)),
                                       __float_as_uint(Wqm[j]), __float_as_uint(Wqmu[j]));
                    }
                    nseg += __popc(bal);
                }
                __syncwarp();
                if constexpr (!kStoreEarly) drows = Wrows[lane];
            } else {
                for (int j = lane; j < nq; j += 32) Wdef[j] = (unsigned short)j;
                ndef = nq;
                __syncwarp();
            }
            // pass 3: remainder, clamp, store (sites left to the general sampler
            // are finished and stored by it).  When zero_fixed holds a +0 draw --
            // every absorbing site -- finishes as +0 and skips the arithmetic.
            if (act && !kStoreEarly) {
                const T* __restrict__ sb3 = A.site_b ? A.site_b + A.it.off[k] : nullptr;
                for (int r = 0; r < rows; ++r) {
                    if ((drows >> r) & 1u) continue;
                    const T rs = Wres[r * 32 + lane];
                    T res = rs;
                    if (!(A.zero_fixed && is_pos_zero(rs))) {
                        const T bi = sb3 ? sb3[(long long)(y0 + r) * L + x] : A.b;
                        res = finish_site<T, REM>(A, rs, bi, st);
                    }
                    dst[(long long)(y0 + r) * L + x] = res;
                }
            }
            if (st) atomicOr(A.it.status + k, st);
        }
        // FP64 general sampler: the carried sites, then this task's list, 32 per
        // pass so that every lane draws; fewer than 32 are carried on (all of
        // them on the trip after the last task)
        if constexpr (sizeof(T) == 4) {
            if (!more) {
                if (lane == 0) A.dcnt[gw] = (unsigned)nseg;
                break;
            }
            __syncwarp();
            continue;
        }
        const int tot = nc + ndef;
        const int lim = more ? (tot & ~31) : tot;
        for (int done = 0; done < lim; done += 32) {
            const int e = done + lane;
            if (e < lim) {
                int ke = k;
                uint32_t se;
                T me, mue;
                if (e < nc) {
                    ke = Ck[e];
                    se = Cs[e];
                    me = Cm[e];
                    mue = Cmu[e];
                } else {
                    const int j = Wdef[e - nc];
                    const int li = Wqi[j];
                    se = site_index(y0 + (li >> 5), L, x0 + (li & 31));
                    me = Wqm[j];
                    mue = Wqmu[j];
                }
                draw_general_site<T, REM, SAMP, CAP>(A, tab, step, ke, se, me, mue);
            }
        }
        if (!more) break;
        __syncwarp();
        const int left = tot - lim;
        // a carried entry that is still left keeps its slot (lim == 0, e == lane)
        if (lane < left && lim + lane >= nc) {
            const int j = Wdef[lim + lane - nc];
            const int li = Wqi[j];
            Ck[lane] = k;
            Cs[lane] = site_index(y0 + (li >> 5), L, x0 + (li & 31));
            Cm[lane] = Wqm[j];
            Cmu[lane] = Wqmu[j];
        }
        nc = left;
        __syncwarp();
    }
}

// The FP32 sites the straight-line draw deferred, drawn by the general sampler
// from their list entries (instance, site, Poisson mean, Gamma shape): one warp
// per segment of the step kernel's grid, 32 entries at a time.
template <typename T, int REM, int SAMP, int CAP>
__global__ void __launch_bounds__(256) dornic_deferred_kernel(const DornicArgs<T> A, int n_seg)
{
    __shared__ SmemTab<T> tab;
    tab.fill();
    __syncthreads();
    const long long step = (A.step_base ? *A.step_base : 0LL) + A.step_off;
    const int lane = threadIdx.x & 31;
    const int gw = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int nw = (int)((gridDim.x * blockDim.x) >> 5);
    for (int w = gw; w < n_seg; w += nw) {
        const int n = (int)A.dcnt[w];
        const uint4* seg = A.dlist + (long long)w * A.seg_cap;
        for (int i = lane; i < n; i += 32) {
            const uint4 d = seg[i];
            draw_general_site<T, REM, SAMP, CAP>(A, tab, step, (int)d.x, d.y, __uint_as_float(d.z),
                                                 __uint_as_float(d.w));
        }
    }
}

template <typename T, int REM, int SAMP, int CAP = kSamplerCap>
cudaError_t launch_dornic_t(const DornicArgs<T>& a, int grid, int block, size_t smem, cudaStream_t s)
{
    static bool attr_set = false;
    if (!attr_set) {
        const int full = (int)(warp_scratch_bytes<T>(kMaxRowsPerTask) * kWarps);
        const cudaError_t e = cudaFuncSetAttribute(dornic_step_kernel<T, REM, SAMP, CAP>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, full);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    const int n_seg = grid * (block >> 5);   // one list segment per warp of the step kernel
    if constexpr (sizeof(T) == 4) {
        // every warp's segment must hold all sites of its tasks
        const long long need = ((long long)a.n_tasks + n_seg - 1) / n_seg * a.rows_cap * 32;
        if (a.dlist == nullptr || a.dcnt == nullptr || need > a.seg_cap || (long long)n_seg > a.max_seg ||
            (long long)n_seg * a.seg_cap > a.dlist_cap)
            return cudaErrorInvalidValue;
    }
    dornic_step_kernel<T, REM, SAMP, CAP><<<grid, block, smem, s>>>(a);
    if constexpr (sizeof(T) == 4) dornic_deferred_kernel<T, REM, SAMP, CAP><<<(n_seg + 7) / 8, 256, 0, s>>>(a, n_seg);
    return cudaGetLastError();
}

template <typename T, int REM>
cudaError_t launch_dornic_r(const DornicArgs<T>& a, int grid, int block, size_t smem, cudaStream_t s)
{
    if (a.cap1) {  // the sampler-cap probe: DP, Euler-exact remainder, exact sampler only
        if (REM == 0 && a.sampler == 0) return launch_dornic_t<T, 0, 0, 1>(a, grid, block, smem, s);
        return cudaErrorInvalidValue;
    }
    if (a.sampler == 0) return launch_dornic_t<T, REM, 0>(a, grid, block, smem, s);
    if (a.sampler == 1) return launch_dornic_t<T, REM, 1>(a, grid, block, smem, s);
    if (a.sampler == 2) return launch_dornic_t<T, REM, 2>(a, grid, block, smem, s);
    return cudaErrorInvalidValue;
}

template <typename T>
cudaError_t launch_dornic(const DornicArgs<T>& a, int rem, int grid, int block, cudaStream_t s)
{
    if (a.n_tasks <= 0) return cudaSuccess;
    if (block != 32 * kWarps || a.rows_cap < 1 || a.rows_cap > kMaxRowsPerTask) return cudaErrorInvalidValue;
    const size_t smem = warp_scratch_bytes<T>(a.rows_cap) * kWarps;
    if (rem == 0) return launch_dornic_r<T, 0>(a, grid, block, smem, s);
    if (rem == 1) return launch_dornic_r<T, 1>(a, grid, block, smem, s);
    if (rem == 2) return launch_dornic_r<T, 2>(a, grid, block, smem, s);
    return cudaErrorInvalidValue;
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

// Kadanoff block means (sde_RFT_2D...DEF.f:474-516): one thread per box x box
// block, summed in row order in FP64.
template <typename T>
__global__ void box_means_kernel(const T* f, int L, int box, double* out)
{
    const int nb = L / box;
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb * nb) return;
    const int by = b / nb, bx = b - by * nb;
    double s = 0.0;
    for (int y = 0; y < box; ++y)
        for (int x = 0; x < box; ++x) s += (double)f[(long long)(by * box + y) * L + bx * box + x];
    out[b] = s / ((double)box * (double)box);
}

template <typename T>
cudaError_t launch_box_means(const T* field, int L, int box, double* out, cudaStream_t s)
{
    const int n = (L / box) * (L / box);
    box_means_kernel<T><<<(n + 127) / 128, 128, 0, s>>>(field, L, box, out);
    return cudaGetLastError();
}
template cudaError_t launch_box_means<float>(const float*, int, int, double*, cudaStream_t);
template cudaError_t launch_box_means<double>(const double*, int, int, double*, cudaStream_t);

cudaError_t launch_set_step(long long* d_step, long long v, cudaStream_t s)
{
    set_step_kernel<<<1, 1, 0, s>>>(d_step, v);
    return cudaGetLastError();
}

}  // namespace tmg
