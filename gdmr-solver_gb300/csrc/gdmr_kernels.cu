// Device kernels of the GB300 DMR restart cycle.  See gdmr_kernels.cuh.
#include "gdmr_kernels.cuh"

#include <type_traits>

#include <math.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

namespace gdmr {

namespace {

constexpr int NT = 256;            // threads per CTA of the streaming kernels
constexpr int NW = NT / 32;
constexpr int QMAX = 168;          // max coefficients per projection (basisDim <= 160 -> m+1 <= 161)

template <class C> __device__ __forceinline__ C from_d(double2 a);
template <> __device__ __forceinline__ float2 from_d<float2>(double2 a) { return make_float2((float)a.x, (float)a.y); }
template <> __device__ __forceinline__ double2 from_d<double2>(double2 a) { return a; }
template <> __device__ __forceinline__ dfc from_d<dfc>(double2 a) {
    dfc c;
    c.x = dfr(a.x);
    c.y = dfr(a.y);
    return c;
}
__device__ __forceinline__ double2 to_d(float2 a) { return make_double2(a.x, a.y); }
__device__ __forceinline__ double2 to_d(double2 a) { return a; }
__device__ __forceinline__ double2 to_d(dfc a) { return make_double2((double)a.x, (double)a.y); }

template <class C> __device__ __forceinline__ C czero() { C z; z.x = 0; z.y = 0; return z; }

// a * b + c in the working real type
__device__ __forceinline__ float rfma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double rfma(double a, double b, double c) { return ::fma(a, b, c); }
// Double-float a * b + c for accumulation chains: the exact two-product and two-sum, with no
// renormalisation; hi + lo stays exact and lo grows by about an ulp of hi per step, so a
// chain ends with canon() before its value is stored or squared.
__device__ __forceinline__ dfr rfma(dfr a, dfr b, dfr c) {
    const float p = a.hi * b.hi;
    const float pe = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, fmaf(a.hi, b.hi, -p)));
    const float s = p + c.hi, bb = s - p;
    return dfr(s, ((p - (s - bb)) + (c.hi - bb)) + (pe + c.lo));
}
// canonical form of an accumulated value (identity for the native types)
__device__ __forceinline__ float2 canon(float2 a) { return a; }
__device__ __forceinline__ double2 canon(double2 a) { return a; }
__device__ __forceinline__ dfc canon(dfc a) {
    a.x = df_renorm(a.x.hi, a.x.lo);
    a.y = df_renorm(a.y.hi, a.y.lo);
    return a;
}
// |a|^2 in double
__device__ __forceinline__ double abs2_d(float2 a) { return (double)a.x * a.x + (double)a.y * a.y; }
__device__ __forceinline__ double abs2_d(double2 a) { return a.x * a.x + a.y * a.y; }
__device__ __forceinline__ double abs2_d(dfc a) {
    const double x = (double)a.x, y = (double)a.y;
    return x * x + y * y;
}

// acc += a * b
template <class C> __device__ __forceinline__ void cfma(C &acc, C a, C b) {
    acc.x = rfma(a.x, b.x, acc.x);
    acc.x = rfma(-a.y, b.y, acc.x);
    acc.y = rfma(a.x, b.y, acc.y);
    acc.y = rfma(a.y, b.x, acc.y);
}
// acc += a * b where a is known to be real when `real` (its zero imaginary part would add
// zeros: the same value either way, with half the multiplies)
template <class C> __device__ __forceinline__ void cfma_r(C &acc, C a, C b, bool real) {
    if (real) {
        acc.x = rfma(a.x, b.x, acc.x);
        acc.y = rfma(a.x, b.y, acc.y);
    } else {
        cfma(acc, a, b);
    }
}
// acc -= a * b
template <class C> __device__ __forceinline__ void cfms(C &acc, C a, C b) {
    acc.x = rfma(-a.x, b.x, acc.x);
    acc.x = rfma(a.y, b.y, acc.x);
    acc.y = rfma(-a.x, b.y, acc.y);
    acc.y = rfma(-a.y, b.x, acc.y);
}
// acc -= a * b, a real when `real` (as cfma_r)
template <class C> __device__ __forceinline__ void cfms_r(C &acc, C a, C b, bool real) {
    if (real) {
        acc.x = rfma(-a.x, b.x, acc.x);
        acc.y = rfma(-a.x, b.y, acc.y);
    } else {
        cfms(acc, a, b);
    }
}
// acc += conj(a) * b
template <class C> __device__ __forceinline__ void cdotacc(C &acc, C a, C b) {
    acc.x = rfma(a.x, b.x, acc.x);
    acc.x = rfma(a.y, b.y, acc.x);
    acc.y = rfma(a.x, b.y, acc.y);
    acc.y = rfma(-a.y, b.x, acc.y);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ dfr warp_sum(dfr v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v = v + dfr(__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o));
    return v;
}

// Block-wide sum of NV doubles per thread; result valid in thread 0.
template <int NV> __device__ __forceinline__ void block_sum(double (&v)[NV], double (*red)[NW]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < NV; ++j) v[j] = warp_sum(v[j]);
    if (lane == 0)
#pragma unroll
        for (int j = 0; j < NV; ++j) red[j][warp] = v[j];
    __syncthreads();
    if (threadIdx.x == 0)
#pragma unroll
        for (int j = 0; j < NV; ++j) {
            double s = 0;
#pragma unroll
            for (int w = 0; w < NW; ++w) s += red[j][w];
            v[j] = s;
        }
}

// Block-wide sum of NV floats per thread, warp sums in FP32 (an FP64 warp butterfly is five FP64
// warp instructions, ~20 SM clocks each on GB300, per value and CTA) and the warps' sums added in
// FP64 in warp order; result valid in thread 0.
template <int NV> __device__ __forceinline__ void block_sum_f(const float (&f)[NV], double (&v)[NV], double (*red)[NW]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < NV; ++j) {
        const float s = warp_sum(f[j]);
        if (lane == 0) red[j][warp] = (double)s;
    }
    __syncthreads();
    if (threadIdx.x == 0)
#pragma unroll
        for (int j = 0; j < NV; ++j) {
            double s = 0;
#pragma unroll
            for (int w = 0; w < NW; ++w) s += red[j][w];
            v[j] = s;
        }
}

// Complex64 kernels keep their cross-CTA partial sums as double-float (two floats in the slot
// of a double): the per-CTA and last-CTA sums then run on the FP32 pipes, and a result is
// converted to double once.  A last CTA summing a few hundred FP64 partials per coefficient in
// FP64 spent ~20 SM clocks per FP64 warp instruction, about 2% of a projection launch.
__device__ __forceinline__ void store_df(double *slot, dfr v) { *reinterpret_cast<dfr *>(slot) = v; }
__device__ __forceinline__ dfr load_df(const double *slot) {
    const float2 t = __ldcg(reinterpret_cast<const float2 *>(slot));
    return dfr(t.x, t.y);
}
// As block_sum_f, with the warps' sums added in double-float and returned as such (thread 0).
template <int NV> __device__ __forceinline__ void block_sum_df(const float (&f)[NV], dfr (&v)[NV], float (*red)[NW]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < NV; ++j) {
        const float s = warp_sum(f[j]);
        if (lane == 0) red[j][warp] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0)
#pragma unroll
        for (int j = 0; j < NV; ++j) {
            dfr s(0.f, 0.f);
#pragma unroll
            for (int w = 0; w < NW; ++w) s = s + dfr(red[j][w], 0.f);
            v[j] = s;
        }
}

// Last-CTA-done protocol: returns true in every thread of the CTA that arrived last.
__device__ __forceinline__ bool arrive_last(unsigned *ticket, unsigned count) {
    __shared__ unsigned s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = (atomicAdd(ticket, 1u) == count - 1) ? 1u : 0u;
    __syncthreads();
    if (s_last) __threadfence();
    return s_last != 0;
}

// Sums NV partial vectors of length G (layout part[j*G + g]) with the whole CTA;
// result valid in thread 0.  Fixed order: deterministic for a given grid.
template <int NV> __device__ __forceinline__ void sum_partials(const double *part, int G, double (&out)[NV], double (*red)[NW]) {
#pragma unroll
    for (int j = 0; j < NV; ++j) {
        double s = 0;
        for (int g = threadIdx.x; g < G; g += NT) s += __ldcg(part + (size_t)j * G + g);
        out[j] = s;
    }
    block_sum<NV>(out, red);
}

int g_num_sms = 0;

int num_sms() {
    if (g_num_sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || g_num_sms <= 0)
            g_num_sms = 152;
    }
    return g_num_sms;
}

template <class R> __host__ __device__ constexpr int ept() { return sizeof(R) == 4 ? 8 : 4; }

// Chunks of NT*EPT elements: the per-system grid dimension of the projection, update and
// combination kernels (one chunk per CTA).  The system index is the fastest grid index, so
// the CTAs that read the same chunk of the shared vectors (W, Z) run together and the
// shared data comes from HBM once and from L2 for the other systems.
template <class R> int nchunks(int n) {
    const int ch = NT * ept<R>();
    int c = (n + ch - 1) / ch;
    return c > 0 ? c : 1;
}
// Capped per-system grid for the grid-stride kernels (norms, FP64 residual).
int capped_grid(int n, int nsys, int per_sm) {
    int chunks = (n + NT - 1) / NT;
    int target = (num_sms() * per_sm + nsys - 1) / (nsys > 0 ? nsys : 1);
    if (target < 1) target = 1;
    return chunks < target ? (chunks > 0 ? chunks : 1) : target;
}

// ----------------------------------------------------------------- finishing
// run_finish: gdmr_kernels.cuh

// ----------------------------------------------------------------- multi-dot
// A CTA owns one chunk of NT*EPT elements of one system.  Thread tid holds EPT/VEC
// packets of VEC consecutive elements, packet e at element c0 + (e*NT + tid)*VEC, so
// every load instruction of a warp covers one contiguous 32*VEC*sizeof(C)-byte span
// (VEC = 2 with complex64: 16-byte loads).
template <class C, int VEC> struct Pack {
    C v[VEC];
};
template <class C, int VEC> __device__ __forceinline__ Pack<C, VEC> load_pack(const C *p, long i0, int n) {
    Pack<C, VEC> r;
    if constexpr (VEC == 2 && std::is_same<C, float2>::value) {
      if (i0 + 1 < n) {
        const float4 f = *reinterpret_cast<const float4 *>(p + i0);
        r.v[0].x = f.x; r.v[0].y = f.y;
        r.v[VEC - 1].x = f.z; r.v[VEC - 1].y = f.w;
        return r;
      }
    }
#pragma unroll
    for (int j = 0; j < VEC; ++j) r.v[j] = (i0 + j < n) ? p[i0 + j] : czero<C>();
    return r;
}
template <class C, int VEC> __device__ __forceinline__ void store_pack(C *p, long i0, int n, const Pack<C, VEC> &r) {
    if constexpr (VEC == 2 && std::is_same<C, float2>::value) {
        if (i0 + 1 < n) {
            *reinterpret_cast<float4 *>(p + i0) = make_float4(r.v[0].x, r.v[0].y, r.v[VEC - 1].x, r.v[VEC - 1].y);
            return;
        }
    }
#pragma unroll
    for (int j = 0; j < VEC; ++j)
        if (i0 + j < n) p[i0 + j] = r.v[j];
}
// Warp sum of PU complex double-float partials as a reduce-scatter butterfly: at offsets 16, 8,
// ... each lane keeps half of its components (chosen by its lane bit) and adds the partner's
// copy of that half, so the 2*PU components take log2(2 PU) halving levels and then full
// levels for the rest, instead of 5 full levels each.  Component c = 2u + (0 re | 1 im) ends in
// the lanes whose top bits spell c; the first of them writes dst[p0 + u].
template <int PU> __device__ __forceinline__ void df_reduce_scatter(dfc (&a)[PU], dfc *dst, int p0, int q, int lane) {
    constexpr int Q = 2 * PU;
    dfr v[Q];
#pragma unroll
    for (int u = 0; u < PU; ++u) {
        v[2 * u] = a[u].x;
        v[2 * u + 1] = a[u].y;
    }
    int off = 16;
#pragma unroll
    for (int cnt = Q; cnt > 1; cnt >>= 1, off >>= 1) {
        const bool hi = (lane & off) != 0;
        const int half = cnt >> 1;
#pragma unroll
        for (int i = 0; i < half; ++i) {
            const dfr keep = hi ? v[half + i] : v[i], send = hi ? v[i] : v[half + i];
            const dfr got(__shfl_xor_sync(0xffffffffu, send.hi, off), __shfl_xor_sync(0xffffffffu, send.lo, off));
            v[i] = keep + got;
        }
    }
    for (; off > 0; off >>= 1)
        v[0] = v[0] + dfr(__shfl_xor_sync(0xffffffffu, v[0].hi, off), __shfl_xor_sync(0xffffffffu, v[0].lo, off));
    // lanes 32/Q * c hold component c
    constexpr int SPAN = 32 / Q;
    if ((lane & (SPAN - 1)) == 0) {
        const int c = lane / SPAN, u = c >> 1;
        if (p0 + u < q) {
            if (c & 1) dst[p0 + u].y = v[0];
            else dst[p0 + u].x = v[0];
        }
    }
}

template <class C> __host__ __device__ constexpr int min_blocks(int ept, int pu) {
    // double-float values carry two FP32 words per component plus two-sum temporaries
    return std::is_same<C, dfc>::value || ept * pu * (int)sizeof(C) > 128 ? 2 : 3;
}

// coef_s[p] = <B_p, w_s> for B = [segA (qa vectors) | segB_s (qb vectors)].
// Grid (systems, chunks), w in registers, PU basis vectors in flight per thread, warp
// reductions in the working precision, last CTA of each system sums the chunk partials.
// PF: the next group's basis vectors are loaded before the current group is reduced, so the
// double-float forms (about 44 FP32 operations per element and vector) keep their loads in flight.
template <class R, int EPT, int PU, int VEC, bool PF = false>
__global__ void __launch_bounds__(NT, PF ? 2 : min_blocks<typename CT<R>::t>(EPT, PU))
    k_mdot(int n, const typename CT<R>::t *__restrict__ segA, int qa, const typename CT<R>::t *__restrict__ segB0,
           size_t strideB, int qb, const typename CT<R>::t *__restrict__ w0, size_t strideW,
           const int *__restrict__ act, double2 *__restrict__ partials, int qmax, unsigned *tickets,
           double2 *__restrict__ coef0, size_t strideC, SysState *state, int skip_broken) {
    using C = typename CT<R>::t;
    constexpr int NP = EPT / VEC;
    const int slot = blockIdx.x, s = act[slot], chunk = blockIdx.y, G = gridDim.y;
    if (skip_broken && state[s].broken) return;
    const C *segB = segB0 + (size_t)s * strideB;
    const C *w = w0 + (size_t)s * strideW;
    const int q = qa + qb, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    __shared__ C wsum[NW][QMAX];
    const long c0 = (long)chunk * NT * EPT;
    Pack<C, VEC> wv[NP];
#pragma unroll
    for (int e = 0; e < NP; ++e) wv[e] = load_pack<C, VEC>(w, c0 + ((long)e * NT + tid) * VEC, n);
    Pack<C, VEC> vv[PU][NP], nx[PU][NP];
    auto load_group = [&](int g0, Pack<C, VEC>(&dst)[PU][NP]) {
#pragma unroll
        for (int u = 0; u < PU; ++u) {
            const int p = g0 + u < q ? g0 + u : q - 1;   // duplicate the last vector; its result is dropped
            const C *vp = p < qa ? segA + (size_t)p * n : segB + (size_t)(p - qa) * n;
#pragma unroll
            for (int e = 0; e < NP; ++e) dst[u][e] = load_pack<C, VEC>(vp, c0 + ((long)e * NT + tid) * VEC, n);
        }
    };
    // with no basis vectors (q = 0) the clamped index q - 1 would address 16n bytes before segA
    if constexpr (PF)
        if (q > 0) load_group(0, vv);
    for (int p0 = 0; p0 < q; p0 += PU) {
        if constexpr (PF) {
            if (p0 + PU < q) load_group(p0 + PU, nx);
        } else {
            load_group(p0, vv);
        }
        if constexpr (std::is_same<C, dfc>::value) {
            // double-float: all PU partials first, then one reduce-scatter butterfly over the
            // 2*PU real components (each lane keeps half of what it holds at every level)
            C a[PU];
#pragma unroll
            for (int u = 0; u < PU; ++u) {
                a[u] = czero<C>();
#pragma unroll
                for (int e = 0; e < NP; ++e)
#pragma unroll
                    for (int j = 0; j < VEC; ++j) cdotacc(a[u], vv[u][e].v[j], wv[e].v[j]);
            }
            df_reduce_scatter<PU>(a, &wsum[warp][0], p0, q, lane);
        } else {
#pragma unroll
            for (int u = 0; u < PU; ++u) {
                C a = czero<C>();
#pragma unroll
                for (int e = 0; e < NP; ++e)
#pragma unroll
                    for (int j = 0; j < VEC; ++j) cdotacc(a, vv[u][e].v[j], wv[e].v[j]);
                a.x = warp_sum(a.x);
                a.y = warp_sum(a.y);
                if (lane == 0 && p0 + u < q) wsum[warp][p0 + u] = a;
            }
        }
        if constexpr (PF) {
#pragma unroll
            for (int u = 0; u < PU; ++u)
#pragma unroll
                for (int e = 0; e < NP; ++e) vv[u][e] = nx[u][e];
        }
    }
    __syncthreads();
    double *part = (double *)partials + (size_t)slot * qmax * 2 * G;   // [p][re|im][G]
    constexpr bool DFP = std::is_same<C, float2>::value;   // double-float partials (complex64)
    for (int p = tid; p < q; p += NT) {
        double *pp = part + (size_t)p * 2 * G;
        if constexpr (DFP) {
            dfr re(0.f, 0.f), im(0.f, 0.f);
#pragma unroll
            for (int ww = 0; ww < NW; ++ww) {
                re = re + dfr((float)wsum[ww][p].x, 0.f);
                im = im + dfr((float)wsum[ww][p].y, 0.f);
            }
            store_df(pp + chunk, re);
            store_df(pp + G + chunk, im);
        } else {
            double re = 0, im = 0;
#pragma unroll
            for (int ww = 0; ww < NW; ++ww) { re += (double)wsum[ww][p].x; im += (double)wsum[ww][p].y; }
            pp[chunk] = re;
            pp[G + chunk] = im;
        }
    }
    if (!arrive_last(&tickets[slot], G)) return;
    // one warp per coefficient, lanes stride over the G partials (fixed order)
    double2 *coef = coef0 + (size_t)s * strideC;
    for (int p = warp; p < q; p += NW) {
        const double *pp = part + (size_t)p * 2 * G;
        if constexpr (DFP) {
            dfr re(0.f, 0.f), im(0.f, 0.f);
            for (int g = lane; g < G; g += 32) {
                re = re + load_df(pp + g);
                im = im + load_df(pp + G + g);
            }
            re = warp_sum(re);
            im = warp_sum(im);
            if (lane == 0) coef[p] = make_double2((double)re, (double)im);
        } else {
            double re = 0, im = 0;
            for (int g = lane; g < G; g += 32) { re += __ldcg(pp + g); im += __ldcg(pp + G + g); }
            re = warp_sum(re);
            im = warp_sum(im);
            if (lane == 0) coef[p] = make_double2(re, im);
        }
    }
    if (tid == 0) tickets[slot] = 0;
}

// ----------------------------------------------------------------- update + norms
template <class R, int EPT, int PU, int VEC, bool PF = false>
__global__ void __launch_bounds__(NT, PF ? 2 : min_blocks<typename CT<R>::t>(EPT, PU))
    k_update(int n, const typename CT<R>::t *__restrict__ segA, int qa, const typename CT<R>::t *__restrict__ segB0,
             size_t strideB, int qb, const typename CT<R>::t *__restrict__ w0, size_t strideW,
             typename CT<R>::t *__restrict__ out0, size_t strideO, const int *__restrict__ act,
             const double2 *__restrict__ coef0, size_t strideC, double2 *__restrict__ partials, unsigned *tickets,
             SysState *state, FinishArgs fin, int skip_broken) {
    using C = typename CT<R>::t;
    constexpr int NP = EPT / VEC;
    const int slot = blockIdx.x, s = act[slot], chunk = blockIdx.y, G = gridDim.y;
    if (skip_broken && state[s].broken) return;
    const C *segB = segB0 + (size_t)s * strideB;
    const C *w = w0 + (size_t)s * strideW;
    C *out = out0 + (size_t)s * strideO;
    const int q = qa + qb, tid = threadIdx.x;
    __shared__ C cs[QMAX];
    __shared__ double red[3][NW];
    const double2 *coef = coef0 + (size_t)s * strideC;
    for (int p = tid; p < q; p += NT) cs[p] = from_d<C>(coef[p]);
    __syncthreads();
    const long c0 = (long)chunk * NT * EPT;
    Pack<C, VEC> acc[NP], org[NP];
#pragma unroll
    for (int e = 0; e < NP; ++e) {
        org[e] = load_pack<C, VEC>(w, c0 + ((long)e * NT + tid) * VEC, n);
        acc[e] = org[e];
    }
    Pack<C, VEC> vv[PU][NP], nx[PU][NP];
    auto load_group = [&](int g0, Pack<C, VEC>(&dst)[PU][NP]) {
#pragma unroll
        for (int u = 0; u < PU; ++u) {
            const int p = g0 + u < q ? g0 + u : q - 1;
            const C *vp = p < qa ? segA + (size_t)p * n : segB + (size_t)(p - qa) * n;
#pragma unroll
            for (int e = 0; e < NP; ++e) dst[u][e] = load_pack<C, VEC>(vp, c0 + ((long)e * NT + tid) * VEC, n);
        }
    };
    if constexpr (PF) {
        if (q > 0) load_group(0, vv);
    }
    for (int p0 = 0; p0 < q; p0 += PU) {
        if constexpr (PF) {
            if (p0 + PU < q) load_group(p0 + PU, nx);
        } else {
            load_group(p0, vv);
        }
#pragma unroll
        for (int u = 0; u < PU; ++u) {
            if (p0 + u < q) {
                const C c = cs[p0 + u];
#pragma unroll
                for (int e = 0; e < NP; ++e)
#pragma unroll
                    for (int j = 0; j < VEC; ++j) cfms(acc[e].v[j], c, vv[u][e].v[j]);
            }
        }
        if constexpr (std::is_same<C, dfc>::value) {   // keep double-float chains short
#pragma unroll
            for (int e = 0; e < NP; ++e)
#pragma unroll
                for (int j = 0; j < VEC; ++j) acc[e].v[j] = canon(acc[e].v[j]);
        }
        if constexpr (PF) {
#pragma unroll
            for (int u = 0; u < PU; ++u)
#pragma unroll
                for (int e = 0; e < NP; ++e) vv[u][e] = nx[u][e];
        }
    }
    C ln = czero<C>(), lc = czero<C>();
#pragma unroll
    for (int e = 0; e < NP; ++e) {
#pragma unroll
        for (int j = 0; j < VEC; ++j) acc[e].v[j] = canon(acc[e].v[j]);
        store_pack<C, VEC>(out, c0 + ((long)e * NT + tid) * VEC, n, acc[e]);
#pragma unroll
        for (int j = 0; j < VEC; ++j) {
            cdotacc(ln, acc[e].v[j], acc[e].v[j]);
            cdotacc(lc, acc[e].v[j], org[e].v[j]);
        }
    }
    double *part = (double *)partials + (size_t)slot * 3 * G;
    if constexpr (std::is_same<C, float2>::value) {
        // double-float partials, summed on the FP32 pipes
        __shared__ float redf[3][NW];
        const float f[3] = {ln.x, lc.x, lc.y};
        dfr v[3];
        block_sum_df<3>(f, v, redf);
        if (tid == 0) {
            store_df(part + chunk, v[0]);
            store_df(part + G + chunk, v[1]);
            store_df(part + 2 * G + chunk, v[2]);
        }
        if (!arrive_last(&tickets[slot], G)) return;
        const int lane = tid & 31, warp = tid >> 5;
        __shared__ dfr tw[3][NW];
        dfr a[3] = {dfr(0.f, 0.f), dfr(0.f, 0.f), dfr(0.f, 0.f)};
        for (int g = tid; g < G; g += NT)
#pragma unroll
            for (int j = 0; j < 3; ++j) a[j] = a[j] + load_df(part + (size_t)j * G + g);
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            a[j] = warp_sum(a[j]);
            if (lane == 0) tw[j][warp] = a[j];
        }
        __syncthreads();
        if (tid == 0) {
            double tot[3];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                dfr t(0.f, 0.f);
#pragma unroll
                for (int w = 0; w < NW; ++w) t = t + tw[j][w];
                tot[j] = (double)t;
            }
            run_finish(fin, s, state[s], tot[0], tot[1], tot[2]);
            tickets[slot] = 0;
        }
    } else {
        double v[3] = {(double)ln.x, (double)lc.x, (double)lc.y};
        block_sum<3>(v, red);
        if (tid == 0) {
            part[chunk] = v[0];
            part[G + chunk] = v[1];
            part[2 * G + chunk] = v[2];
        }
        if (!arrive_last(&tickets[slot], G)) return;
        double tot[3];
        __syncthreads();
        sum_partials<3>(part, G, tot, red);
        if (tid == 0) {
            run_finish(fin, s, state[s], tot[0], tot[1], tot[2]);
            tickets[slot] = 0;
        }
    }
}

// ----------------------------------------------------------------- persistent Gram-Schmidt
// The two Gram-Schmidt kernels for a few systems at 16 bytes an element (complex128, double-
// float): grid (systems, G) with about two CTAs per SM in all, each CTA striding over the
// element chunks of NT x EPT.  A projection group of PU basis vectors accumulates over every
// chunk of its CTA before its one warp reduction, and the update's norm and cross term are
// summed once per CTA.  In the chunked kernels above, one CTA per chunk, those reductions came
// once per 4 elements a thread: the double-float warp butterflies and the FP64 block sums
// (one FP64 warp instruction is ~64 clocks of a scheduler on GB300) were about half of the
// double-float projection's 93 instructions per complex multiply-add.
inline int persist_grid(int n, int ept, int nsys) {
    const long nch = ((long)n + (long)NT * ept - 1) / ((long)NT * ept);
    long G = (2L * num_sms() + nsys - 1) / nsys;
    if (G > nch) G = nch;
    return G < 1 ? 1 : (int)G;
}

template <class R, int EPT, int PU, bool PF = false>
__global__ void __launch_bounds__(NT, 2)
    k_mdot_persist(int n, const typename CT<R>::t *__restrict__ segA, int qa,
                   const typename CT<R>::t *__restrict__ segB0, size_t strideB, int qb,
                   const typename CT<R>::t *__restrict__ w0, size_t strideW, const int *__restrict__ act,
                   double2 *__restrict__ partials, int qmax, unsigned *tickets, double2 *__restrict__ coef0,
                   size_t strideC, SysState *state, int skip_broken) {
    using C = typename CT<R>::t;
    const int slot = blockIdx.x, s = act[slot], G = gridDim.y;
    if (skip_broken && state[s].broken) return;
    const C *segB = segB0 + (size_t)s * strideB;
    const C *w = w0 + (size_t)s * strideW;
    const int q = qa + qb, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    __shared__ C wsum[NW][QMAX];
    const long span = (long)NT * EPT, nch = ((long)n + span - 1) / span;
    for (int p0 = 0; p0 < q; p0 += PU) {
        const C *vp[PU];
#pragma unroll
        for (int u = 0; u < PU; ++u) {
            const int p = p0 + u < q ? p0 + u : q - 1;   // duplicate the last vector; its result is dropped
            vp[u] = p < qa ? segA + (size_t)p * n : segB + (size_t)(p - qa) * n;
        }
        C a[PU];
#pragma unroll
        for (int u = 0; u < PU; ++u) a[u] = czero<C>();
        C wv[EPT], vv[PU][EPT];
        auto load = [&](long ch, C(&wd)[EPT], C(&vd)[PU][EPT]) {
            const long c0 = ch * span + tid;
#pragma unroll
            for (int e = 0; e < EPT; ++e) wd[e] = c0 + (long)e * NT < n ? w[c0 + (long)e * NT] : czero<C>();
#pragma unroll
            for (int u = 0; u < PU; ++u)
#pragma unroll
                for (int e = 0; e < EPT; ++e) vd[u][e] = c0 + (long)e * NT < n ? vp[u][c0 + (long)e * NT] : czero<C>();
        };
        if constexpr (PF)
            if (blockIdx.y < nch) load(blockIdx.y, wv, vv);
        for (long ch = blockIdx.y; ch < nch; ch += G) {
            C wn[PF ? EPT : 1], vn[PF ? PU : 1][PF ? EPT : 1];
            if constexpr (PF) {   // the next chunk's loads go out before this chunk's arithmetic
                if (ch + G < nch) load(ch + G, wn, vn);
            } else {
                load(ch, wv, vv);
            }
#pragma unroll
            for (int u = 0; u < PU; ++u) {
#pragma unroll
                for (int e = 0; e < EPT; ++e) cdotacc(a[u], vv[u][e], wv[e]);
                a[u] = canon(a[u]);
            }
            if constexpr (PF) {
#pragma unroll
                for (int e = 0; e < EPT; ++e) wv[e] = wn[e];
#pragma unroll
                for (int u = 0; u < PU; ++u)
#pragma unroll
                    for (int e = 0; e < EPT; ++e) vv[u][e] = vn[u][e];
            }
        }
        if constexpr (std::is_same<C, dfc>::value) {
            df_reduce_scatter<PU>(a, &wsum[warp][0], p0, q, lane);
        } else {
#pragma unroll
            for (int u = 0; u < PU; ++u) {
                a[u].x = warp_sum(a[u].x);
                a[u].y = warp_sum(a[u].y);
                if (lane == 0 && p0 + u < q) wsum[warp][p0 + u] = a[u];
            }
        }
    }
    __syncthreads();
    const int chunk = blockIdx.y;
    double *part = (double *)partials + (size_t)slot * qmax * 2 * G;   // [p][re|im][G]
    for (int p = tid; p < q; p += NT) {
        double re = 0, im = 0;
#pragma unroll
        for (int ww = 0; ww < NW; ++ww) { re += (double)wsum[ww][p].x; im += (double)wsum[ww][p].y; }
        double *pp = part + (size_t)p * 2 * G;
        pp[chunk] = re;
        pp[G + chunk] = im;
    }
    if (!arrive_last(&tickets[slot], G)) return;
    double2 *coef = coef0 + (size_t)s * strideC;
    for (int p = warp; p < q; p += NW) {
        const double *pp = part + (size_t)p * 2 * G;
        double re = 0, im = 0;
        for (int g = lane; g < G; g += 32) { re += __ldcg(pp + g); im += __ldcg(pp + G + g); }
        re = warp_sum(re);
        im = warp_sum(im);
        if (lane == 0) coef[p] = make_double2(re, im);
    }
    if (tid == 0) tickets[slot] = 0;
}

template <class R, int EPT, int PU, bool PF = false>
__global__ void __launch_bounds__(NT, 2)
    k_update_persist(int n, const typename CT<R>::t *__restrict__ segA, int qa,
                     const typename CT<R>::t *__restrict__ segB0, size_t strideB, int qb,
                     const typename CT<R>::t *__restrict__ w0, size_t strideW, typename CT<R>::t *__restrict__ out0,
                     size_t strideO, const int *__restrict__ act, const double2 *__restrict__ coef0, size_t strideC,
                     double2 *__restrict__ partials, unsigned *tickets, SysState *state, FinishArgs fin,
                     int skip_broken) {
    using C = typename CT<R>::t;
    const int slot = blockIdx.x, s = act[slot], G = gridDim.y;
    if (skip_broken && state[s].broken) return;
    const C *segB = segB0 + (size_t)s * strideB;
    const C *w = w0 + (size_t)s * strideW;
    C *out = out0 + (size_t)s * strideO;
    const int q = qa + qb, tid = threadIdx.x;
    __shared__ C cs[QMAX];
    __shared__ double red[3][NW];
    const double2 *coef = coef0 + (size_t)s * strideC;
    for (int p = tid; p < q; p += NT) cs[p] = from_d<C>(coef[p]);
    __syncthreads();
    const long span = (long)NT * EPT, nch = ((long)n + span - 1) / span;
    C ln = czero<C>(), lc = czero<C>();
    for (long ch = blockIdx.y; ch < nch; ch += G) {
        const long c0 = ch * span + tid;
        C org[EPT], acc[EPT];
#pragma unroll
        for (int e = 0; e < EPT; ++e) {
            org[e] = c0 + (long)e * NT < n ? w[c0 + (long)e * NT] : czero<C>();
            acc[e] = org[e];
        }
        C vv[PU][EPT];
        auto load = [&](int g0, C(&vd)[PU][EPT]) {
#pragma unroll
            for (int u = 0; u < PU; ++u) {
                const int p = g0 + u < q ? g0 + u : q - 1;
                const C *vp = p < qa ? segA + (size_t)p * n : segB + (size_t)(p - qa) * n;
#pragma unroll
                for (int e = 0; e < EPT; ++e) vd[u][e] = c0 + (long)e * NT < n ? vp[c0 + (long)e * NT] : czero<C>();
            }
        };
        // an update with no basis vectors (q = 0: the deflation loop's first vector) loads
        // nothing; the clamped index q - 1 would address 16n bytes before segA
        if constexpr (PF)
            if (q > 0) load(0, vv);
        for (int p0 = 0; p0 < q; p0 += PU) {
            C vn[PF ? PU : 1][PF ? EPT : 1];
            if constexpr (PF) {   // the next group's loads go out before this group's arithmetic
                if (p0 + PU < q) load(p0 + PU, vn);
            } else {
                load(p0, vv);
            }
#pragma unroll
            for (int u = 0; u < PU; ++u) {
                if (p0 + u < q) {
                    const C c = cs[p0 + u];
#pragma unroll
                    for (int e = 0; e < EPT; ++e) cfms(acc[e], c, vv[u][e]);
                }
            }
            if constexpr (std::is_same<C, dfc>::value) {   // keep double-float chains short
#pragma unroll
                for (int e = 0; e < EPT; ++e) acc[e] = canon(acc[e]);
            }
            if constexpr (PF) {
#pragma unroll
                for (int u = 0; u < PU; ++u)
#pragma unroll
                    for (int e = 0; e < EPT; ++e) vv[u][e] = vn[u][e];
            }
        }
#pragma unroll
        for (int e = 0; e < EPT; ++e) {
            acc[e] = canon(acc[e]);
            if (c0 + (long)e * NT < n) out[c0 + (long)e * NT] = acc[e];
            cdotacc(ln, acc[e], acc[e]);
            cdotacc(lc, acc[e], org[e]);
        }
        ln = canon(ln);
        lc = canon(lc);
    }
    double v[3] = {(double)ln.x, (double)lc.x, (double)lc.y};
    block_sum<3>(v, red);
    const int chunk = blockIdx.y;
    double *part = (double *)partials + (size_t)slot * 3 * G;
    if (tid == 0) {
        part[chunk] = v[0];
        part[G + chunk] = v[1];
        part[2 * G + chunk] = v[2];
    }
    if (!arrive_last(&tickets[slot], G)) return;
    double tot[3];
    __syncthreads();
    sum_partials<3>(part, G, tot, red);
    if (tid == 0) {
        run_finish(fin, s, state[s], tot[0], tot[1], tot[2]);
        tickets[slot] = 0;
    }
}

// ----------------------------------------------------------------- bulk-copy Gram-Schmidt (double-float)
// The double-float projection and update as copy/compute pipelines: one CTA per SM, a producer
// warp streams 8 KB vector tiles (512 complex double-float elements) into shared memory with
// cp.async.bulk (the TMA engine, no tensor map), and eight consumer warps compute from shared
// memory behind "full"/"empty" mbarriers.  The register-tiled kernels above issue their loads
// and then wait for them (ncu: 3.3 long-scoreboard stalls per issue); here 4-5 stages (~160 KB)
// are in flight per SM while the consumers work (0.5 long-scoreboard stalls per issue).
// Measured on the 96^3 plain fp64e solve (8 vectors): 38.8 us against 32.7 us for the
// persistent register-tiled projection, 63 against 45 us for the update; the consumers'
// double-float arithmetic (44 FP32 instructions per complex multiply-add) issues at ~39% with
// 2 warps a scheduler, and 16 consumer warps measured slower still (42.8 us).  They stay as
// tuner candidates.  Every mbarrier wait is bounded (about two seconds
// of clock): a timeout is counted in g_bulk_timeouts, the kernel stops issuing and consuming,
// and the producer waits (bounded) for the copies it issued before the CTA exits.
constexpr int BK_TILE = 512;                   // elements per vector tile (8 KB)
constexpr int BK_CONS = 256;                   // consumer threads, 8 warps; warp 8 produces
constexpr int BK_CW = BK_CONS / 32;            // consumer warps
constexpr int BK_THREADS = BK_CONS + 32;
constexpr int BK_EPT = BK_TILE / BK_CONS;      // elements per consumer thread and tile
constexpr int BK_PU = 4;                       // vector tiles per stage
constexpr int BK_MSTAGES = 4, BK_USTAGES = 5;
constexpr long long BK_WAIT_CYCLES = 4000000000LL;   // drain waits: ~2 s at 2 GHz, fixed
__device__ unsigned g_bulk_timeouts = 0;
// stage waits and grid barriers: the process's wait limit (set_wait_limit_ms), in clock cycles
__constant__ long long c_wait_cycles = BK_WAIT_CYCLES;

__device__ __forceinline__ uint32_t bk_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void bk_init(uint32_t a, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ void bk_arrive(uint32_t a) {
    asm volatile("{\n.reg .b64 st;\nmbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(a) : "memory");
}
__device__ __forceinline__ void bk_arrive_tx(uint32_t a, uint32_t bytes) {
    asm volatile("{\n.reg .b64 st;\nmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}\n" ::"r"(a), "r"(bytes)
                 : "memory");
}
// global -> shared bulk copy: 16-byte aligned addresses, size a multiple of 16
__device__ __forceinline__ void bk_copy(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}
__device__ __forceinline__ bool bk_wait(uint32_t a, uint32_t parity, volatile int *abort, long long limit) {
    const long long t0 = clock64();
    while (true) {
        uint32_t ok;
        asm volatile("{\n.reg .pred P;\nmbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\nselp.b32 %0, 1, 0, P;\n}\n"
                     : "=r"(ok) : "r"(a), "r"(parity) : "memory");
        if (ok) return true;
        if ((abort && *abort) || clock64() - t0 > limit) return false;
    }
}
// lane 0 waits, the warp follows its verdict; a timeout raises the CTA's abort flag
__device__ __forceinline__ bool bk_warp_wait(uint32_t a, uint32_t parity, volatile int *abort, int lane) {
    int ok = 1;
    if (lane == 0) {
        ok = bk_wait(a, parity, abort, c_wait_cycles);
        if (!ok && !*abort) {
            atomicAdd(&g_bulk_timeouts, 1u);
            *abort = 1;
        }
    }
    return __shfl_sync(0xffffffffu, ok, 0) != 0;
}
// Sum of three doubles over the warps of a pipeline CTA; the result is valid in thread 0.
__device__ __forceinline__ void bk_block_sum3(double (&v)[3], double (*red)[BK_CW + 1]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < 3; ++j) v[j] = warp_sum(v[j]);
    if (lane == 0)
#pragma unroll
        for (int j = 0; j < 3; ++j) red[j][warp] = v[j];
    __syncthreads();
    if (threadIdx.x == 0)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            double t = 0;
            for (int ww = 0; ww < BK_CW + 1; ++ww) t += red[j][ww];
            v[j] = t;
        }
}
__host__ __device__ constexpr size_t bk_mdot_smem() { return (size_t)BK_MSTAGES * (BK_PU + 1) * BK_TILE * sizeof(dfc); }
__host__ __device__ constexpr size_t bk_update_smem() { return (size_t)BK_USTAGES * BK_PU * BK_TILE * sizeof(dfc); }

// The producer's side of a pipeline over `total` stages: stage k goes to buffer k % NS after
// the consumers released that buffer's previous use; items(k, j) gives the source of tile j of
// stage k (nullptr: no tile) and bytes(k) the size of every tile of the stage.  Afterwards it
// waits for the last use of each buffer, so no copy is in flight when the CTA exits.
template <int NS, int PER, class Items, class Bytes>
__device__ void bk_produce(long total, unsigned char *base, unsigned long long *full, unsigned long long *empty,
                           volatile int *abort, Items items, Bytes bytes) {
    long last[NS];
#pragma unroll
    for (int b = 0; b < NS; ++b) last[b] = -1;
    for (long k = 0; k < total && !*abort; ++k) {
        const int b = (int)(k % NS);
        const long use = k / NS;
        if (use > 0 && !bk_wait(bk_u32(&empty[b]), (uint32_t)((use - 1) & 1), abort, c_wait_cycles)) {
            if (!*abort) { atomicAdd(&g_bulk_timeouts, 1u); *abort = 1; }
            break;
        }
        const uint32_t nb = bytes(k);
        int cnt = 0;
#pragma unroll
        for (int j = 0; j < PER; ++j) cnt += items(k, j) != nullptr;
        bk_arrive_tx(bk_u32(&full[b]), nb * cnt);
#pragma unroll
        for (int j = 0; j < PER; ++j) {
            const void *src = items(k, j);
            if (src) bk_copy(bk_u32(base + ((size_t)b * PER + j) * BK_TILE * sizeof(dfc)), src, nb, bk_u32(&full[b]));
        }
        last[b] = use;
    }
#pragma unroll
    for (int b = 0; b < NS; ++b)
        if (last[b] >= 0 && !bk_wait(bk_u32(&full[b]), (uint32_t)(last[b] & 1), nullptr, BK_WAIT_CYCLES))
            atomicAdd(&g_bulk_timeouts, 1u);   // drain: the fixed bound, whatever the process limit
}

__global__ void __launch_bounds__(BK_THREADS, 1)
    k_mdot_bulk(int n, const dfc *__restrict__ segA, int qa, const dfc *__restrict__ segB0, size_t strideB, int qb,
                const dfc *__restrict__ w0, size_t strideW, const int *__restrict__ act, double2 *__restrict__ partials,
                int qmax, unsigned *tickets, double2 *__restrict__ coef0, size_t strideC, SysState *state,
                int skip_broken) {
    extern __shared__ __align__(128) unsigned char bk_sm[];
    __shared__ __align__(8) unsigned long long full[BK_MSTAGES], empty[BK_MSTAGES];
    __shared__ int s_abort;
    __shared__ dfc wsum[BK_CW][QMAX];
    const int slot = blockIdx.x, s = act[slot], G = gridDim.y, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (skip_broken && state[s].broken) return;
    const dfc *segB = segB0 + (size_t)s * strideB;
    const dfc *w = w0 + (size_t)s * strideW;
    const int q = qa + qb, ngroups = (q + BK_PU - 1) / BK_PU;
    const long ntiles = ((long)n + BK_TILE - 1) / BK_TILE;
    const long my = blockIdx.y < ntiles ? (ntiles - blockIdx.y + G - 1) / G : 0;   // tiles of this CTA
    const long total = (long)ngroups * my;                                         // stages, group-major
    if (tid == 0) {
        for (int b = 0; b < BK_MSTAGES; ++b) {
            bk_init(bk_u32(&full[b]), 1);
            bk_init(bk_u32(&empty[b]), BK_CW);
        }
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    auto vec = [&](int p) { return p < qa ? segA + (size_t)p * n : segB + (size_t)(p - qa) * n; };
    if (warp == BK_CW) {
        if (lane == 0)
            bk_produce<BK_MSTAGES, BK_PU + 1>(
                total, bk_sm, full, empty, &s_abort,
                [&](long k, int j) -> const void * {
                    const int g = (int)(k / my);
                    const long e0 = (blockIdx.y + (k % my) * G) * (long)BK_TILE;
                    if (j == 0) return w + e0;
                    const int p = g * BK_PU + j - 1;
                    return vec(p < q ? p : q - 1) + e0;   // the last group repeats the last vector
                },
                [&](long k) -> uint32_t {
                    const long e0 = (blockIdx.y + (k % my) * G) * (long)BK_TILE;
                    return (uint32_t)((n - e0 < BK_TILE ? n - e0 : BK_TILE) * sizeof(dfc));
                });
    } else {
        bool ok = true;
        for (int g = 0; g < ngroups && ok; ++g) {
            dfc a[BK_PU];
#pragma unroll
            for (int u = 0; u < BK_PU; ++u) a[u] = czero<dfc>();
            for (long i = 0; i < my; ++i) {
                const long k = (long)g * my + i;
                const int b = (int)(k % BK_MSTAGES);
                if (!bk_warp_wait(bk_u32(&full[b]), (uint32_t)((k / BK_MSTAGES) & 1), &s_abort, lane)) { ok = false; break; }
                const dfc *st = reinterpret_cast<const dfc *>(bk_sm) + (size_t)b * (BK_PU + 1) * BK_TILE;
                const long e0 = (blockIdx.y + i * G) * (long)BK_TILE;
#pragma unroll
                for (int e = 0; e < BK_EPT; ++e) {
                    const int idx = e * BK_CONS + tid;
                    if (e0 + idx < n) {
                        const dfc wv = st[idx];
#pragma unroll
                        for (int u = 0; u < BK_PU; ++u) cdotacc(a[u], st[(size_t)(u + 1) * BK_TILE + idx], wv);
                    }
                }
                __syncwarp();
                if (lane == 0) bk_arrive(bk_u32(&empty[b]));
#pragma unroll
                for (int u = 0; u < BK_PU; ++u) a[u] = canon(a[u]);
            }
            if (ok) df_reduce_scatter<BK_PU>(a, &wsum[warp][0], g * BK_PU, q, lane);
        }
    }
    __syncthreads();
    const int chunk = blockIdx.y;
    double *part = (double *)partials + (size_t)slot * qmax * 2 * G;   // [p][re|im][G]
    for (int p = tid; p < q; p += blockDim.x) {
        double re = 0, im = 0;
#pragma unroll
        for (int ww = 0; ww < BK_CW; ++ww) { re += (double)wsum[ww][p].x; im += (double)wsum[ww][p].y; }
        double *pp = part + (size_t)p * 2 * G;
        pp[chunk] = re;
        pp[G + chunk] = im;
    }
    if (!arrive_last(&tickets[slot], G)) return;
    double2 *coef = coef0 + (size_t)s * strideC;
    for (int p = warp; p < q; p += BK_CW + 1) {
        const double *pp = part + (size_t)p * 2 * G;
        double re = 0, im = 0;
        for (int g = lane; g < G; g += 32) { re += __ldcg(pp + g); im += __ldcg(pp + G + g); }
        re = warp_sum(re);
        im = warp_sum(im);
        if (lane == 0) coef[p] = make_double2(re, im);
    }
    if (tid == 0) tickets[slot] = 0;
}

__global__ void __launch_bounds__(BK_THREADS, 1)
    k_update_bulk(int n, const dfc *__restrict__ segA, int qa, const dfc *__restrict__ segB0, size_t strideB, int qb,
                  const dfc *__restrict__ w0, size_t strideW, dfc *__restrict__ out0, size_t strideO,
                  const int *__restrict__ act, const double2 *__restrict__ coef0, size_t strideC,
                  double2 *__restrict__ partials, unsigned *tickets, SysState *state, FinishArgs fin,
                  int skip_broken) {
    extern __shared__ __align__(128) unsigned char bk_sm[];
    __shared__ __align__(8) unsigned long long full[BK_USTAGES], empty[BK_USTAGES];
    __shared__ int s_abort;
    __shared__ dfc cs[QMAX];
    __shared__ double red9[3][BK_CW + 1];
    const int slot = blockIdx.x, s = act[slot], G = gridDim.y, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (skip_broken && state[s].broken) return;
    const dfc *segB = segB0 + (size_t)s * strideB;
    const dfc *w = w0 + (size_t)s * strideW;
    dfc *out = out0 + (size_t)s * strideO;
    const int q = qa + qb, per_tile = (q + 1 + BK_PU - 1) / BK_PU;   // stages per tile: [w, v_0 .. v_q-1]
    const long ntiles = ((long)n + BK_TILE - 1) / BK_TILE;
    const long my = blockIdx.y < ntiles ? (ntiles - blockIdx.y + G - 1) / G : 0;
    const long total = (long)per_tile * my;                                        // stages, tile-major
    const double2 *coef = coef0 + (size_t)s * strideC;
    for (int p = tid; p < q; p += blockDim.x) cs[p] = from_d<dfc>(coef[p]);
    if (tid == 0) {
        for (int b = 0; b < BK_USTAGES; ++b) {
            bk_init(bk_u32(&full[b]), 1);
            bk_init(bk_u32(&empty[b]), BK_CW);
        }
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    dfc ln = czero<dfc>(), lc = czero<dfc>();
    if (warp == BK_CW) {
        if (lane == 0)
            bk_produce<BK_USTAGES, BK_PU>(
                total, bk_sm, full, empty, &s_abort,
                [&](long k, int j) -> const void * {
                    const long e0 = (blockIdx.y + (k / per_tile) * G) * (long)BK_TILE;
                    const int li = (int)(k % per_tile) * BK_PU + j;   // 0: w, 1 + p: v_p
                    if (li > q) return nullptr;
                    if (li == 0) return w + e0;
                    const int p = li - 1;
                    return (p < qa ? segA + (size_t)p * n : segB + (size_t)(p - qa) * n) + e0;
                },
                [&](long k) -> uint32_t {
                    const long e0 = (blockIdx.y + (k / per_tile) * G) * (long)BK_TILE;
                    return (uint32_t)((n - e0 < BK_TILE ? n - e0 : BK_TILE) * sizeof(dfc));
                });
    } else {
        bool ok = true;
        for (long i = 0; i < my && ok; ++i) {
            const long e0 = (blockIdx.y + i * G) * (long)BK_TILE;
            dfc org[BK_EPT], acc[BK_EPT];
            for (int c = 0; c < per_tile; ++c) {
                const long k = i * per_tile + c;
                const int b = (int)(k % BK_USTAGES);
                if (!bk_warp_wait(bk_u32(&full[b]), (uint32_t)((k / BK_USTAGES) & 1), &s_abort, lane)) { ok = false; break; }
                const dfc *st = reinterpret_cast<const dfc *>(bk_sm) + (size_t)b * BK_PU * BK_TILE;
#pragma unroll
                for (int j = 0; j < BK_PU; ++j) {
                    const int li = c * BK_PU + j;
                    if (li > q) break;
#pragma unroll
                    for (int e = 0; e < BK_EPT; ++e) {
                        const dfc v = st[(size_t)j * BK_TILE + e * BK_CONS + tid];
                        if (li == 0) {
                            org[e] = v;
                            acc[e] = v;
                        } else {
                            cfms(acc[e], cs[li - 1], v);
                        }
                    }
                }
                __syncwarp();
                if (lane == 0) bk_arrive(bk_u32(&empty[b]));
#pragma unroll
                for (int e = 0; e < BK_EPT; ++e) acc[e] = canon(acc[e]);
            }
            if (!ok) break;
#pragma unroll
            for (int e = 0; e < BK_EPT; ++e) {
                const long idx = e0 + e * BK_CONS + tid;
                if (idx < n) {
                    out[idx] = acc[e];
                    cdotacc(ln, acc[e], acc[e]);
                    cdotacc(lc, acc[e], org[e]);
                }
            }
            ln = canon(ln);
            lc = canon(lc);
        }
    }
    double v[3] = {(double)ln.x, (double)lc.x, (double)lc.y};   // the producer warp adds zeros
    bk_block_sum3(v, red9);
    const int chunk = blockIdx.y;
    double *part = (double *)partials + (size_t)slot * 3 * G;
    if (tid == 0) {
        part[chunk] = v[0];
        part[G + chunk] = v[1];
        part[2 * G + chunk] = v[2];
    }
    if (!arrive_last(&tickets[slot], G)) return;
    double tot[3] = {0, 0, 0};
    if (tid < BK_CONS)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            for (int g = tid; g < G; g += BK_CONS) tot[j] += __ldcg(part + (size_t)j * G + g);
    bk_block_sum3(tot, red9);
    if (tid == 0) {
        run_finish(fin, s, state[s], tot[0], tot[1], tot[2]);
        tickets[slot] = 0;
    }
}

// ----------------------------------------------------------------- fused Krylov loop, one small system
// The whole Krylov loop of a restart cycle for one system with a SELL operator and n <= 32 x
// (CTAs that fit on the device at once), in one cooperative launch.  For small n the
// per-step kernels (operator, projection, update, scaling: four launches with a last-CTA
// reduction each) are latency: 53 us a step on the 64 x 64 Helmholtz operator, where the data
// of a step is ~3 MB.  Here CTA b owns rows 32b .. 32b+31 (one SELL slice); warp 0 applies the
// operator to them, the eight warps split the basis vectors of the projection and the update,
// and four grid barriers a step exchange the CTAs' partial sums:
//   projection partials -> | CTA p mod G sums coefficient p -> | update, norm partials -> |
//   every CTA sums the norms in the same order, CTA 0 runs the step's finish (H column,
//   breakdown test), all scale their rows into V_j -> | next step.
// Values other CTAs wrote in this launch are read with ld.global.cg (L2), never from L1.  The
// barrier is a monotonic counter (zeroed before the launch); its wait is bounded (about two
// seconds of clock), and a timeout is counted in g_bulk_timeouts and ends every CTA's loop.
constexpr int KS_THREADS = 256;
constexpr int KS_WARPS = KS_THREADS / 32;
constexpr int KS_PCHUNK = 64;   // projection products staged in shared memory per round

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}
// Grid barrier: the CTA's writes are ordered before thread 0's release increment by the block
// barrier (cumulativity), and its acquire loads order what the CTA reads after the closing block
// barrier, so no separate full fences are needed.
__device__ bool ks_grid_sync(unsigned *bar, unsigned target, int *abort) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("red.release.gpu.global.add.u32 [%0], 1;\n" ::"l"(bar) : "memory");
        const long long t0 = clock64();
        int ok = 1;
        while (ld_acquire_gpu(bar) < target) {
            if (*(volatile int *)abort) { ok = 0; break; }
            if (clock64() - t0 > c_wait_cycles) {
                atomicAdd(&g_bulk_timeouts, 1u);
                atomicExch(abort, 1);
                ok = 0;
                break;
            }
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}
template <class C> __device__ __forceinline__ C ldcg_c(const C *p);
template <> __device__ __forceinline__ double2 ldcg_c<double2>(const double2 *p) { return __ldcg(p); }
template <> __device__ __forceinline__ float2 ldcg_c<float2>(const float2 *p) { return __ldcg(p); }
template <> __device__ __forceinline__ dfc ldcg_c<dfc>(const dfc *p) {
    const float4 f = __ldcg(reinterpret_cast<const float4 *>(p));
    dfc c;
    c.x = dfr(f.x, f.y);
    c.y = dfr(f.z, f.w);
    return c;
}
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ dfc csub(dfc a, dfc b) {
    dfc r;
    r.x = a.x - b.x;
    r.y = a.y - b.y;
    return r;
}

template <class R> struct KrylovSmallArgs {
    using C = typename CT<R>::t;
    int n, kk, m, compat_eye, qmax;
    double tol;
    const int *slice_ptr, *cols;
    const C *vals;
    const C *W;
    C *V0;                  // basis of system 0; system s at V0 + s * strideV
    size_t strideV;
    const int *act;         // act[0]: the system
    SysState *state;
    double2 *H0;            // system s at H0 + s * strideH
    size_t strideH;
    double2 *coef0;         // system s at coef0 + s * strideC
    size_t strideC;
    double *part;           // G x qmax x 2 projection partials
    double *npart;          // G x 3 norm partials
    unsigned *bar;          // [0] barrier counter (zeroed before the launch), [1] abort flag
};

template <class R>
__global__ void __launch_bounds__(KS_THREADS) k_krylov_small(KrylovSmallArgs<R> a) {
    using C = typename CT<R>::t;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, b = blockIdx.x, G = gridDim.x;
    const int s = a.act[0], n = a.n, kk = a.kk, row = 32 * b + lane;
    C *V = a.V0 + (size_t)s * a.strideV;
    double2 *coef = a.coef0 + (size_t)s * a.strideC;
    SysState *st = a.state + s;
    int *abort = reinterpret_cast<int *>(a.bar + 1);
    __shared__ C ys[32], ws[32], upd[KS_WARPS][32], prod[KS_PCHUNK][32];
    __shared__ double red[3];
    unsigned k = 0;   // barriers passed
    for (int j = 1; j <= a.m - kk; ++j) {
        const int q = kk + j;
        // (1) y = A v_{j-1} on the CTA's slice; v_{j-1} comes from every CTA: read through L2
        if (warp == 0) {
            C acc = czero<C>();
            if (row < n) {
                const int beg = a.slice_ptr[b], width = (a.slice_ptr[b + 1] - beg) >> 5;
                const C *x = V + (size_t)(j - 1) * n;
                for (int e = 0; e < width; ++e) {
                    const int idx = beg + e * 32 + lane;
                    cfma(acc, a.vals[idx], ldcg_c(x + a.cols[idx]));
                    if constexpr (std::is_same<C, dfc>::value)
                        if ((e & 3) == 3) acc = canon(acc);
                }
            }
            ys[lane] = canon(acc);
        }
        __syncthreads();
        // (2) projection partials <B_p, y> over the slice: warp w forms the 32 products of
        // p = w, w + 8, ... into shared memory, then thread p sums its 32 in order (a warp
        // butterfly would repeat every add in 32 lanes, at GB300's FP64 rate the bulk of a step)
        for (int p0 = 0; p0 < q; p0 += KS_PCHUNK) {
            const int pe = min(q, p0 + KS_PCHUNK);
            for (int p = p0 + warp; p < pe; p += KS_WARPS) {
                const C *B = p < kk ? a.W + (size_t)p * n : V + (size_t)(p - kk) * n;
                C acc = czero<C>();
                if (row < n) cdotacc(acc, B[row], ys[lane]);
                prod[p - p0][lane] = canon(acc);
            }
            __syncthreads();
            for (int p = p0 + tid; p < pe; p += KS_THREADS) {
                C acc = czero<C>();
                for (int l = 0; l < 32; ++l) {
                    const C v = prod[p - p0][l];
                    acc.x = acc.x + v.x;
                    acc.y = acc.y + v.y;
                }
                a.part[((size_t)b * a.qmax + p) * 2] = (double)acc.x;
                a.part[((size_t)b * a.qmax + p) * 2 + 1] = (double)acc.y;
            }
            __syncthreads();
        }
        if (!ks_grid_sync(a.bar, (++k) * G, abort)) return;
        // (3) coefficient p summed over the CTAs by CTA p mod G (fixed order: lanes stride, butterfly)
        if (warp == 0)
            for (int p = b; p < q; p += G) {
                double re = 0, im = 0;
                for (int c = lane; c < G; c += 32) {
                    re += __ldcg(a.part + ((size_t)c * a.qmax + p) * 2);
                    im += __ldcg(a.part + ((size_t)c * a.qmax + p) * 2 + 1);
                }
                re = warp_sum(re);
                im = warp_sum(im);
                if (lane == 0) coef[p] = make_double2(re, im);
            }
        if (!ks_grid_sync(a.bar, (++k) * G, abort)) return;
        // (4) w = y - sum_p c_p B_p, warps splitting p; norm and cross-term partials
        {
            C acc = czero<C>();
            for (int p = warp; p < q; p += KS_WARPS) {
                const C *B = p < kk ? a.W + (size_t)p * n : V + (size_t)(p - kk) * n;
                const double2 cd = __ldcg(coef + p);
                if (row < n) cfma(acc, from_d<C>(cd), B[row]);
            }
            upd[warp][lane] = canon(acc);
        }
        __syncthreads();
        if (warp == 0) {
            C w = ys[lane];
#pragma unroll
            for (int u = 0; u < KS_WARPS; ++u) w = csub(w, upd[u][lane]);
            w = canon(w);
            if (row >= n) w = czero<C>();
            ws[lane] = w;
            C ln = czero<C>(), lc = czero<C>();
            cdotacc(ln, w, w);
            cdotacc(lc, w, ys[lane]);
            double v0 = (double)canon(ln).x, v1 = (double)canon(lc).x, v2 = (double)canon(lc).y;
            v0 = warp_sum(v0);
            v1 = warp_sum(v1);
            v2 = warp_sum(v2);
            if (lane == 0) {
                a.npart[(size_t)b * 3] = v0;
                a.npart[(size_t)b * 3 + 1] = v1;
                a.npart[(size_t)b * 3 + 2] = v2;
            }
        }
        if (!ks_grid_sync(a.bar, (++k) * G, abort)) return;
        // (5) the norms, summed by every CTA in the same order; CTA 0 runs the step's finish
        if (warp == 0) {
            double v0 = 0, v1 = 0, v2 = 0;
            for (int c = lane; c < G; c += 32) {
                v0 += __ldcg(a.npart + (size_t)c * 3);
                v1 += __ldcg(a.npart + (size_t)c * 3 + 1);
                v2 += __ldcg(a.npart + (size_t)c * 3 + 2);
            }
            v0 = warp_sum(v0);
            v1 = warp_sum(v1);
            v2 = warp_sum(v2);
            if (lane == 0) { red[0] = v0; red[1] = v1; red[2] = v2; }
        }
        __syncthreads();
        const double n2 = red[0], nrm = sqrt(n2);
        const bool broken = nrm < a.tol;
        if (b == 0) {
            // the H column from the coefficients (other CTAs wrote them: through L2), then the
            // finish proper (subdiagonal, breakdown identity tail, state) with nco = 0
            double2 *Hs = a.H0 + (size_t)s * a.strideH;
            for (int p = tid; p < q; p += KS_THREADS) Hs[(size_t)(kk + j - 1) * (a.m + 1) + p] = __ldcg(coef + p);
            if (tid == 0) {
                FinishArgs f{};
                f.mode = FIN_KRYLOV; f.col = kk + j - 1; f.nco = 0; f.ldH = a.m + 1; f.m = a.m; f.kk = kk;
                f.compat_eye = a.compat_eye; f.tol = a.tol; f.H = a.H0; f.strideH = a.strideH;
                f.coef = a.coef0; f.strideC = a.strideC;
                run_finish(f, s, *st, n2, red[1], red[2]);
            }
        }
        // (6) v_j = w / ||w||; a breakdown ends the cycle's Krylov loop with v_j and the rest of
        // the basis zero, as the reference clears it (gDMR.cu:2256-2289): the cycle-end
        // projection reads all of it
        if (warp == 0 && row < n) {
            C v = ws[lane];
            const R al = broken ? R(0.f) : R(1.0 / nrm);
            v.x = v.x * al;
            v.y = v.y * al;
            if (broken) v = czero<C>();
            V[(size_t)j * n + row] = v;
            if (broken)
                for (int jj = j + 1; jj <= a.m - kk; ++jj) V[(size_t)jj * n + row] = czero<C>();
        }
        if (broken) return;
        if (!ks_grid_sync(a.bar, (++k) * G, abort)) return;
    }
}

// ----------------------------------------------------------------- many systems, one launch
// The Krylov loops of one restart cycle of many systems, of operators of different sizes, in one
// cooperative launch: the restart cycles of the 48-operator workload run in lockstep, and the
// Krylov loop of every system still in flight (the per-system convergence mask is the job list)
// is one kernel instead of four launches a step on each operator's stream.  Each job (one
// system) owns a contiguous range of CTAs sized to its n; its warps own SELL slices
// g, g + W, ... (g the warp's index in the job, W the job's warps), the same slices in every
// phase, so a warp only reads other warps' rows where the operator gathers v_{j-1}.  A step
// (arnoldiDMR's Krylov loop with the deflator, gDMR.cu:2069-2328):
//   SpMV of v_{j-1} into the job's scratch y, projection partials of [W V] against y (eight
//   coefficients a pass, warp sums, CTA sums in warp order) -> | CTA c sums coefficients
//   c, c + ncta, ... over the CTAs in order -> | update out = y - sum c_p B_p in place of y,
//   norm and cross-term partials -> | every CTA sums those in the same order, CTA 0 of the job
//   runs the step's finish (H column, breakdown test and identity tail), all scale their rows
//   into V_j -> | next step.
// The barriers are per job (the job's counter, target = passes x ncta); values other CTAs wrote
// are read through L2 (ld.global.cg).  Every wait is bounded by the process's wait limit and a
// timeout raises a flag that ends every job's loop.
// KrylovJob<R>: gdmr_kernels.cuh

constexpr int KM_THREADS = 256, KM_WARPS = KM_THREADS / 32, KM_PB = 8;   // coefficients a pass


template <class R>
__global__ void __launch_bounds__(KM_THREADS, 3) k_krylov_multi(const KrylovJob<R> *__restrict__ jobs,
                                                                 const int *__restrict__ cta_job, int *abort) {
    using C = typename CT<R>::t;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const KrylovJob<R> &a = jobs[cta_job[blockIdx.x]];
    const int c = blockIdx.x - a.cta0, ncta = a.ncta, n = a.n, kk = a.kk, nsl = a.nslices;
    const int gw = c * KM_WARPS + warp, nw = ncta * KM_WARPS;   // the warp's index in the job
    // the job's fields in registers: the loops store through other pointers, so fields read
    // through the reference would be loaded again before every use
    const C *__restrict__ W = a.W;
    C *__restrict__ V = a.V;
    C *__restrict__ y = a.y;
    const int *__restrict__ slice_ptr = a.slice_ptr;
    const int *__restrict__ cols = a.cols;
    const C *__restrict__ vals = a.vals;
    double2 *coef = a.coef;
    unsigned *bar = a.bar;
    const int m = a.m, qmax = a.qmax;
    double *part = a.part;
    double *npart = part + (size_t)ncta * qmax * 2;
    __shared__ double wsum[KM_WARPS][KM_PB][2];
    __shared__ double red[KM_WARPS][3];
    __shared__ C cs[QMAX];
    __shared__ double s_norm[3];
    unsigned k = 0;   // barrier passes
    auto basis = [&](int p) -> const C * { return p < kk ? W + (size_t)p * n : V + (size_t)(p - kk) * n; };
    for (int j = 1; j <= m - kk; ++j) {
        const int q = kk + j;
        const C *x = V + (size_t)(j - 1) * n;
        // (1) y = A v_{j-1} on the warp's slices (v_{j-1} rows of other warps through L2); the
        // entries of a slice four at a time, their loads issued before their products
        for (int sl = gw; sl < nsl; sl += nw) {
            const int row = sl * 32 + lane;
            const int beg = slice_ptr[sl], width = (slice_ptr[sl + 1] - beg) >> 5;
            C acc = czero<C>();
            int e = 0;
            for (; e + 4 <= width; e += 4) {
                C av[4], xv[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int idx = beg + (e + u) * 32 + lane;
                    av[u] = vals[idx];
                    xv[u] = ldcg_c(x + cols[idx]);
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) cfma(acc, av[u], xv[u]);
            }
            for (; e < width; ++e) {
                const int idx = beg + e * 32 + lane;
                cfma(acc, vals[idx], ldcg_c(x + cols[idx]));
            }
            if (row < n) y[row] = canon(acc);
        }
        __syncwarp();
        // (2) projection partials <B_p, y>, KM_PB coefficients a pass over the warp's rows
        for (int p0 = 0; p0 < q; p0 += KM_PB) {
            C acc[KM_PB];
#pragma unroll
            for (int u = 0; u < KM_PB; ++u) acc[u] = czero<C>();
            const C *bp[KM_PB];
#pragma unroll
            for (int u = 0; u < KM_PB; ++u) bp[u] = basis(p0 + u < q ? p0 + u : q - 1);
#pragma unroll 2
            for (int sl = gw; sl < nsl; sl += nw) {
                const int row = sl * 32 + lane;
                if (row >= n) continue;
                const C yv = y[row];
                C bv[KM_PB];
#pragma unroll
                for (int u = 0; u < KM_PB; ++u) bv[u] = bp[u][row];
#pragma unroll
                for (int u = 0; u < KM_PB; ++u) cdotacc(acc[u], bv[u], yv);
            }
#pragma unroll
            for (int u = 0; u < KM_PB; ++u) {
                // warp sums in the working precision: FP32 butterflies for complex64 (an FP64 warp
                // instruction is ~20 SM clocks on GB300)
                const double re = (double)warp_sum(acc[u].x), im = (double)warp_sum(acc[u].y);
                if (lane == 0) {
                    wsum[warp][u][0] = re;
                    wsum[warp][u][1] = im;
                }
            }
            __syncthreads();
            if (tid < 2 * KM_PB && p0 + tid / 2 < q) {
                double t = 0;
                for (int w = 0; w < KM_WARPS; ++w) t += wsum[w][tid / 2][tid & 1];
                part[((size_t)c * qmax + p0 + tid / 2) * 2 + (tid & 1)] = t;
            }
            __syncthreads();
        }
        if (!ks_grid_sync(bar, (++k) * ncta, abort)) return;
        // (3) coefficient p summed over the job's CTAs by CTA p mod ncta, in order
        if (warp == 0)
            for (int p = c; p < q; p += ncta) {
                double re = 0, im = 0;
                for (int g = lane; g < ncta; g += 32) {
                    re += __ldcg(part + ((size_t)g * qmax + p) * 2);
                    im += __ldcg(part + ((size_t)g * qmax + p) * 2 + 1);
                }
                re = warp_sum(re);
                im = warp_sum(im);
                if (lane == 0) coef[p] = make_double2(re, im);
            }
        if (!ks_grid_sync(bar, (++k) * ncta, abort)) return;
        // (4) out = y - sum_p c_p B_p in place of y (eight basis vectors' loads in flight before
        // their products); ||out||^2 and <out, y> partials
        for (int p = tid; p < q; p += KM_THREADS) cs[p] = from_d<C>(__ldcg(coef + p));
        __syncthreads();
        // per-thread norm accumulators in FP32 for complex64 (no FP64 operation per element)
        using NA = typename std::conditional<std::is_same<C, float2>::value, float, double>::type;
        NA v0 = 0, v1 = 0, v2 = 0;
        for (int sl = gw; sl < nsl; sl += nw) {
            const int row = sl * 32 + lane;
            if (row >= n) continue;
            const C yv = y[row];
            C w = yv;
            int p = 0;
            for (; p + 8 <= q; p += 8) {
                C bv[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) bv[u] = basis(p + u)[row];
#pragma unroll
                for (int u = 0; u < 8; ++u) cfms(w, cs[p + u], bv[u]);
            }
            for (; p < q; ++p) cfms(w, cs[p], basis(p)[row]);
            w = canon(w);
            y[row] = w;
            C ln = czero<C>(), lc = czero<C>();
            cdotacc(ln, w, w);
            cdotacc(lc, w, yv);
            v0 += (NA)canon(ln).x;
            v1 += (NA)canon(lc).x;
            v2 += (NA)canon(lc).y;
        }
        v0 = warp_sum(v0);
        v1 = warp_sum(v1);
        v2 = warp_sum(v2);
        if (lane == 0) { red[warp][0] = (double)v0; red[warp][1] = (double)v1; red[warp][2] = (double)v2; }
        __syncthreads();
        if (tid < 3) {
            double t = 0;
            for (int w = 0; w < KM_WARPS; ++w) t += red[w][tid];
            npart[(size_t)c * 3 + tid] = t;
        }
        if (!ks_grid_sync(bar, (++k) * ncta, abort)) return;
        // (5) the norms summed by every CTA in the same order; CTA 0 of the job runs the finish
        if (tid < 3) {
            double t = 0;
            for (int g = 0; g < ncta; ++g) t += __ldcg(npart + (size_t)g * 3 + tid);
            s_norm[tid] = t;
        }
        __syncthreads();
        const double n2 = s_norm[0], nrm = sqrt(n2);
        const bool broken = nrm < a.tol;
        if (c == 0) {
            for (int p = tid; p < q; p += KM_THREADS) a.H[(size_t)(kk + j - 1) * (m + 1) + p] = __ldcg(coef + p);
            if (tid == 0) {
                FinishArgs f{};
                f.mode = FIN_KRYLOV; f.col = kk + j - 1; f.nco = 0; f.ldH = a.m + 1; f.m = m; f.kk = kk;
                f.compat_eye = a.compat_eye; f.tol = a.tol; f.H = a.H; f.strideH = 0;
                f.coef = coef; f.strideC = 0;
                run_finish(f, 0, *a.state, n2, s_norm[1], s_norm[2]);
            }
        }
        // (6) v_j = out / ||out|| on the warp's rows; a breakdown ends the loop with v_j and the
        // rest of the basis zero (gDMR.cu:2256-2289), which the cycle-end projection reads
        const R al = broken ? R(0.f) : R(1.0 / nrm);
        for (int sl = gw; sl < nsl; sl += nw) {
            const int row = sl * 32 + lane;
            if (row >= n) continue;
            C v = y[row];
            v.x = v.x * al;
            v.y = v.y * al;
            if (broken) v = czero<C>();
            V[(size_t)j * n + row] = v;
            if (broken)
                for (int jj = j + 1; jj <= m - kk; ++jj) V[(size_t)jj * n + row] = czero<C>();
        }
        if (broken) return;
        if (!ks_grid_sync(bar, (++k) * ncta, abort)) return;
    }
}

// ----------------------------------------------------------------- batched W projection
// coef_s[p] = <W_p, y_s> for every active system s and deflation vector p: the shared part
// of a batched projection as one split-K product, so W is read once for the whole batch
// instead of once per system.  Persistent CTAs walk row tiles; a tile of W (kk x RT) and of
// the batch (nsys x RT) is copied into shared memory with cp.async, double-buffered, in its
// natural vector-major layout (leading dimension RT+2, so the strided thread tiling below
// reads distinct banks).  Thread (ip, js) of row group grp accumulates the 4 x 4 outputs
// p = ip + tilesP*a, s = js + tilesS*b over the rows grp, grp+KS, ... of each tile, and
// flushes them to double after every tile.  The KS row groups are summed in shared memory
// in a fixed order, and k_wproj_reduce sums the CTAs' partials in a fixed order.
constexpr int WP_KMAX = 32, WP_SMAX = 64;
template <class R> __host__ __device__ constexpr int wp_rt() { return sizeof(R) == 4 ? 64 : 32; }

__device__ __forceinline__ void cp_async_el(void *dst, const void *src, int bytes, bool valid) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    const int sz = valid ? bytes : 0;   // 0: zero-fill, nothing read
    if (bytes == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src), "r"(sz) : "memory");
    else
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(sz) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

struct WprojShape {
    int tilesP, tilesS, KP, SP, nout, KS;
};
__host__ __device__ inline WprojShape wproj_shape(int kk, int nsys) {
    WprojShape w;
    w.tilesP = (kk + 3) / 4;
    w.tilesS = (nsys + 3) / 4;
    w.KP = 4 * w.tilesP;
    w.SP = 4 * w.tilesS;
    w.nout = w.tilesP * w.tilesS;
    w.KS = NT / w.nout;
    if (w.KS > 8) w.KS = 8;
    return w;
}
template <class R> size_t wproj_smem(int kk, int nsys) {
    const WprojShape w = wproj_shape(kk, nsys);
    const size_t tiles = 2 * (size_t)(w.KP + w.SP) * (wp_rt<R>() + 2) * sizeof(typename CT<R>::t);
    const size_t red = (size_t)NT * 16 * sizeof(double2);
    return tiles > red ? tiles : red;
}

template <class R>
__global__ void __launch_bounds__(NT, 2) k_wproj(int n, int kk, const typename CT<R>::t *__restrict__ W,
                                                 const typename CT<R>::t *__restrict__ Y0, size_t strideY,
                                                 const int *__restrict__ act, int nsys, double *__restrict__ part) {
    using C = typename CT<R>::t;
    constexpr int RT = wp_rt<R>(), LD = RT + 2;
    extern __shared__ __align__(16) unsigned char wp_sm[];
    __shared__ int s_act[WP_SMAX];
    const WprojShape sh = wproj_shape(kk, nsys);
    const int stage = (sh.KP + sh.SP) * LD;
    C *buf = reinterpret_cast<C *>(wp_sm);
    const int tid = threadIdx.x, G = gridDim.x;
    const int grp = tid / sh.nout, o = tid % sh.nout, ip = o % sh.tilesP, js = o / sh.tilesP;
    const bool mine = grp < sh.KS;
    // zero both buffers once: the padding vectors (p >= kk, s >= nsys) are never copied
    for (int e = tid; e < 2 * stage; e += NT) buf[e] = czero<C>();
    if (tid < nsys) s_act[tid] = act[tid];
    __syncthreads();
    const long nrt = (n + RT - 1) / RT;
    auto issue = [&](long rt, int b) {
        C *Wt = buf + (size_t)b * stage;
        C *Yt = Wt + (size_t)sh.KP * LD;
        const long r0 = rt * RT;
        for (int e = tid; e < kk * RT; e += NT) {
            const int p = e / RT, r = e % RT;
            const bool v = r0 + r < n;
            cp_async_el(Wt + p * LD + r, W + (size_t)p * n + (v ? r0 + r : 0), sizeof(C), v);
        }
        for (int e = tid; e < nsys * RT; e += NT) {
            const int sl = e / RT, r = e % RT;
            const bool v = r0 + r < n;
            cp_async_el(Yt + sl * LD + r, Y0 + (size_t)s_act[sl] * strideY + (v ? r0 + r : 0), sizeof(C), v);
        }
        cp_async_commit();
    };
    double2 accd[4][4];
    C acc[4][4];   // complex64: one tile's sums; complex128: the running sums
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            accd[a][c] = make_double2(0.0, 0.0);
            acc[a][c] = czero<C>();
        }
    int b = 0;
    if ((long)blockIdx.x < nrt) issue(blockIdx.x, 0);
    for (long rt = blockIdx.x; rt < nrt; rt += G, b ^= 1) {
        if (rt + G < nrt) issue(rt + G, b ^ 1);
        else cp_async_commit();   // empty group keeps wait_group 1 meaning "tile rt landed"
        cp_async_wait1();
        __syncthreads();
        if (mine) {
            const C *Wt = buf + (size_t)b * stage;
            const C *Yt = Wt + (size_t)sh.KP * LD;
            if constexpr (sizeof(R) == 4) {
#pragma unroll
                for (int a = 0; a < 4; ++a)
#pragma unroll
                    for (int c = 0; c < 4; ++c) acc[a][c] = czero<C>();
            }
#pragma unroll 2
            for (int r = grp; r < RT; r += sh.KS) {
                C wv[4], yv[4];
#pragma unroll
                for (int a = 0; a < 4; ++a) wv[a] = Wt[(ip + sh.tilesP * a) * LD + r];
#pragma unroll
                for (int c = 0; c < 4; ++c) yv[c] = Yt[(js + sh.tilesS * c) * LD + r];
#pragma unroll
                for (int a = 0; a < 4; ++a)
#pragma unroll
                    for (int c = 0; c < 4; ++c) cdotacc(acc[a][c], wv[a], yv[c]);
            }
            if constexpr (sizeof(R) == 4) {   // complex64: flush the tile's sums to double
#pragma unroll
                for (int a = 0; a < 4; ++a)
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        accd[a][c].x += (double)acc[a][c].x;
                        accd[a][c].y += (double)acc[a][c].y;
                    }
            }
        }
        __syncthreads();
    }
    if constexpr (sizeof(R) == 8) {
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int c = 0; c < 4; ++c) accd[a][c] = make_double2(acc[a][c].x, acc[a][c].y);
    }
    // sum the row groups (fixed order) through shared memory, then write this CTA's partials
    double2 *red = reinterpret_cast<double2 *>(wp_sm);   // [thread][16]
    if (mine && grp > 0)
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int c = 0; c < 4; ++c) red[(size_t)tid * 16 + a * 4 + c] = accd[a][c];
    __syncthreads();
    if (mine && grp == 0) {
        for (int g = 1; g < sh.KS; ++g) {
            const double2 *rg = red + (size_t)(g * sh.nout + o) * 16;
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    accd[a][c].x += rg[a * 4 + c].x;
                    accd[a][c].y += rg[a * 4 + c].y;
                }
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int p = ip + sh.tilesP * a, sl = js + sh.tilesS * c;
                if (p < kk && sl < nsys) {
                    double *pp = part + ((size_t)p * nsys + sl) * 2 * G;
                    pp[blockIdx.x] = accd[a][c].x;
                    pp[G + blockIdx.x] = accd[a][c].y;
                }
            }
    }
}

// coef_s[p] = sum over the G partials of output (p, s), one warp per output, fixed order.
__global__ void __launch_bounds__(NT) k_wproj_reduce(int kk, int nsys, int G, const double *__restrict__ part,
                                                     const int *__restrict__ act, double2 *__restrict__ coef0,
                                                     size_t strideC) {
    const int lane = threadIdx.x & 31;
    const int o = blockIdx.x * NW + (threadIdx.x >> 5);
    if (o >= kk * nsys) return;
    const int p = o / nsys, sl = o % nsys;
    const double *pp = part + (size_t)o * 2 * G;
    double re = 0, im = 0;
    for (int g = lane; g < G; g += 32) { re += pp[g]; im += pp[G + g]; }
    re = warp_sum(re);
    im = warp_sum(im);
    if (lane == 0) coef0[(size_t)act[sl] * strideC + p] = make_double2(re, im);
}

// ----------------------------------------------------------------- batched update, W in registers
// out_s = w_s - W c_s[0:kk] - V_s c_s[kk:kk+qb] for a group of SGU systems and NT rows per CTA:
// each thread keeps its row of W (kk <= KW values) in registers and applies it to every system
// of the group, so W is read from memory once per group instead of once per system.  Norm
// partials reduce per warp into shared memory and once per CTA; the finish is k_update's.
// Grid (groups, chunks): the groups of one chunk run side by side and share W through L2.
template <class R, int KW, int SGU>
__global__ void __launch_bounds__(NT, 2) k_update_wreg(int n, int kk, const typename CT<R>::t *__restrict__ W,
                                                       const typename CT<R>::t *__restrict__ V0, size_t strideV, int qb,
                                                       const typename CT<R>::t *__restrict__ w0, size_t strideW,
                                                       typename CT<R>::t *__restrict__ out0, size_t strideO,
                                                       const int *__restrict__ act, int nsys,
                                                       const double2 *__restrict__ coef0, size_t strideC,
                                                       double2 *__restrict__ partials, unsigned *tickets,
                                                       SysState *state, FinishArgs fin, int skip_broken) {
    using C = typename CT<R>::t;
    extern __shared__ __align__(16) unsigned char uw_sm[];
    const int q = kk + qb;
    C *cs = reinterpret_cast<C *>(uw_sm);   // [SGU][q]
    __shared__ double red[3][SGU][NW];
    __shared__ int s_act[SGU], s_live[SGU];
    __shared__ unsigned lastmask;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g0 = blockIdx.x * SGU, ng = min(SGU, nsys - g0);
    const int chunk = blockIdx.y, G = gridDim.y;
    const long i = (long)chunk * NT + tid;
    const bool in = i < n;
    C wr[KW];
#pragma unroll
    for (int p = 0; p < KW; ++p) wr[p] = (p < kk && in) ? W[(size_t)p * n + i] : czero<C>();
    for (int e = tid; e < ng * q; e += NT) {
        const int g = e / q, p = e % q;
        cs[(size_t)g * q + p] = from_d<C>(coef0[(size_t)act[g0 + g] * strideC + p]);
    }
    if (tid < ng) {
        const int s = act[g0 + tid];
        s_act[tid] = s;
        s_live[tid] = !(skip_broken && state[s].broken);
    }
    __syncthreads();
    for (int g = 0; g < ng; ++g) {
        const int s = s_act[g];
        C org = czero<C>(), acc = czero<C>();
        if (s_live[g] && in) {
            org = w0[(size_t)s * strideW + i];
            acc = org;
            const C *c = cs + (size_t)g * q;
#pragma unroll
            for (int p = 0; p < KW; ++p)
                if (p < kk) cfms(acc, c[p], wr[p]);
            const C *V = V0 + (size_t)s * strideV + i;
#pragma unroll 4
            for (int p = 0; p < qb; ++p) cfms(acc, c[kk + p], V[(size_t)p * n]);
            out0[(size_t)s * strideO + i] = acc;
        }
        C ln = czero<C>(), lc = czero<C>();
        cdotacc(ln, acc, acc);
        cdotacc(lc, acc, org);
        const double v0 = warp_sum((double)ln.x), v1 = warp_sum((double)lc.x), v2 = warp_sum((double)lc.y);
        if (lane == 0) {
            red[0][g][warp] = v0;
            red[1][g][warp] = v1;
            red[2][g][warp] = v2;
        }
    }
    __syncthreads();
    if (tid < ng) {
        double t0 = 0, t1 = 0, t2 = 0;
#pragma unroll
        for (int w = 0; w < NW; ++w) {
            t0 += red[0][tid][w];
            t1 += red[1][tid][w];
            t2 += red[2][tid][w];
        }
        double *part = (double *)partials + (size_t)(g0 + tid) * 3 * G;
        part[chunk] = t0;
        part[G + chunk] = t1;
        part[2 * G + chunk] = t2;
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) {
        unsigned mk = 0;
        for (int g = 0; g < ng; ++g)
            if (atomicAdd(&tickets[g0 + g], 1u) == (unsigned)G - 1) mk |= 1u << g;
        lastmask = mk;
    }
    __syncthreads();
    if (!lastmask) return;
    __threadfence();
    __shared__ double red2[3][NW];
    for (int g = 0; g < ng; ++g) {
        if (!(lastmask >> g & 1u)) continue;
        const int s = s_act[g];
        double tot[3];
        sum_partials<3>((double *)partials + (size_t)(g0 + g) * 3 * G, G, tot, red2);
        if (tid == 0) {
            if (s_live[g]) run_finish(fin, s, state[s], tot[0], tot[1], tot[2]);
            tickets[g0 + g] = 0;
        }
        __syncthreads();
    }
}

// ----------------------------------------------------------------- row-stationary batched update
// The complex64 batched update with a shared deflation segment, every system of the batch in
// one CTA.  Each thread keeps its row of W (the kk shared vectors) in registers and walks the
// systems, so W is read from memory once per launch and the shared part W c_s never goes
// through memory (the tensor-core apply writes it and the per-system update reads it back,
// 16 bytes a row a system on top of the algorithmic bytes).  CTAs own contiguous ranges of
// 256-row chunks, about two a SM.  Two systems' V loads go out together, VB vectors of each
// ahead of the arithmetic, and the shared part is computed while they are in flight.  Norm and cross term are
// summed per warp in FP32 butterflies (one FP64 warp instruction is ~64 scheduler clocks on
// GB300, three FP64 butterflies per system per chunk would bound the kernel), accumulated per
// warp in shared memory over the CTA's chunks and summed in FP64 once per CTA; the last CTA
// sums the CTAs' partials, one warp a system, in a fixed order.
inline size_t update_rows_smem(int nsys, int q) {
    return sizeof(float2) * (size_t)nsys * q + sizeof(float) * (size_t)nsys * 3 * NW + 2 * sizeof(int) * (size_t)nsys;
}

template <int KW, int VB>
__global__ void __launch_bounds__(NT, 2) k_update_rows(int n, int kk, const float2 *__restrict__ W,
                                                       const float2 *__restrict__ V0, size_t strideV, int qb,
                                                       const float2 *__restrict__ w0, size_t strideW,
                                                       float2 *__restrict__ out0, size_t strideO,
                                                       const int *__restrict__ act, int nsys,
                                                       const double2 *__restrict__ coef0, size_t strideC, int cpb,
                                                       double *__restrict__ partials, unsigned *tickets,
                                                       SysState *state, FinishArgs fin, int skip_broken) {
    extern __shared__ __align__(16) unsigned char ur_sm[];
    const int q = kk + qb;
    float2 *cs = reinterpret_cast<float2 *>(ur_sm);                       // [nsys][q]
    float *red = reinterpret_cast<float *>(cs + (size_t)nsys * q);         // [nsys * 3][NW]
    int *s_act = reinterpret_cast<int *>(red + (size_t)nsys * 3 * NW);    // [nsys]
    int *s_live = s_act + nsys;                                           // [nsys]
    __shared__ unsigned s_last;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, G = gridDim.x;
    for (int e = tid; e < nsys * q; e += NT) {
        const int g = e / q, p = e - g * q;
        cs[e] = from_d<float2>(coef0[(size_t)act[g] * strideC + p]);
    }
    for (int e = tid; e < nsys * 3 * NW; e += NT) red[e] = 0.f;
    for (int g = tid; g < nsys; g += NT) {
        const int s = act[g];
        s_act[g] = s;
        s_live[g] = !(skip_broken && state[s].broken);
    }
    __syncthreads();
    const long nch = ((long)n + NT - 1) / NT, c0 = (long)blockIdx.x * cpb;
    const long c1 = c0 + cpb < nch ? c0 + cpb : nch;
    for (long c = c0; c < c1; ++c) {
        const long i = c * NT + tid;
        const bool in = i < n;
        float2 wr[KW];
#pragma unroll
        for (int p = 0; p < KW; ++p) wr[p] = (p < kk && in) ? W[(size_t)p * n + i] : czero<float2>();
        // two systems at a time: 2 (VB + 1) loads in flight before their products
        for (int g = 0; g < nsys; g += 2) {
            const bool two = g + 1 < nsys;
            const int gb = two ? g + 1 : g;
            const int sa = s_act[g], sb = s_act[gb];
            const bool la = in && s_live[g], lb = in && two && s_live[gb];
            const float2 *ca = cs + (size_t)g * q, *cb = cs + (size_t)gb * q;
            const float2 *Va = V0 + (size_t)sa * strideV + i, *Vb = V0 + (size_t)sb * strideV + i;
            float2 va[VB], vb[VB];
#pragma unroll
            for (int u = 0; u < VB; ++u) {
                va[u] = (la && u < qb) ? Va[(size_t)u * n] : czero<float2>();
                vb[u] = (lb && u < qb) ? Vb[(size_t)u * n] : czero<float2>();
            }
            const float2 oa = la ? w0[(size_t)sa * strideW + i] : czero<float2>();
            const float2 ob = lb ? w0[(size_t)sb * strideW + i] : czero<float2>();
            float2 aa = oa, ab = ob;
#pragma unroll
            for (int p = 0; p < KW; ++p)
                if (p < kk) {
                    cfms(aa, ca[p], wr[p]);
                    cfms(ab, cb[p], wr[p]);
                }
#pragma unroll
            for (int u = 0; u < VB; ++u)
                if (u < qb) {
                    cfms(aa, ca[kk + u], va[u]);
                    cfms(ab, cb[kk + u], vb[u]);
                }
            for (int p0 = VB; p0 < qb; p0 += VB) {
#pragma unroll
                for (int u = 0; u < VB; ++u) {
                    va[u] = (la && p0 + u < qb) ? Va[(size_t)(p0 + u) * n] : czero<float2>();
                    vb[u] = (lb && p0 + u < qb) ? Vb[(size_t)(p0 + u) * n] : czero<float2>();
                }
#pragma unroll
                for (int u = 0; u < VB; ++u)
                    if (p0 + u < qb) {
                        cfms(aa, ca[kk + p0 + u], va[u]);
                        cfms(ab, cb[kk + p0 + u], vb[u]);
                    }
            }
            if (la) out0[(size_t)sa * strideO + i] = aa;
            if (lb) out0[(size_t)sb * strideO + i] = ab;
            float2 na = czero<float2>(), xa = czero<float2>(), nb = czero<float2>(), xb = czero<float2>();
            cdotacc(na, aa, aa);
            cdotacc(xa, aa, oa);
            cdotacc(nb, ab, ab);
            cdotacc(xb, ab, ob);
            const float v0 = warp_sum(na.x), v1 = warp_sum(xa.x), v2 = warp_sum(xa.y);
            const float v3 = warp_sum(nb.x), v4 = warp_sum(xb.x), v5 = warp_sum(xb.y);
            if (lane == 0) {
                red[((size_t)g * 3 + 0) * NW + warp] += v0;
                red[((size_t)g * 3 + 1) * NW + warp] += v1;
                red[((size_t)g * 3 + 2) * NW + warp] += v2;
                if (two) {
                    red[((size_t)gb * 3 + 0) * NW + warp] += v3;
                    red[((size_t)gb * 3 + 1) * NW + warp] += v4;
                    red[((size_t)gb * 3 + 2) * NW + warp] += v5;
                }
            }
        }
    }
    __syncthreads();
    for (int e = tid; e < nsys * 3; e += NT) {
        double t = 0;
#pragma unroll
        for (int w = 0; w < NW; ++w) t += (double)red[(size_t)e * NW + w];
        partials[(size_t)e * G + blockIdx.x] = t;
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(&tickets[0], 1u) == (unsigned)G - 1 ? 1u : 0u;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    for (int g = warp; g < nsys; g += NW) {
        double t[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            double a = 0;
            for (int b = lane; b < G; b += 32) a += __ldcg(partials + ((size_t)g * 3 + j) * G + b);
            t[j] = warp_sum(a);
        }
        if (lane == 0 && s_live[g]) run_finish(fin, s_act[g], state[s_act[g]], t[0], t[1], t[2]);
    }
    __syncthreads();
    if (tid == 0) tickets[0] = 0;
}

// ----------------------------------------------------------------- split-vector projection
// For short vectors the chunk count is small, so a CTA per chunk walks all q vectors in
// series.  Here blockIdx.z also splits the vectors into groups of VPG: each (coefficient,
// chunk) partial is still written by exactly one CTA, and the last of the G x groups CTAs of
// a system sums them in the fixed order of k_mdot.
template <class R, int VPG>
__global__ void __launch_bounds__(NT) k_mdot_vs(int n, const typename CT<R>::t *__restrict__ segA, int qa,
                                                const typename CT<R>::t *__restrict__ segB0, size_t strideB, int qb,
                                                const typename CT<R>::t *__restrict__ w0, size_t strideW,
                                                const int *__restrict__ act, double2 *__restrict__ partials,
                                                int qmax, unsigned *tickets, double2 *__restrict__ coef0,
                                                size_t strideC, SysState *state, int skip_broken) {
    using C = typename CT<R>::t;
    const int slot = blockIdx.x, s = act[slot], chunk = blockIdx.y, G = gridDim.y;
    if (skip_broken && state[s].broken) return;
    const C *segB = segB0 + (size_t)s * strideB;
    const C *w = w0 + (size_t)s * strideW;
    const int q = qa + qb, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int p0 = blockIdx.z * VPG, p1 = min(q, p0 + VPG);
    __shared__ C wsum[NW][VPG];
    const long i = (long)chunk * NT + tid;
    const C wv = i < n ? w[i] : czero<C>();
    C vv[VPG];
#pragma unroll
    for (int u = 0; u < VPG; ++u) {
        const int p = p0 + u < p1 ? p0 + u : p0;
        const C *vp = p < qa ? segA + (size_t)p * n : segB + (size_t)(p - qa) * n;
        vv[u] = i < n ? vp[i] : czero<C>();
    }
#pragma unroll
    for (int u = 0; u < VPG; ++u) {
        C a = czero<C>();
        cdotacc(a, vv[u], wv);
        a.x = warp_sum(a.x);
        a.y = warp_sum(a.y);
        if (lane == 0) wsum[warp][u] = a;
    }
    __syncthreads();
    double *part = (double *)partials + (size_t)slot * qmax * 2 * G;
    for (int u = tid; u < p1 - p0; u += NT) {
        double re = 0, im = 0;
#pragma unroll
        for (int ww = 0; ww < NW; ++ww) { re += (double)wsum[ww][u].x; im += (double)wsum[ww][u].y; }
        double *pp = part + (size_t)(p0 + u) * 2 * G;
        pp[chunk] = re;
        pp[G + chunk] = im;
    }
    if (!arrive_last(&tickets[slot], (unsigned)G * gridDim.z)) return;
    double2 *coef = coef0 + (size_t)s * strideC;
    for (int p = warp; p < q; p += NW) {
        const double *pp = part + (size_t)p * 2 * G;
        double re = 0, im = 0;
        for (int g = lane; g < G; g += 32) { re += __ldcg(pp + g); im += __ldcg(pp + G + g); }
        re = warp_sum(re);
        im = warp_sum(im);
        if (lane == 0) coef[p] = make_double2(re, im);
    }
    if (tid == 0) tickets[slot] = 0;
}

// ----------------------------------------------------------------- system-grouped variants
// One CTA serves SB systems of one chunk: every tile of the shared vectors (segment A, the
// deflation basis W) is loaded once and used for all SB systems, instead of once per system
// (from L2), which matters when a batch of systems shares W.  Per-system results, the
// partial layout and the last-CTA finishing are those of k_mdot / k_update.
template <class R, int EPT, int SB>
__global__ void __launch_bounds__(NT, 2)
    k_mdot_grp(int n, const typename CT<R>::t *__restrict__ segA, int qa, const typename CT<R>::t *__restrict__ segB0,
               size_t strideB, int qb, const typename CT<R>::t *__restrict__ w0, size_t strideW,
               const int *__restrict__ act, int nsys, double2 *__restrict__ partials, int qmax, unsigned *tickets,
               double2 *__restrict__ coef0, size_t strideC) {
    using C = typename CT<R>::t;
    extern __shared__ unsigned char grp_sm[];
    C *wsum = reinterpret_cast<C *>(grp_sm);           // [NW][SB][qmax]
    const int slot0 = blockIdx.x * SB, ns = min(SB, nsys - slot0), chunk = blockIdx.y, G = gridDim.y;
    const int q = qa + qb, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long c0 = (long)chunk * NT * EPT;
    int sys[SB];
    C wv[SB][EPT];
#pragma unroll
    for (int g = 0; g < SB; ++g) {
        sys[g] = act[slot0 + (g < ns ? g : 0)];
        const C *w = w0 + (size_t)sys[g] * strideW;
#pragma unroll
        for (int e = 0; e < EPT; ++e) {
            const long i = c0 + tid + (long)e * NT;
            wv[g][e] = (g < ns && i < n) ? w[i] : czero<C>();
        }
    }
    // shared segment: one load per tile, SB dot products
    for (int p = 0; p < qa; ++p) {
        C a[EPT];
        const C *vp = segA + (size_t)p * n;
#pragma unroll
        for (int e = 0; e < EPT; ++e) {
            const long i = c0 + tid + (long)e * NT;
            a[e] = i < n ? vp[i] : czero<C>();
        }
#pragma unroll
        for (int g = 0; g < SB; ++g) {
            C d = czero<C>();
#pragma unroll
            for (int e = 0; e < EPT; ++e) cdotacc(d, a[e], wv[g][e]);
            d.x = warp_sum(d.x);
            d.y = warp_sum(d.y);
            if (lane == 0) wsum[((size_t)warp * SB + g) * qmax + p] = d;
        }
    }
    // per-system segments
#pragma unroll
    for (int g = 0; g < SB; ++g) {
        if (g >= ns) break;
        const C *segB = segB0 + (size_t)sys[g] * strideB;
        for (int p = 0; p < qb; p += 2) {
            C a0[EPT], a1[EPT];
            const C *v0 = segB + (size_t)p * n;
            const C *v1 = segB + (size_t)(p + 1 < qb ? p + 1 : p) * n;
#pragma unroll
            for (int e = 0; e < EPT; ++e) {
                const long i = c0 + tid + (long)e * NT;
                a0[e] = i < n ? v0[i] : czero<C>();
                a1[e] = i < n ? v1[i] : czero<C>();
            }
            C d0 = czero<C>(), d1 = czero<C>();
#pragma unroll
            for (int e = 0; e < EPT; ++e) {
                cdotacc(d0, a0[e], wv[g][e]);
                cdotacc(d1, a1[e], wv[g][e]);
            }
            d0.x = warp_sum(d0.x);
            d0.y = warp_sum(d0.y);
            d1.x = warp_sum(d1.x);
            d1.y = warp_sum(d1.y);
            if (lane == 0) {
                wsum[((size_t)warp * SB + g) * qmax + qa + p] = d0;
                if (p + 1 < qb) wsum[((size_t)warp * SB + g) * qmax + qa + p + 1] = d1;
            }
        }
    }
    __syncthreads();
    for (int e = tid; e < ns * q; e += NT) {
        const int g = e / q, p = e % q;
        double re = 0, im = 0;
#pragma unroll
        for (int ww = 0; ww < NW; ++ww) {
            const C v = wsum[((size_t)ww * SB + g) * qmax + p];
            re += (double)v.x;
            im += (double)v.y;
        }
        double *pp = (double *)partials + ((size_t)(slot0 + g) * qmax + p) * 2 * G;
        pp[chunk] = re;
        pp[G + chunk] = im;
    }
    __shared__ unsigned lastmask;
    __threadfence();
    __syncthreads();
    if (tid == 0) {
        unsigned mk = 0;
        for (int g = 0; g < ns; ++g)
            if (atomicAdd(&tickets[slot0 + g], 1u) == (unsigned)G - 1) mk |= 1u << g;
        lastmask = mk;
    }
    __syncthreads();
    if (!lastmask) return;
    __threadfence();
    for (int g = 0; g < ns; ++g) {
        if (!(lastmask >> g & 1u)) continue;
        double2 *coef = coef0 + (size_t)sys[g] * strideC;
        const double *part = (const double *)partials + (size_t)(slot0 + g) * qmax * 2 * G;
        for (int p = warp; p < q; p += NW) {
            const double *pp = part + (size_t)p * 2 * G;
            double re = 0, im = 0;
            for (int gg = lane; gg < G; gg += 32) { re += __ldcg(pp + gg); im += __ldcg(pp + G + gg); }
            re = warp_sum(re);
            im = warp_sum(im);
            if (lane == 0) coef[p] = make_double2(re, im);
        }
        if (tid == 0) tickets[slot0 + g] = 0;
    }
}

template <class R, int EPT, int SB>
__global__ void __launch_bounds__(NT, 2)
    k_update_grp(int n, const typename CT<R>::t *__restrict__ segA, int qa, const typename CT<R>::t *__restrict__ segB0,
                 size_t strideB, int qb, const typename CT<R>::t *__restrict__ w0, size_t strideW,
                 typename CT<R>::t *__restrict__ out0, size_t strideO, const int *__restrict__ act, int nsys,
                 const double2 *__restrict__ coef0, size_t strideC, double2 *__restrict__ partials,
                 unsigned *tickets, SysState *state, FinishArgs fin, int skip_broken) {
    using C = typename CT<R>::t;
    extern __shared__ unsigned char grp_sm[];
    C *cs = reinterpret_cast<C *>(grp_sm);              // [SB][qmax] coefficients
    __shared__ double red[3][NW];
    const int slot0 = blockIdx.x * SB, ns = min(SB, nsys - slot0), chunk = blockIdx.y, G = gridDim.y;
    const int q = qa + qb, tid = threadIdx.x;
    const int qmax = q;   // coefficient table row length (strideC may be 0: one shared coefficient vector)
    int sys[SB];
    bool live[SB];
#pragma unroll
    for (int g = 0; g < SB; ++g) {
        sys[g] = act[slot0 + (g < ns ? g : 0)];
        live[g] = g < ns && !(skip_broken && state[sys[g]].broken);
    }
    for (int e = tid; e < ns * q; e += NT) {
        const int g = e / q, p = e % q;
        cs[(size_t)g * qmax + p] = from_d<C>(coef0[(size_t)sys[g] * strideC + p]);
    }
    __syncthreads();
    const long c0 = (long)chunk * NT * EPT;
    C acc[SB][EPT], org[SB][EPT];
#pragma unroll
    for (int g = 0; g < SB; ++g) {
        const C *w = w0 + (size_t)sys[g] * strideW;
#pragma unroll
        for (int e = 0; e < EPT; ++e) {
            const long i = c0 + tid + (long)e * NT;
            org[g][e] = (live[g] && i < n) ? w[i] : czero<C>();
            acc[g][e] = org[g][e];
        }
    }
    for (int p = 0; p < qa; ++p) {
        C a[EPT];
        const C *vp = segA + (size_t)p * n;
#pragma unroll
        for (int e = 0; e < EPT; ++e) {
            const long i = c0 + tid + (long)e * NT;
            a[e] = i < n ? vp[i] : czero<C>();
        }
#pragma unroll
        for (int g = 0; g < SB; ++g) {
            const C c = g < ns ? cs[(size_t)g * qmax + p] : czero<C>();
#pragma unroll
            for (int e = 0; e < EPT; ++e) cfms(acc[g][e], c, a[e]);
        }
    }
#pragma unroll
    for (int g = 0; g < SB; ++g) {
        if (!live[g]) continue;
        const C *segB = segB0 + (size_t)sys[g] * strideB;
        for (int p = 0; p < qb; p += 2) {
            C a0[EPT], a1[EPT];
            const C *v0 = segB + (size_t)p * n;
            const C *v1 = segB + (size_t)(p + 1 < qb ? p + 1 : p) * n;
#pragma unroll
            for (int e = 0; e < EPT; ++e) {
                const long i = c0 + tid + (long)e * NT;
                a0[e] = i < n ? v0[i] : czero<C>();
                a1[e] = i < n ? v1[i] : czero<C>();
            }
            const C c0v = cs[(size_t)g * qmax + qa + p];
            const C c1v = p + 1 < qb ? cs[(size_t)g * qmax + qa + p + 1] : czero<C>();
#pragma unroll
            for (int e = 0; e < EPT; ++e) {
                cfms(acc[g][e], c0v, a0[e]);
                cfms(acc[g][e], c1v, a1[e]);
            }
        }
    }
    // per-system outputs and norms
#pragma unroll
    for (int g = 0; g < SB; ++g) {
        C ln = czero<C>(), lc = czero<C>();
        if (live[g]) {
            C *out = out0 + (size_t)sys[g] * strideO;
#pragma unroll
            for (int e = 0; e < EPT; ++e) {
                const long i = c0 + tid + (long)e * NT;
                acc[g][e] = canon(acc[g][e]);
                if (i < n) out[i] = acc[g][e];
                cdotacc(ln, acc[g][e], acc[g][e]);
                cdotacc(lc, acc[g][e], org[g][e]);
            }
        }
        double v[3];
        if constexpr (std::is_same<C, float2>::value) {
            const float f[3] = {ln.x, lc.x, lc.y};
            block_sum_f<3>(f, v, red);
        } else {
            v[0] = (double)ln.x;
            v[1] = (double)lc.x;
            v[2] = (double)lc.y;
            block_sum<3>(v, red);
        }
        if (tid == 0 && g < ns) {
            double *part = (double *)partials + (size_t)(slot0 + g) * 3 * G;
            part[chunk] = v[0];
            part[G + chunk] = v[1];
            part[2 * G + chunk] = v[2];
        }
        __syncthreads();
    }
    __shared__ unsigned lastmask;
    __threadfence();
    __syncthreads();
    if (tid == 0) {
        unsigned mk = 0;
        for (int g = 0; g < ns; ++g)
            if (atomicAdd(&tickets[slot0 + g], 1u) == (unsigned)G - 1) mk |= 1u << g;
        lastmask = mk;
    }
    __syncthreads();
    if (!lastmask) return;
    __threadfence();
    for (int g = 0; g < ns; ++g) {
        if (!(lastmask >> g & 1u)) continue;
        double tot[3];
        sum_partials<3>((double *)partials + (size_t)(slot0 + g) * 3 * G, G, tot, red);
        if (tid == 0) {
            if (live[g]) run_finish(fin, sys[g], state[sys[g]], tot[0], tot[1], tot[2]);
            tickets[slot0 + g] = 0;
        }
        __syncthreads();
    }
}

// ----------------------------------------------------------------- scale
template <class R>
__global__ void __launch_bounds__(NT) k_scale(int n, const typename CT<R>::t *__restrict__ in0, size_t strideI,
                                              typename CT<R>::t *__restrict__ o10, size_t strideO1,
                                              typename CT<R>::t *__restrict__ o20, size_t strideO2,
                                              const int *__restrict__ act, const SysState *__restrict__ state,
                                              int honour_broken) {
    using C = typename CT<R>::t;
    const int s = act[blockIdx.y];
    const bool zero = honour_broken && state[s].broken;
    const R a = (R)state[s].alpha;
    const C *in = in0 + (size_t)s * strideI;
    C *o1 = o10 + (size_t)s * strideO1;
    C *o2 = o20 ? o20 + (size_t)s * strideO2 : nullptr;
    for (long i = (long)blockIdx.x * NT + threadIdx.x; i < n; i += (long)gridDim.x * NT) {
        C v = zero ? czero<C>() : in[i];
        v.x *= a;
        v.y *= a;
        if (zero) v = czero<C>();
        o1[i] = v;
        if (o2) o2[i] = v;
    }
}

// ----------------------------------------------------------------- cycle-end combination
template <class R>
__global__ void __launch_bounds__(NT) k_combine(int n, int kk, int m, const typename CT<R>::t *__restrict__ W,
                                                const typename CT<R>::t *__restrict__ Z,
                                                const typename CT<R>::t *__restrict__ V0, size_t strideV,
                                                typename CT<R>::t *__restrict__ r0, size_t strideR,
                                                typename CT<R>::t *__restrict__ x0, size_t strideX,
                                                const double2 *__restrict__ t0, const double2 *__restrict__ y0,
                                                size_t strideC, const int *__restrict__ act,
                                                double2 *__restrict__ partials, unsigned *tickets, SysState *state) {
    using C = typename CT<R>::t;
    constexpr int EPT = ept<R>();
    const int slot = blockIdx.x, s = act[slot], chunk = blockIdx.y, G = gridDim.y;
    const C *V = V0 + (size_t)s * strideV;
    C *r = r0 + (size_t)s * strideR;
    C *x = x0 + (size_t)s * strideX;
    const int tid = threadIdx.x;
    __shared__ C ts[QMAX], ys[QMAX];
    __shared__ double red[1][NW];
    const R ra = (R)state[s].rho_abs;
    for (int p = tid; p <= m; p += NT) {
        ts[p] = from_d<C>(t0[(size_t)s * strideC + p]);
        C yy = p < m ? from_d<C>(y0[(size_t)s * strideC + p]) : czero<C>();
        yy.x *= ra;
        yy.y *= ra;
        ys[p] = yy;
    }
    __syncthreads();
    const long c0 = (long)chunk * NT * EPT;
    C ra_[EPT], xa[EPT];
#pragma unroll
    for (int e = 0; e < EPT; ++e) {
        long i = c0 + tid + (long)e * NT;
        ra_[e] = i < n ? r[i] : czero<C>();
        xa[e] = i < n ? x[i] : czero<C>();
    }
#pragma unroll 2
    for (int p = 0; p < kk; ++p) {
        const C tc = ts[p], yc = ys[p];
        const C *wp = W + (size_t)p * n;
        const C *zp = Z + (size_t)p * n;
#pragma unroll
        for (int e = 0; e < EPT; ++e) {
            long i = c0 + tid + (long)e * NT;
            if (i < n) {
                cfms(ra_[e], tc, wp[i]);
                cfma(xa[e], yc, zp[i]);
            }
            ra_[e] = canon(ra_[e]);
            xa[e] = canon(xa[e]);
        }
    }
#pragma unroll 4
    for (int p = 0; p <= m - kk; ++p) {
        const C tc = ts[kk + p], yc = ys[kk + p];   // ys[m] = 0: the last Krylov vector is target-side only
        const C *vp = V + (size_t)p * n;
#pragma unroll
        for (int e = 0; e < EPT; ++e) {
            long i = c0 + tid + (long)e * NT;
            if (i < n) {
                const C vv = vp[i];
                cfms(ra_[e], tc, vv);
                cfma(xa[e], yc, vv);
            }
            ra_[e] = canon(ra_[e]);
            xa[e] = canon(xa[e]);
        }
    }
    C ln = czero<C>();
#pragma unroll
    for (int e = 0; e < EPT; ++e) {
        long i = c0 + tid + (long)e * NT;
        ra_[e] = canon(ra_[e]);
        xa[e] = canon(xa[e]);
        if (i < n) {
            r[i] = ra_[e];
            x[i] = xa[e];
        }
        cdotacc(ln, ra_[e], ra_[e]);
    }
    double v[1] = {(double)ln.x};
    if constexpr (std::is_same<C, float2>::value) {
        const float f[1] = {ln.x};
        block_sum_f<1>(f, v, red);
    } else {
        block_sum<1>(v, red);
    }
    double *part = (double *)partials + (size_t)slot * G;
    if (tid == 0) part[chunk] = v[0];
    if (!arrive_last(&tickets[slot], G)) return;
    double tot[1];
    __syncthreads();
    sum_partials<1>(part, G, tot, red);
    if (tid == 0) {
        FinishArgs f{};
        f.mode = FIN_RESIDUAL;
        run_finish(f, s, state[s], tot[0], 0, 0);
        tickets[slot] = 0;
    }
}

// The cycle-end combinations for a batch, SB systems a CTA: each element of the shared W and Z
// is loaded once for the SB systems of the group (k_combine has every system re-read them from
// L2), then each system's own basis.  Per element the operations and their order are
// k_combine's; the norm partials are summed per system as there (last CTA of each system).
template <class R, int SB, int EPT>
__global__ void __launch_bounds__(NT) k_combine_grp(int n, int kk, int m, const typename CT<R>::t *__restrict__ W,
                                                    const typename CT<R>::t *__restrict__ Z,
                                                    const typename CT<R>::t *__restrict__ V0, size_t strideV,
                                                    typename CT<R>::t *__restrict__ r0, size_t strideR,
                                                    typename CT<R>::t *__restrict__ x0, size_t strideX,
                                                    const double2 *__restrict__ t0, const double2 *__restrict__ y0,
                                                    size_t strideC, const int *__restrict__ act, int nsys,
                                                    double2 *__restrict__ partials, unsigned *tickets, SysState *state) {
    using C = typename CT<R>::t;
    const int g0 = blockIdx.x * SB, chunk = blockIdx.y, G = gridDim.y, tid = threadIdx.x;
    const int ns = min(SB, nsys - g0);
    __shared__ C ts[SB][QMAX], ys[SB][QMAX];
    __shared__ double red[SB][NW];
    __shared__ int sys[SB];
    if (tid < SB) sys[tid] = tid < ns ? act[g0 + tid] : act[g0];
    __syncthreads();
    for (int e = tid; e < SB * (m + 1); e += NT) {
        const int g = e / (m + 1), p = e % (m + 1), s = sys[g];
        const R ra = (R)state[s].rho_abs;
        ts[g][p] = from_d<C>(t0[(size_t)s * strideC + p]);
        C yy = p < m ? from_d<C>(y0[(size_t)s * strideC + p]) : czero<C>();
        yy.x *= ra;
        yy.y *= ra;
        ys[g][p] = yy;
    }
    __syncthreads();
    const long c0 = (long)chunk * NT * EPT;
    C ra_[SB][EPT], xa[SB][EPT];
#pragma unroll
    for (int g = 0; g < SB; ++g)
#pragma unroll
        for (int e = 0; e < EPT; ++e) {
            const long i = c0 + tid + (long)e * NT;
            const bool in = g < ns && i < n;
            ra_[g][e] = in ? r0[(size_t)sys[g] * strideR + i] : czero<C>();
            xa[g][e] = in ? x0[(size_t)sys[g] * strideX + i] : czero<C>();
        }
    // Loads go out in batches ahead of their products (WB shared vectors of W and of Z, VB
    // vectors of V_s), so that a thread has 2 WB EPT or VB EPT loads in flight; the products
    // run in the order of the one-vector loop.
    constexpr int WB = 4, VB = 8;
    for (int p0 = 0; p0 < kk; p0 += WB) {
        C wv[WB][EPT], zv[WB][EPT];
#pragma unroll
        for (int u = 0; u < WB; ++u)
#pragma unroll
            for (int e = 0; e < EPT; ++e) {
                const long i = c0 + tid + (long)e * NT;
                const bool ok = p0 + u < kk && i < n;
                wv[u][e] = ok ? W[(size_t)(p0 + u) * n + i] : czero<C>();
                zv[u][e] = ok ? Z[(size_t)(p0 + u) * n + i] : czero<C>();
            }
#pragma unroll
        for (int u = 0; u < WB; ++u) {
            if (p0 + u >= kk) break;
#pragma unroll
            for (int g = 0; g < SB; ++g) {
                const C tc = ts[g][p0 + u], yc = ys[g][p0 + u];
#pragma unroll
                for (int e = 0; e < EPT; ++e) {
                    cfms(ra_[g][e], tc, wv[u][e]);
                    cfma(xa[g][e], yc, zv[u][e]);
                    ra_[g][e] = canon(ra_[g][e]);
                    xa[g][e] = canon(xa[g][e]);
                }
            }
        }
    }
    const int nv = m - kk + 1;
#pragma unroll
    for (int g = 0; g < SB; ++g) {
        if (g >= ns) break;
        const C *V = V0 + (size_t)sys[g] * strideV;
        for (int p0 = 0; p0 < nv; p0 += VB) {
            C vb[VB][EPT];
#pragma unroll
            for (int u = 0; u < VB; ++u)
#pragma unroll
                for (int e = 0; e < EPT; ++e) {
                    const long i = c0 + tid + (long)e * NT;
                    vb[u][e] = (p0 + u < nv && i < n) ? V[(size_t)(p0 + u) * n + i] : czero<C>();
                }
#pragma unroll
            for (int u = 0; u < VB; ++u) {
                if (p0 + u >= nv) break;
                const C tc = ts[g][kk + p0 + u], yc = ys[g][kk + p0 + u];   // ys[m] = 0: target side only
#pragma unroll
                for (int e = 0; e < EPT; ++e) {
                    const long i = c0 + tid + (long)e * NT;
                    if (i < n) {
                        cfms(ra_[g][e], tc, vb[u][e]);
                        cfma(xa[g][e], yc, vb[u][e]);
                    }
                    ra_[g][e] = canon(ra_[g][e]);
                    xa[g][e] = canon(xa[g][e]);
                }
            }
        }
    }
    double v[SB];
    float fv[SB];
#pragma unroll
    for (int g = 0; g < SB; ++g) {
        C ln = czero<C>();
#pragma unroll
        for (int e = 0; e < EPT; ++e) {
            const long i = c0 + tid + (long)e * NT;
            ra_[g][e] = canon(ra_[g][e]);
            xa[g][e] = canon(xa[g][e]);
            if (g < ns && i < n) {
                r0[(size_t)sys[g] * strideR + i] = ra_[g][e];
                x0[(size_t)sys[g] * strideX + i] = xa[g][e];
            }
            cdotacc(ln, ra_[g][e], ra_[g][e]);
        }
        v[g] = (double)ln.x;
        if constexpr (std::is_same<C, float2>::value) fv[g] = ln.x;
    }
    if constexpr (std::is_same<C, float2>::value) block_sum_f<SB>(fv, v, red);
    else block_sum<SB>(v, red);
    if (tid == 0)
        for (int g = 0; g < ns; ++g) ((double *)partials)[(size_t)(g0 + g) * G + chunk] = v[g];
    for (int g = 0; g < ns; ++g) {
        const int slot = g0 + g;
        if (!arrive_last(&tickets[slot], G)) continue;
        double tot[1];
        __syncthreads();
        sum_partials<1>((double *)partials + (size_t)slot * G, G, tot, red);
        if (tid == 0) {
            FinishArgs f{};
            f.mode = FIN_RESIDUAL;
            run_finish(f, sys[g], state[sys[g]], tot[0], 0, 0);
            tickets[slot] = 0;
        }
        __syncthreads();
    }
}

// ----------------------------------------------------------------- deflation-space update
// Z_new = [Z V_lead] vs: m x k complex multiply-adds per element, a compute-bound GEMM.  The
// complex128 engine runs it in double-float on the FP32 pipes (about 2^-48 per operation):
// m k = 1152 complex FP64 multiply-adds per element at GB300's 1 TFLOP/s FP64 rate took 6.5 ms
// a cycle on the 96^3 operator, a fifth of the plain FP64 form's kernel time.  The FP64 operands
// are split into double-float and the results joined back by bit operations, so no FP64
// instruction sits in the element loop.

// Exact float -> double by bit operations (normal floats, zero, inf/nan; subnormals flush to 0).
__device__ __forceinline__ double f2d_bits(float f) {
    const unsigned u = __float_as_uint(f), e = (u >> 23) & 0xffu;
    const unsigned long long sgn = (unsigned long long)(u >> 31) << 63;
    if (e == 0) return __longlong_as_double((long long)sgn);
    const unsigned long long de = e == 0xffu ? 0x7ffull : (unsigned long long)(e - 127u + 1023u);
    return __longlong_as_double((long long)(sgn | de << 52 | (unsigned long long)(u & 0x7fffffu) << 29));
}
// double -> double-float by bit operations: hi = x truncated to 24 significant bits, lo = the
// remaining 29 bits rounded to float (so hi + lo = x to 2^-47 relative; lo has the sign of hi
// and is below ulp(hi), a valid, if unnormalised, pair).  |x| outside [2^-70, 2^70) and zero
// take the conversion instructions.
__device__ __forceinline__ dfr d2df_bits(double x) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    const unsigned hw = (unsigned)(u >> 32), lw = (unsigned)u;
    const int e = (int)((hw >> 20) & 0x7ffu);
    if (e < 1023 - 70 || e >= 1023 + 70) {
        const float h = (float)x;
        return dfr(h, (float)(x - (double)h));
    }
    const unsigned sgn = hw & 0x80000000u;
    const float hi = __uint_as_float(sgn | (unsigned)(e - 1023 + 127) << 23 | ((hw & 0xfffffu) << 3) | (lw >> 29));
    const float scale = __uint_as_float((unsigned)(e - 1075 + 127) << 23);   // 2^(e - 1075), a normal float
    const float lo = (float)(lw & 0x1fffffffu) * scale;
    return dfr(hi, sgn ? -lo : lo);
}

// Working type of the deflation GEMM and the conversions in and out of it.
template <class C> struct ZW { using t = C; };
template <> struct ZW<double2> { using t = dfc; };
__device__ __forceinline__ float2 zin(float2 a) { return a; }
__device__ __forceinline__ dfc zin(dfc a) { return a; }
__device__ __forceinline__ dfc zin(double2 a) {
    dfc c;
    c.x = d2df_bits(a.x);
    c.y = d2df_bits(a.y);
    return c;
}
template <class C> __device__ __forceinline__ C zout(typename ZW<C>::t a) { return a; }
template <> __device__ __forceinline__ double2 zout<double2>(dfc a) {
    return make_double2(f2d_bits(a.x.hi) + f2d_bits(a.x.lo), f2d_bits(a.y.hi) + f2d_bits(a.y.lo));
}
// |a|^2 accumulated in the working real type; converted to double once per thread
__device__ __forceinline__ void zacc_norm(float &s, float2 a) { s = fmaf(a.x, a.x, fmaf(a.y, a.y, s)); }
__device__ __forceinline__ void zacc_norm(dfr &s, dfc a) { s = rfma(a.x, a.x, rfma(a.y, a.y, s)); }

template <class R, int KB>
__global__ void __launch_bounds__(NT) k_zupdate(int n, int kk, int m, int k, int t0, const typename CT<R>::t *__restrict__ Z,
                                                const typename CT<R>::t *__restrict__ V0, size_t strideV,
                                                const int *__restrict__ lead, const double2 *__restrict__ vs,
                                                typename CT<R>::t *__restrict__ Znew, double2 *__restrict__ partials,
                                                unsigned *ticket, double *znorm2) {
    using C = typename CT<R>::t;
    using W = typename ZW<C>::t;
    using WR = decltype(W::x);
    constexpr bool DF = std::is_same<W, dfc>::value;
    const C *__restrict__ V = V0 + (size_t)(*lead) * strideV;
    extern __shared__ unsigned char smraw[];
    W *cs = reinterpret_cast<W *>(smraw);            // m x KB coefficients
    __shared__ double red[KB][NW];
    const int nt = min(KB, k - t0), G = gridDim.x, tid = threadIdx.x;
    for (int i = tid; i < m * KB; i += NT) {
        int p = i / KB, t = i % KB;
        cs[i] = t < nt ? from_d<W>(vs[(size_t)(t0 + t) * m + p]) : czero<W>();
    }
    __syncthreads();
    WR nrm_w[KB];
#pragma unroll
    for (int t = 0; t < KB; ++t) nrm_w[t] = WR(0.f);
    // basis values are loaded PA steps ahead of their products (a ring of raw values), so a
    // thread has PA loads in flight instead of waiting on each one
    constexpr int PA = sizeof(C) == 8 ? 4 : 2;
    auto ld = [&](int p, long i) -> C { return p < kk ? Z[(size_t)p * n + i] : V[(size_t)(p - kk) * n + i]; };
    for (long i = (long)blockIdx.x * NT + tid; i < n; i += (long)G * NT) {
        W acc[KB];
#pragma unroll
        for (int t = 0; t < KB; ++t) acc[t] = czero<W>();
        C pf[PA];
#pragma unroll
        for (int u = 0; u < PA; ++u) pf[u] = u < m ? ld(u, i) : czero<C>();
        for (int p0 = 0; p0 < m; p0 += PA) {
#pragma unroll
            for (int u = 0; u < PA; ++u) {
                const int p = p0 + u;
                if (p < m) {
                    const W b = zin(pf[u]);
                    if (p + PA < m) pf[u] = ld(p + PA, i);
#pragma unroll
                    for (int t = 0; t < KB; ++t) {
                        cfma(acc[t], cs[p * KB + t], b);
                        if constexpr (DF)
                            if ((p & 3) == 3) acc[t] = canon(acc[t]);
                    }
                }
            }
        }
#pragma unroll
        for (int t = 0; t < KB; ++t) {
            acc[t] = canon(acc[t]);
            if (t < nt) Znew[(size_t)(t0 + t) * n + i] = zout<C>(acc[t]);
            zacc_norm(nrm_w[t], acc[t]);
            if constexpr (DF) nrm_w[t] = canon(dfc{nrm_w[t], dfr(0.f, 0.f)}).x;
        }
    }
    // column norms: warp sums in the working type (FP32 or double-float butterflies; FP64 warp
    // arithmetic is slow on GB300), the CTA's warps summed in FP64 by one thread per column, and
    // the last CTA sums the CTAs' partials, one warp per column, in a fixed order
    const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int t = 0; t < KB; ++t) {
        const WR v = warp_sum(nrm_w[t]);
        if (lane == 0) red[t][warp] = (double)v;
    }
    __syncthreads();
    double *part = (double *)partials;
    if (tid < nt) {
        double sacc = 0;
#pragma unroll
        for (int w = 0; w < NW; ++w) sacc += red[tid][w];
        part[(size_t)tid * G + blockIdx.x] = sacc;
    }
    if (!arrive_last(ticket, gridDim.x)) return;
    for (int t = warp; t < nt; t += NW) {
        double sacc = 0;
        for (int g = lane; g < G; g += 32) sacc += __ldcg(part + (size_t)t * G + g);
        sacc = warp_sum(sacc);
        if (lane == 0) znorm2[t0 + t] = sacc;
    }
    if (tid == 0) *ticket = 0;
}

template <class R>
__global__ void __launch_bounds__(NT) k_znormalise(int n, const typename CT<R>::t *__restrict__ Znew,
                                                   const double *__restrict__ znorm2, typename CT<R>::t *__restrict__ Z) {
    using C = typename CT<R>::t;
    const int t = blockIdx.y;
    const R a = (R)(1.0 / sqrt(znorm2[t]));
    for (long i = (long)blockIdx.x * NT + threadIdx.x; i < n; i += (long)gridDim.x * NT) {
        C v = Znew[(size_t)t * n + i];
        v.x *= a;
        v.y *= a;
        Z[(size_t)t * n + i] = v;
    }
}

// ----------------------------------------------------------------- least squares (FP64 Givens)
// H is upper Hessenberg, (m+1) x m, ld m+1.  Column c is stored packed in shared
// memory at off(c) = c(c+3)/2, rows 0..c+1.
__device__ __forceinline__ int hoff(int c) { return c * (c + 3) / 2; }

__global__ void __launch_bounds__(128) k_ls(int m, const double2 *__restrict__ H0, size_t strideH,
                                            const double2 *__restrict__ g0, double2 *__restrict__ y0,
                                            double2 *__restrict__ t0, size_t strideC, const int *__restrict__ act) {
    extern __shared__ double2 sm[];
    const int s = act[blockIdx.x], tid = threadIdx.x, ld = m + 1;
    const double2 *H = H0 + (size_t)s * strideH;
    double2 *Hp = sm;                         // packed Hessenberg
    double2 *gg = sm + hoff(m);               // m+1
    double2 *yy = gg + (m + 1);               // m
    double *cs = (double *)(yy + m);          // m cosines
    double2 *sn = (double2 *)(cs + m + (m & 1));   // m sines (keep 16-byte alignment)
    for (int c = 0; c < m; ++c)
        for (int r = tid; r <= c + 1 && r <= m; r += blockDim.x) Hp[hoff(c) + r] = H[(size_t)c * ld + r];
    for (int r = tid; r <= m; r += blockDim.x) gg[r] = g0[(size_t)s * strideC + r];
    __syncthreads();
    for (int i = 0; i < m; ++i) {
        if (tid == 0) {
            double2 a = Hp[hoff(i) + i], b = Hp[hoff(i) + i + 1];
            double aa = hypot(a.x, a.y), bb = hypot(b.x, b.y);
            double c, rr;
            double2 sv, ph;
            if (bb == 0.0) {
                c = 1.0; sv = make_double2(0, 0); rr = aa; ph = aa > 0 ? make_double2(a.x / aa, a.y / aa) : make_double2(1, 0);
            } else if (aa == 0.0) {
                c = 0.0; sv = make_double2(b.x / bb, -b.y / bb); rr = bb; ph = make_double2(1, 0);
            } else {
                double rho = hypot(aa, bb);
                ph = make_double2(a.x / aa, a.y / aa);
                c = aa / rho;
                // s = ph * conj(b) / rho
                sv = make_double2((ph.x * b.x + ph.y * b.y) / rho, (ph.y * b.x - ph.x * b.y) / rho);
                rr = rho;
            }
            cs[i] = c;
            sn[i] = sv;
            Hp[hoff(i) + i] = make_double2(ph.x * rr, ph.y * rr);
            Hp[hoff(i) + i + 1] = make_double2(0, 0);
            double2 g1 = gg[i], g2 = gg[i + 1];
            // [c s; -conj(s) c] [g1; g2]
            gg[i] = make_double2(c * g1.x + sv.x * g2.x - sv.y * g2.y, c * g1.y + sv.x * g2.y + sv.y * g2.x);
            gg[i + 1] = make_double2(-(sv.x * g1.x + sv.y * g1.y) + c * g2.x, -(sv.x * g1.y - sv.y * g1.x) + c * g2.y);
        }
        __syncthreads();
        const double c = cs[i];
        const double2 sv = sn[i];
        for (int col = i + 1 + tid; col < m; col += blockDim.x) {
            double2 h1 = Hp[hoff(col) + i], h2 = Hp[hoff(col) + i + 1];
            Hp[hoff(col) + i] = make_double2(c * h1.x + sv.x * h2.x - sv.y * h2.y, c * h1.y + sv.x * h2.y + sv.y * h2.x);
            Hp[hoff(col) + i + 1] = make_double2(-(sv.x * h1.x + sv.y * h1.y) + c * h2.x, -(sv.x * h1.y - sv.y * h1.x) + c * h2.y);
        }
        __syncthreads();
    }
    // back substitution R y = g (R = upper m x m part); zero pivots give zero components
    for (int c = m - 1; c >= 0; --c) {
        if (tid == 0) {
            double2 d = Hp[hoff(c) + c], g = gg[c];
            double dd = d.x * d.x + d.y * d.y;
            yy[c] = dd > 0 ? make_double2((g.x * d.x + g.y * d.y) / dd, (g.y * d.x - g.x * d.y) / dd) : make_double2(0, 0);
        }
        __syncthreads();
        const double2 yc = yy[c];
        for (int r = tid; r < c; r += blockDim.x) {
            double2 h = Hp[hoff(c) + r];
            gg[r].x -= h.x * yc.x - h.y * yc.y;
            gg[r].y -= h.x * yc.y + h.y * yc.x;
        }
        __syncthreads();
    }
    for (int c = tid; c < m; c += blockDim.x) y0[(size_t)s * strideC + c] = yy[c];
    // t = H y with the original H
    for (int r = tid; r <= m; r += blockDim.x) {
        double2 acc = make_double2(0, 0);
        for (int c = (r > 0 ? r - 1 : 0); c < m; ++c) {
            double2 h = H[(size_t)c * ld + r], yc = yy[c];
            acc.x += h.x * yc.x - h.y * yc.y;
            acc.y += h.x * yc.y + h.y * yc.x;
        }
        t0[(size_t)s * strideC + r] = acc;
    }
}

// ----------------------------------------------------------------- SVD (one-sided Jacobi, FP32 then double-float)
// Right singular vectors of H ((m+1) x m) by one-sided Jacobi (Hestenes 1958) with the
// round-robin ("circle") ordering of disjoint column pairs, in one CTA:
//   1. FP32 sweeps to FP32 convergence;
//   2. double-float (the FP32 pipes): V made unitary to double-float precision by the
//      second-order polar correction V <- V (I - E/2 + 3 E^2/8), E = V^H V - I, then A = H V;
//   3. double-float sweeps restricted to the pairs with a column of the k smallest singular
//      values, to the FP64 tolerance.
// GB300 retires FP64 at about 1/64 of its FP32 rate; in one CTA that is about one FP64 warp
// instruction per 80 clocks per scheduler, and phases 2 and 3 in native FP64 took 1.4 of the
// 2.0 ms of an m = 40 SVD.

// Pair (p < q) of slot pi in round r (0 <= r < mm - 1) of the circle method over mm (even)
// slots.
__device__ __forceinline__ void circle_pair(int r, int pi, int mm, int &p, int &q) {
    auto pos = [&](int i) {
        if (i == 0) return 0;
        int x = i - 1 + r;                  // < 2 (mm - 1): one conditional subtraction
        if (x >= mm - 1) x -= mm - 1;
        return 1 + x;
    };
    p = pos(pi);
    q = pos(mm - 1 - pi);
    if (p > q) { const int t = p; p = q; q = t; }
}

// QR with column pivoting (Businger and Golub 1965) of A ((m+1) x m, column-major, FP32) in
// place, by Householder reflections in the conventions of LAPACK's xLARFG: on return the upper
// triangle holds R, and column j of R comes from column perm[j] of A.  Pivoting on the largest
// remaining column norm grades R, which lets one-sided Jacobi on R^H converge in about half
// the sweeps it takes on A (Drmac and Veselic 2008).  The partial norms are recomputed after
// each step, not downdated.  pn (m) is scratch; s_c a shared scalar.
__device__ void qrcp_f32(int m, float2 *A, int *perm, float *pn, float2 *s_c) {
    const int rows = m + 1, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    for (int c = warp; c < m; c += nwarps) {
        float a = 0.f;
        for (int r = lane; r < rows; r += 32) { const float2 v = A[(size_t)c * rows + r]; a += v.x * v.x + v.y * v.y; }
        a = warp_sum(a);
        if (lane == 0) { pn[c] = a; perm[c] = c; }
    }
    __syncthreads();
    for (int j = 0; j < m; ++j) {
        float2 *aj = A + (size_t)j * rows;
        if (warp == 0) {
            // pivot: the largest remaining norm, lowest index on ties; swap it into column j
            float best = -1.f;
            int bi = j;
            for (int c = j + lane; c < m; c += 32)
                if (pn[c] > best) { best = pn[c]; bi = c; }
            for (int o = 16; o > 0; o >>= 1) {
                const float ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            if (bi != j) {
                float2 *ap = A + (size_t)bi * rows;
                for (int r = lane; r < rows; r += 32) { const float2 t = aj[r]; aj[r] = ap[r]; ap[r] = t; }
                if (lane == 0) {
                    const int t = perm[j]; perm[j] = perm[bi]; perm[bi] = t;
                    const float u = pn[j]; pn[j] = pn[bi]; pn[bi] = u;
                }
                __syncwarp();
            }
            // reflector H = I - tau v v^H, v = (1, x / (alpha - beta))
            float xn = 0.f;
            for (int r = j + 1 + lane; r < rows; r += 32) xn += aj[r].x * aj[r].x + aj[r].y * aj[r].y;
            xn = warp_sum(xn);
            const float2 al = aj[j];
            float2 tau = make_float2(0.f, 0.f);
            if (xn > 0.f || al.y != 0.f) {
                const float beta = -copysignf(sqrtf(al.x * al.x + al.y * al.y + xn), al.x);
                tau = make_float2((beta - al.x) / beta, -al.y / beta);
                const float2 d = make_float2(al.x - beta, al.y);                  // 1 / (alpha - beta)
                const float id = 1.f / (d.x * d.x + d.y * d.y);
                const float2 sc = make_float2(d.x * id, -d.y * id);
                for (int r = j + 1 + lane; r < rows; r += 32) {
                    const float2 x = aj[r];
                    aj[r] = make_float2(x.x * sc.x - x.y * sc.y, x.x * sc.y + x.y * sc.x);
                }
                __syncwarp();
                if (lane == 0) aj[j] = make_float2(beta, 0.f);
            }
            if (lane == 0) *s_c = tau;
        }
        __syncthreads();
        const float2 tau = *s_c;
        for (int c = j + 1 + warp; c < m; c += nwarps) {   // a_c <- (I - conj(tau) v v^H) a_c
            float2 *ac = A + (size_t)c * rows;
            float wr = 0.f, wi = 0.f;
            for (int r = j + lane; r < rows; r += 32) {
                const float2 v = (r == j) ? make_float2(1.f, 0.f) : aj[r], a = ac[r];
                wr += v.x * a.x + v.y * a.y;
                wi += v.x * a.y - v.y * a.x;
            }
            wr = warp_sum(wr);
            wi = warp_sum(wi);
            const float fr = tau.x * wr + tau.y * wi, fi = tau.x * wi - tau.y * wr;   // conj(tau) w
            float s = 0.f;
            for (int r = j + lane; r < rows; r += 32) {
                const float2 v = (r == j) ? make_float2(1.f, 0.f) : aj[r];
                float2 a = ac[r];
                a.x -= fr * v.x - fi * v.y;
                a.y -= fr * v.y + fi * v.x;
                ac[r] = a;
                if (r > j) s += a.x * a.x + a.y * a.y;
            }
            s = warp_sum(s);
            if (lane == 0) pn[c] = s;
        }
        __syncthreads();
    }
}

// The circle schedule as a table: entry round * (mm/2) + pi = p | q << 8 (p < q < mm <= 256).
// With `only`, each round keeps just the pairs with a flagged column, packed to the front, and
// cnt[round] says how many.
__device__ void pair_table(int m, unsigned short *tab, int *cnt, const unsigned char *only) {
    const int mm = m + (m & 1), npairs = mm / 2;
    for (int r = threadIdx.x; r < mm - 1; r += blockDim.x) {
        int n = 0;
        for (int pi = 0; pi < npairs; ++pi) {
            int p, q;
            circle_pair(r, pi, mm, p, q);
            if (!only || (q < m && (only[p] || only[q]))) tab[r * npairs + n++] = (unsigned short)(p | (q << 8));
        }
        if (cnt) cnt[r] = n;
    }
}

// 1/sqrt(x) in FP32 to about an ulp: the hardware estimate and one Newton step.
__device__ __forceinline__ float rsqrt_nr(float x) {
    const float r = rsqrtf(x);
    return r * fmaf(-0.5f * x * r, r, 1.5f);
}

// Jacobi rotation tangent t = sign(zeta) / (|zeta| + sqrt(1 + zeta^2)), zeta = (b - a) / (2 |gamma|):
// the root of t^2 + 2 zeta t - 1 of smaller magnitude.  Above 2^40, t = 1 / (2 zeta) to FP32
// precision (and zeta^2 could overflow).
__device__ __forceinline__ float jacobi_t(float zeta) {
    const float az = fabsf(zeta);
    if (az > 0x1p40f) return __fdividef(0.5f, zeta);
    const float z2 = fmaf(az, az, 1.f);
    return __fdividef((zeta >= 0.f) ? 1.f : -1.f, az + z2 * rsqrtf(z2));
}

// Sweeps of FP32 one-sided Jacobi on A (rows x m) accumulating V (m x m; none when V is null),
// both column-major with leading dimensions rows and m.  One warp per column pair, every lane
// computing the rotation parameters; the pairs of each round come from `tab` (p | q << 8,
// p < q, built by pair_table), which takes the schedule arithmetic off the critical path of a
// round.  The angle only has to shrink the off-diagonal element (the double-float phase
// finishes the job), so it uses the hardware estimates; c and the phase of gamma are
// Newton-refined, which keeps each rotation unitary to about an ulp.
__device__ int jacobi_sweeps_f32(int m, int rows, float2 *A, float2 *V, float *nrm, float tol, int max_sweeps,
                                 int *s_flag, float *s_off, const unsigned short *tab) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    const int mm = m + (m & 1), npairs = mm / 2;
    const float tol2 = tol * tol;
    int sweep = 0;
    for (; sweep < max_sweeps; ++sweep) {
        for (int c = warp; c < m; c += nwarps) {   // column norms, refreshed every sweep
            float a = 0;
            for (int r = lane; r < rows; r += 32) { float2 v = A[(size_t)c * rows + r]; a += v.x * v.x + v.y * v.y; }
            a = warp_sum(a);
            if (lane == 0) nrm[c] = a;
        }
        if (tid == 0) { *s_flag = 0; *s_off = 0.f; }
        __syncthreads();
        float wmax = 0.f;                           // largest relative off-diagonal this warp saw
        for (int round = 0; round < mm - 1; ++round) {
            for (int pi = warp; pi < npairs; pi += nwarps) {
                const unsigned e = tab[round * npairs + pi];
                const int p = e & 0xff, q = e >> 8;
                if (q >= m) continue;
                float gr = 0, gi = 0;
                for (int r = lane; r < rows; r += 32) {
                    float2 ap = A[(size_t)p * rows + r], aq = A[(size_t)q * rows + r];
                    gr += ap.x * aq.x + ap.y * aq.y;
                    gi += ap.x * aq.y - ap.y * aq.x;
                }
                gr = warp_sum(gr);
                gi = warp_sum(gi);
                const float a = nrm[p], b = nrm[q];
                const float g2 = gr * gr + gi * gi;
                if (!(g2 > tol2 * a * b)) continue;   // |gamma| / sqrt(a b) <= tol, or zero
                const float ig = rsqrt_nr(g2), ag = g2 * ig;
                wmax = fmaxf(wmax, ag * rsqrtf(a * b));
                const float pr = gr * ig, pim = -gi * ig;
                const float zeta = (b - a) * 0.5f * ig;
                const float tt = jacobi_t(zeta);
                const float c = rsqrt_nr(fmaf(tt, tt, 1.f)), sn = c * tt;
                for (int r = lane; r < rows; r += 32) {
                    float2 ap = A[(size_t)p * rows + r], aq0 = A[(size_t)q * rows + r];
                    const float2 aq = make_float2(aq0.x * pr - aq0.y * pim, aq0.x * pim + aq0.y * pr);
                    A[(size_t)p * rows + r] = make_float2(c * ap.x - sn * aq.x, c * ap.y - sn * aq.y);
                    A[(size_t)q * rows + r] = make_float2(sn * ap.x + c * aq.x, sn * ap.y + c * aq.y);
                }
                for (int r = lane; V && r < m; r += 32) {
                    float2 vp = V[(size_t)p * m + r], vq0 = V[(size_t)q * m + r];
                    const float2 vq = make_float2(vq0.x * pr - vq0.y * pim, vq0.x * pim + vq0.y * pr);
                    V[(size_t)p * m + r] = make_float2(c * vp.x - sn * vq.x, c * vp.y - sn * vq.y);
                    V[(size_t)q * m + r] = make_float2(sn * vp.x + c * vq.x, sn * vp.y + c * vq.y);
                }
                if (lane == 0) {
                    nrm[p] = a - tt * ag;
                    nrm[q] = b + tt * ag;
                }
            }
            __syncthreads();
        }
        if (lane == 0 && wmax > 0.f) {
            *s_flag = 1;
            atomicMax((int *)s_off, __float_as_int(wmax));
        }
        __syncthreads();
        if (!*s_flag) break;
        // quadratic convergence: after a sweep whose largest relative off-diagonal was d,
        // the next is of order d^2; stop once that is below the tolerance
        const float d = *s_off;
        __syncthreads();
        if (d * d < tol * 1e-2f) { ++sweep; break; }
    }
    return sweep + 1;
}

// Exact float product as a double-float (FMA two-product).
__device__ __forceinline__ dfr df_prod(float a, float b) {
    const float p = a * b;
    return dfr(p, fmaf(a, b, -p));
}
// acc + a * b for floats a, b, the product exact.
__device__ __forceinline__ dfr df_acc(dfr acc, float a, float b) {
    const float p = a * b, pe = fmaf(a, b, -p);
    const float s = p + acc.hi, bb = s - p;
    return df_renorm(s, ((p - (s - bb)) + (acc.hi - bb)) + (pe + acc.lo));
}
// 1 / sqrt(x) for a double-float x > 0: the FP32 estimate r0 times 1 - e/2 + 3e^2/8 (the
// binomial series of (1 + e)^(-1/2)), e = x r0^2 - 1 kept as the exact pair (hi - 1, lo)
// (hi - 1 is exact for hi in [1/2, 2], Sterbenz).  |e| < 1e-6, so the truncation is O(1e-19).
__device__ __forceinline__ dfr df_rsqrt(dfr x) {
    const float r0 = rsqrtf(x.hi);
    const dfr u = x * df_prod(r0, r0);
    const float eh = u.hi - 1.0f, el = u.lo;
    return dfr(r0, 0.0f) * (dfr(1.0f, 0.0f) + dfr(-0.5f * eh, fmaf(0.375f * eh, eh, -0.5f * el)));
}
__device__ __forceinline__ dfc to_dfc(double2 a) {
    dfc c;
    c.x = dfr(a.x);
    c.y = dfr(a.y);
    return c;
}

// Columns P, Q (length len) <- (c P - s w Q, s P + c w Q), w = wr + i wi.
__device__ __forceinline__ void rotate_df(dfc *P, dfc *Q, int len, int lane, dfr c, dfr s, dfr wr, dfr wi) {
    for (int r = lane; r < len; r += 32) {
        const dfc ap = P[r], q0 = Q[r];
        const dfr qx = q0.x * wr - q0.y * wi, qy = q0.x * wi + q0.y * wr;
        dfc np_, nq_;
        np_.x = c * ap.x - s * qx;
        np_.y = c * ap.y - s * qy;
        nq_.x = s * ap.x + c * qx;
        nq_.y = s * ap.y + c * qy;
        P[r] = np_;
        Q[r] = nq_;
    }
}
// a + b for a double-float a and a float b.
__device__ __forceinline__ dfr df_addf(dfr a, float b) {
    const float s = a.hi + b, bb = s - a.hi;
    return df_renorm(s, ((a.hi - (s - bb)) + (b - bb)) + a.lo);
}
// Small-angle rotation, |t| < 2^-30: c = 1 and s = t to double-float precision, and column Q
// takes the unit phase conj(w), so (P, Q) <- (P - g Q, Q + conj(g) P) with g = t w, unitary up
// to |t|^2 < 1e-18.  g Q and conj(g) P are below 1e-9 of the columns, so FP32 products of
// the leading halves are exact enough.
__device__ __forceinline__ void rotate_small_df(dfc *P, dfc *Q, int len, int lane, float gr, float gi) {
    for (int r = lane; r < len; r += 32) {
        const dfc ap = P[r], aq = Q[r];
        dfc np_, nq_;
        np_.x = df_addf(ap.x, -fmaf(gr, aq.x.hi, -gi * aq.y.hi));
        np_.y = df_addf(ap.y, -fmaf(gr, aq.y.hi, gi * aq.x.hi));
        nq_.x = df_addf(aq.x, fmaf(gr, ap.x.hi, gi * ap.y.hi));
        nq_.y = df_addf(aq.y, fmaf(gr, ap.y.hi, -gi * ap.x.hi));
        P[r] = np_;
        Q[r] = nq_;
    }
}
// Rotation parameters of the pair (p, q) from gamma = <a_p, a_q> and the squared column norms
// a, b (double-float).  Returns false when the pair needs no rotation (relative off-diagonal
// at most tol, or zero).  Otherwise t is the tangent of the rotation (FP32 accuracy), ag =
// |gamma|, and (gx, gy) * igs is the unit complex gamma / |gamma|: gamma is scaled by a power
// of two into [1/2, 2) first, so nothing underflows.
__device__ __forceinline__ bool polish_params(dfr gr, dfr gi, dfr a, dfr b, float tol, float &t, float &ag,
                                              float &gx, float &gy, float &igs) {
    const int ex = max(-120, min(120, ilogbf(fmaxf(fabsf(gr.hi), fabsf(gi.hi)))));
    const float down = __int_as_float((127 - ex) << 23), up = __int_as_float((127 + ex) << 23);
    gx = gr.hi * down;
    gy = gi.hi * down;
    const float g2 = gx * gx + gy * gy;
    if (!(g2 > 0.f)) return false;
    igs = rsqrt_nr(g2);
    ag = g2 * igs * up;
    if (!(ag * rsqrtf(a.hi) * rsqrtf(b.hi) > tol)) return false;
    t = jacobi_t((b - a).hi * 0.5f * igs * down);   // zeta = (b - a) / (2 |gamma|)
    return true;
}

// gamma = <a_p, a_q> over len rows, one thread, in double-float.
__device__ __forceinline__ void dot_df(const dfc *P, const dfc *Q, int len, dfr &gr, dfr &gi) {
    gr = dfr(0.f, 0.f);
    gi = dfr(0.f, 0.f);
    for (int r = 0; r < len; ++r) {
        const dfc ap = P[r], aq = Q[r];
        gr = rfma(ap.x, aq.x, gr);
        gr = rfma(ap.y, aq.y, gr);
        gi = rfma(ap.x, aq.y, gi);
        gi = rfma(-ap.y, aq.x, gi);
    }
    gr = df_renorm(gr.hi, gr.lo);
    gi = df_renorm(gi.hi, gi.lo);
}

// One sweep's worth of small rotations applied at once.  When every rotation of a sweep has
// |t| < 2^-26, the sweep is V <- V (I + T + T^2/2 + ...) with T skew-Hermitian and
// T[q][p] = -g, T[p][q] = conj(g), g = t conj(gamma) / |gamma|, for every pair p < q with a
// flagged column.  Products of two rotations are O(t^2) < 2e-16, so all gammas can come from
// the current A and all updates can be applied together, with no rounds; the diagonal of T^2/2
// (-sum |g|^2 / 2 per column) is kept, which makes the update unitary to O(t^3).  The sums run
// in double-float (the FP32 coefficients times the leading halves of V, exactly).  Only the
// flagged columns of V are updated: they are the output, and A is not needed again (its norms
// move by O(t |gamma|), so the norms the sweep started from stay exact to that order).  fl lists
// the k flagged columns; C (k x m) is scratch, and the k x m sums go in place of A once every
// gamma is formed.  Returns false, having changed nothing, when some rotation is not small
// (the caller then runs an ordinary sweep).
__device__ bool polish_small_all(int m, dfc *A, dfc *V, int ldv, const dfr *nrm, float tol, const int *fl, int k,
                                 float2 *C, int *s_big) {
    const int rows = m + 1, tid = threadIdx.x, nt = blockDim.x;
    dfc *D = A;
    if (tid == 0) *s_big = 0;
    __syncthreads();
    for (int e = tid; e < k * m; e += nt) {   // C[f][q]: coefficient of column q added to flagged f
        const int f = fl[e / m], q0 = e % m;
        float2 coef = make_float2(0.f, 0.f);
        if (q0 != f) {
            const int p = min(f, q0), q = max(f, q0);
            dfr gr, gi;
            dot_df(A + (size_t)p * rows, A + (size_t)q * rows, rows, gr, gi);
            float t, ag, gx, gy, igs;
            if (polish_params(gr, gi, nrm[p], nrm[q], tol, t, ag, gx, gy, igs)) {
                if (!(fabsf(t) < 0x1p-26f)) atomicOr(s_big, 1);
                const float g_r = t * gx * igs, g_i = -t * gy * igs;   // g = t conj(gamma) / |gamma|
                coef = (f == p) ? make_float2(-g_r, -g_i) : make_float2(g_r, -g_i);
            }
        }
        C[e] = coef;
    }
    __syncthreads();
    if (*s_big) return false;
    for (int e = tid; e < k * m; e += nt) {   // D[f][r] = sum_q C[f][q] V[r][q] - |C[f]|^2 / 2 V[r][f]
        const int fi = e / m, r = e % m;
        dfr dx(0.f, 0.f), dy(0.f, 0.f);
        float lx = 0.f, ly = 0.f, kap = 0.f;
        for (int q = 0; q < m; ++q) {
            const float2 c = C[(size_t)fi * m + q];
            const dfc v = V[(size_t)q * ldv + r];
            dx = df_acc(df_acc(dx, c.x, v.x.hi), -c.y, v.y.hi);
            dy = df_acc(df_acc(dy, c.x, v.y.hi), c.y, v.x.hi);
            lx = fmaf(c.x, v.x.lo, fmaf(-c.y, v.y.lo, lx));
            ly = fmaf(c.x, v.y.lo, fmaf(c.y, v.x.lo, ly));
            kap = fmaf(c.x, c.x, fmaf(c.y, c.y, kap));
        }
        const dfc vf = V[(size_t)fl[fi] * ldv + r];
        dfc d;
        d.x = df_addf(dx, fmaf(-0.5f * kap, vf.x.hi, lx));
        d.y = df_addf(dy, fmaf(-0.5f * kap, vf.y.hi, ly));
        D[e] = d;
    }
    __syncthreads();
    for (int e = tid; e < k * m; e += nt) {
        dfc &v = V[(size_t)fl[e / m] * ldv + e % m];
        v.x = v.x + D[e].x;
        v.y = v.y + D[e].y;
    }
    __syncthreads();
    return true;
}

// Double-float one-sided Jacobi sweeps on A ((m+1) x m, leading dimension m+1) accumulating V
// (m x m, leading dimension ldv), restricted to the pairs with a flagged column: rotating each
// flagged column against every other one makes it orthogonal to all columns of A, which
// decouples the flagged block exactly; rotations among unflagged columns cannot change it.
// tab / cnt hold each round's pairs with a flagged column, packed (pair_table), so the active
// pairs go to consecutive warps and spread evenly over the four schedulers.  The angle comes
// from FP32-rounded parameters (b - a formed in double-float first), so a rotation leaves
// about 1e-7 of its off-diagonal element and a sweep still squares the largest one; c, s and
// the phase of gamma are unitary to double-float precision, which keeps V unitary.  From the
// second sweep on, a sweep of small rotations is applied at once (polish_small_all).
// Returns the number of sweeps.
// Returns the number of sweeps; nrm then holds the squared column norms of the result (A itself
// may have been overwritten).
__device__ int jacobi_polish_df(int m, dfc *A, dfc *V, int ldv, dfr *nrm, float tol, int max_sweeps, int *s_flag,
                                float *s_off, const unsigned short *tab, const int *cnt, const int *fl, int k,
                                float2 *C) {
    const int rows = m + 1, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    const int mm = m + (m & 1), npairs = mm / 2;
    __shared__ int s_big;
    auto column_norms = [&]() {
        for (int c = warp; c < m; c += nwarps) {
            dfr a(0.f, 0.f);
            for (int r = lane; r < rows; r += 32) {
                const dfc v = A[(size_t)c * rows + r];
                a = fma(v.x, v.x, a);
                a = fma(v.y, v.y, a);
            }
            a = warp_sum(a);
            if (lane == 0) nrm[c] = a;
        }
    };
    int sweep = 0;
    bool fresh = false;                     // nrm matches the current A
    for (; sweep < max_sweeps; ++sweep) {
        column_norms();
        if (tid == 0) { *s_flag = 0; *s_off = 0.f; }
        __syncthreads();
        if (sweep > 0 && polish_small_all(m, A, V, ldv, nrm, tol, fl, k, C, &s_big)) {
            ++sweep;
            fresh = true;
            break;
        }
        float wmax = 0.f;
        for (int round = 0; round < mm - 1; ++round) {
            for (int j = warp; j < cnt[round]; j += nwarps) {
                const unsigned e = tab[round * npairs + j];
                const int p = e & 0xff, q = e >> 8;
                dfc *Ap = A + (size_t)p * rows, *Aq = A + (size_t)q * rows;
                dfr gr(0.f, 0.f), gi(0.f, 0.f);
                for (int r = lane; r < rows; r += 32) {   // unnormalised chains, canonical below
                    const dfc ap = Ap[r], aq = Aq[r];
                    gr = rfma(ap.x, aq.x, gr);
                    gr = rfma(ap.y, aq.y, gr);
                    gi = rfma(ap.x, aq.y, gi);
                    gi = rfma(-ap.y, aq.x, gi);
                }
                gr = warp_sum(df_renorm(gr.hi, gr.lo));   // identical in every lane: the two-sum is symmetric
                gi = warp_sum(df_renorm(gi.hi, gi.lo));
                const dfr a = nrm[p], b = nrm[q];
                float t, ag, gx, gy, igs;
                if (!polish_params(gr, gi, a, b, tol, t, ag, gx, gy, igs)) continue;
                wmax = fmaxf(wmax, ag * rsqrtf(a.hi) * rsqrtf(b.hi));
                if (fabsf(t) < 0x1p-30f) {
                    const float wr = gx * igs, wi = -gy * igs;
                    rotate_small_df(Ap, Aq, rows, lane, t * wr, t * wi);
                    rotate_small_df(V + (size_t)p * ldv, V + (size_t)q * ldv, m, lane, t * wr, t * wi);
                } else {
                    const dfr c = df_rsqrt(dfr(1.f, 0.f) + df_prod(t, t));
                    const dfr s = c * dfr(t, 0.f);
                    const dfr ig = df_rsqrt(df_prod(gx, gx) + df_prod(gy, gy));
                    const dfr wr = dfr(gx, 0.f) * ig, wi = dfr(-gy, 0.f) * ig;
                    rotate_df(Ap, Aq, rows, lane, c, s, wr, wi);
                    rotate_df(V + (size_t)p * ldv, V + (size_t)q * ldv, m, lane, c, s, wr, wi);
                }
                if (lane == 0) {
                    const dfr tg = df_prod(t, ag);
                    nrm[p] = a - tg;
                    nrm[q] = b + tg;
                }
            }
            __syncthreads();
        }
        if (lane == 0 && wmax > 0.f) {
            *s_flag = 1;
            atomicMax((int *)s_off, __float_as_int(wmax));
        }
        __syncthreads();
        if (!*s_flag) {                     // no rotation: the norms are the ones computed above
            fresh = true;
            break;
        }
        const float d = *s_off;
        __syncthreads();
        if (d * d < tol * 1e-2f) { ++sweep; break; }
    }
    if (!fresh) {
        column_norms();
        __syncthreads();
    }
    return sweep + 1;
}

// Working storage of k_svd, three regions of 16 (m+1) m bytes (shared memory when it fits):
//   Ad  (m+1) x m double-float complex, A = H V;
//   Vd  m x m, leading dimension m | 1 (odd, so the column-strided reads of V^H V hit
//       distinct banks);
//   Sc  scratch: the FP32 A and V of phase 1, then the FP32 E and E^2, then V F, then H as
//       double-float (E and F live in Ad until A is formed).
__host__ __device__ inline size_t svd_work_bytes(int m) { return 3 * sizeof(dfc) * (size_t)(m + 1) * m; }

__global__ void __launch_bounds__(1024) k_svd(int m, int k, const double2 *__restrict__ H0, size_t strideH,
                                              const int *__restrict__ lead, double2 *__restrict__ vs,
                                              double *__restrict__ sigma, double2 *__restrict__ gwork, int use_smem,
                                              int *sweeps_out) {
    const double2 *__restrict__ H = H0 + (size_t)(*lead) * strideH;
    extern __shared__ __align__(16) unsigned char svd_sm[];
    const int rows = m + 1, tid = threadIdx.x, nt = blockDim.x, ldv = m | 1;
    unsigned char *base = use_smem ? svd_sm : (unsigned char *)gwork;
    dfc *Ad = (dfc *)base;
    dfc *Vd = Ad + (size_t)rows * m;
    dfc *Sc = Vd + (size_t)rows * m;
    float2 *A32 = (float2 *)Sc;
    float2 *V32 = A32 + (size_t)rows * m;
    __shared__ dfr nrmd[168];
    __shared__ float nrm32[168];
    __shared__ int s_flag, slot_col[168];
    __shared__ float s_off;
    __shared__ unsigned char small_col[168];
    __shared__ int s_emax, s_bad, flag_list[168], perm[168];
    __shared__ float2 s_c;
    // H scaled by the power of two that brings its largest entry into [1, 2): exact, and it
    // keeps the FP32 phase clear of overflow and underflow whatever the operator's scale
    if (tid == 0) s_emax = 0;
    __syncthreads();
    int em = 0;
    for (int i = tid; i < rows * m; i += nt) {
        const double2 h = H[i];
        em = max(em, (int)((__double_as_longlong(h.x) >> 52) & 0x7ff));
        em = max(em, (int)((__double_as_longlong(h.y) >> 52) & 0x7ff));
    }
    atomicMax(&s_emax, em);
    __syncthreads();
    const int eb = (s_emax == 0 || s_emax == 0x7ff) ? 1023 : min(max(2046 - s_emax, 1), 2046);
    const double sc = __longlong_as_double((long long)eb << 52);
    for (int i = tid; i < rows * m; i += nt) A32[i] = make_float2((float)(H[i].x * sc), (float)(H[i].y * sc));
    pair_table(m, (unsigned short *)Vd, nullptr, nullptr);   // Vd is free until phase 2
    if (tid == 0) s_bad = 0;
    __syncthreads();
    // 1. FP32.  H P = Q R (column pivoting), then one-sided Jacobi on X = R^H with no
    // accumulation: R^H U = V_R Sigma, so the columns of the result are the right singular
    // vectors of R scaled by the singular values, and H's are V = P V_R.  Should a column come
    // out too small to normalise (singular values below ~1e-15 of the largest), the phase is
    // redone as Jacobi on H accumulating V.
    const float tol32 = 4.0f * 1.1920929e-7f * m;
    const unsigned short *tab32 = (const unsigned short *)Vd;
    qrcp_f32(m, A32, perm, nrm32, &s_c);
    float2 *X = V32;                        // m x m, leading dimension m
    for (int e = tid; e < m * m; e += nt) { // X[i][j] = conj(R[j][i]), lower triangular
        const int i = e % m, j = e / m;
        const float2 r = A32[(size_t)i * rows + j];
        X[e] = i >= j ? make_float2(r.x, -r.y) : make_float2(0.f, 0.f);
    }
    __syncthreads();
    int s32 = jacobi_sweeps_f32(m, m, X, nullptr, nrm32, tol32, 40, &s_flag, &s_off, tab32);
    {
        const int lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
        for (int c = warp; c < m; c += nwarps) {
            float a = 0.f;
            for (int r = lane; r < m; r += 32) { const float2 v = X[(size_t)c * m + r]; a += v.x * v.x + v.y * v.y; }
            a = warp_sum(a);
            if (lane == 0) {
                nrm32[c] = a;
                if (!(a > 1e-30f)) s_bad = 1;
            }
        }
    }
    __syncthreads();
    float2 *V1 = A32;                       // the FP32 right singular vectors, m x m, leading dimension m
    if (!s_bad) {
        for (int e = tid; e < m * m; e += nt) {   // V[perm[j]][c] = X[j][c] / |x_c|
            const int j = e % m, c = e / m;
            const float2 x = X[e];
            const float s = rsqrt_nr(nrm32[c]);
            V1[(size_t)c * m + perm[j]] = make_float2(x.x * s, x.y * s);
        }
    } else {
        for (int i = tid; i < rows * m; i += nt) A32[i] = make_float2((float)(H[i].x * sc), (float)(H[i].y * sc));
        for (int i = tid; i < m * m; i += nt) V32[i] = make_float2((i % m) == (i / m) ? 1.f : 0.f, 0.f);
        __syncthreads();
        s32 = 100 + jacobi_sweeps_f32(m, rows, A32, V32, nrm32, tol32, 40, &s_flag, &s_off, tab32);
        V1 = V32;
    }
    __syncthreads();
    // the k columns of smallest norm (smallest singular values) after the FP32 phase; a NaN
    // (from a non-finite Hessenberg) sorts as -inf, so the order stays total and exactly k
    // columns are flagged whatever the input
    auto key32 = [](float v) { return v == v ? v : -INFINITY; };
    for (int c = tid; c < m; c += nt) {
        const float s = key32(nrm32[c]);
        int below = 0;
        for (int c2 = 0; c2 < m; ++c2) {
            const float s2 = key32(nrm32[c2]);
            below += (s2 < s) || (s2 == s && c2 < c);
        }
        small_col[c] = below < k ? 1 : 0;
    }
    // 2. Vd = V32 (exact); E = V^H V - I; V <- V (I + F), F = -E/2 + 3/8 E^2 - 5/16 E^3 (the
    // binomial series of (I + E)^(-1/2)): V^H V = I + O(|E|^4).  |E| is about 1e-5 after the
    // FP32 phase, so E^2 and E^3 need only FP32; E itself is double-float.
    for (int i = tid; i < m * m; i += nt) {
        const float2 v = V1[i];
        dfc d;
        d.x = dfr(v.x, 0.f);
        d.y = dfr(v.y, 0.f);
        Vd[(size_t)(i / m) * ldv + i % m] = d;
    }
    __syncthreads();
    dfc *E = Ad;                            // m x m, leading dimension m; E[i][j] = <v_i, v_j> - d_ij
    float2 *Eh = (float2 *)Sc, *E2 = Eh + (size_t)m * m;   // its leading halves, and E^2
    for (int idx = tid; idx < m * (m + 1) / 2; idx += nt) {
        int j = 0, i = idx;                 // lower triangle i >= j, column by column
        while (i >= m - j) { i -= m - j; ++j; }
        i += j;                             // lanes over i: columns i at stride ldv (odd)
        const dfc *vi = Vd + (size_t)i * ldv, *vj = Vd + (size_t)j * ldv;
        dfr gr(i == j ? -1.f : 0.f, 0.f), gi(0.f, 0.f);
        for (int r = 0; r < m; ++r) {       // conj(v_ri) v_rj; the entries are floats (lo = 0)
            const dfc x = vi[r], y = vj[r]; // whole 16-byte elements: 4 wavefronts, no conflict
            gr = df_acc(df_acc(gr, x.x.hi, y.x.hi), x.y.hi, y.y.hi);
            gi = df_acc(df_acc(gi, x.x.hi, y.y.hi), -x.y.hi, y.x.hi);
        }
        dfc eij, eji;                       // E[i][j] = <v_i, v_j>, E[j][i] its conjugate
        eij.x = gr;
        eij.y = gi;
        eji.x = gr;
        eji.y = -gi;
        E[(size_t)j * m + i] = eij;         // column-major
        E[(size_t)i * m + j] = eji;
        Eh[(size_t)j * m + i] = make_float2(gr.hi, gi.hi);
        Eh[(size_t)i * m + j] = make_float2(gr.hi, -gi.hi);
    }
    __syncthreads();
    for (int e = tid; e < m * m; e += nt) {
        const int i = e % m, j = e / m;     // (E E)[i][j] = sum_l E[i][l] E[l][j], lanes over i
        float sx = 0.f, sy = 0.f;
        for (int l = 0; l < m; ++l) {
            const float2 x = Eh[(size_t)l * m + i], y = Eh[(size_t)j * m + l];
            sx = fmaf(x.x, y.x, fmaf(-x.y, y.y, sx));
            sy = fmaf(x.x, y.y, fmaf(x.y, y.x, sy));
        }
        E2[e] = make_float2(sx, sy);
    }
    __syncthreads();
    for (int e = tid; e < m * m; e += nt) { // F in place of E
        const int i = e % m, j = e / m;     // (E E^2)[i][j]
        float sx = 0.f, sy = 0.f;
        for (int l = 0; l < m; ++l) {
            const float2 x = Eh[(size_t)l * m + i], y = E2[(size_t)j * m + l];
            sx = fmaf(x.x, y.x, fmaf(-x.y, y.y, sx));
            sy = fmaf(x.x, y.y, fmaf(x.y, y.x, sy));
        }
        const float2 q = E2[e];
        dfc f = E[e];
        f.x = dfr(-0.5f * f.x.hi, -0.5f * f.x.lo) + dfr(fmaf(0.375f, q.x, -0.3125f * sx), 0.f);
        f.y = dfr(-0.5f * f.y.hi, -0.5f * f.y.lo) + dfr(fmaf(0.375f, q.y, -0.3125f * sy), 0.f);
        E[e] = f;
    }
    __syncthreads();
    dfc *T = Sc;                            // m x m, leading dimension m
    for (int e = tid; e < m * m; e += nt) {
        const int i = e % m, j = e / m;     // T[i][j] = sum_l V[i][l] F[l][j]
        dfr sx(0.f, 0.f), sy(0.f, 0.f);
        for (int l = 0; l < m; ++l) {
            const dfc v = Vd[(size_t)l * ldv + i], f = E[(size_t)j * m + l];
            sx = fma(dfr(v.x.hi, 0.f), f.x, sx);
            sx = fma(dfr(-v.y.hi, 0.f), f.y, sx);
            sy = fma(dfr(v.x.hi, 0.f), f.y, sy);
            sy = fma(dfr(v.y.hi, 0.f), f.x, sy);
        }
        T[e].x = sx;
        T[e].y = sy;
    }
    __syncthreads();
    for (int e = tid; e < m * m; e += nt) {
        dfc &v = Vd[(size_t)(e / m) * ldv + e % m];
        v.x = v.x + T[e].x;
        v.y = v.y + T[e].y;
    }
    __syncthreads();
    dfc *Hd = Sc;                           // H as double-float, (m+1) x m
    for (int i = tid; i < rows * m; i += nt) Hd[i] = to_dfc(make_double2(H[i].x * sc, H[i].y * sc));
    __syncthreads();
    for (int e = tid; e < rows * m; e += nt) {
        const int r = e % rows, c = e / rows;   // A[r][c] = sum_p H[r][p] V[p][c]
        dfr sx(0.f, 0.f), sy(0.f, 0.f);
        for (int p = 0; p < m; ++p) {
            const dfc h = Hd[(size_t)p * rows + r], v = Vd[(size_t)c * ldv + p];
            sx = fma(h.x, v.x, sx);
            sx = fma(-h.y, v.y, sx);
            sy = fma(h.x, v.y, sy);
            sy = fma(h.y, v.x, sy);
        }
        Ad[e].x = sx;
        Ad[e].y = sy;
    }
    __syncthreads();
    // 3. double-float polish of the k smallest.  Sc (H no longer needed) takes the packed pair
    // table of the flagged pairs, its counts, and the k x m coefficients of polish_small_all.
    const int mm = m + (m & 1);
    unsigned short *ptab = (unsigned short *)Sc;
    int *pcnt = (int *)(((uintptr_t)(ptab + (size_t)(mm - 1) * (mm / 2)) + 15) & ~(uintptr_t)15);
    float2 *coefs = (float2 *)(((uintptr_t)(pcnt + mm) + 15) & ~(uintptr_t)15);
    pair_table(m, ptab, pcnt, small_col);
    for (int c = tid; c < m; c += nt)
        if (small_col[c]) {
            int idx = 0;
            for (int c2 = 0; c2 < c; ++c2) idx += small_col[c2];
            flag_list[idx] = c;
        }
    __syncthreads();
    // Two sweeps when the FP32 vectors are good (the 64 x 64 Helmholtz Hessenbergs); where FP32
    // could not resolve the small singular values (condition ~1e6 and up) it takes more: 11 for
    // m = 96 over six decades.
    const int sdf = jacobi_polish_df(m, Ad, Vd, ldv, nrmd, 4.0f * 2.220446e-16f * m, 30, &s_flag, &s_off, ptab, pcnt,
                                     flag_list, k, coefs);
    // singular values in descending order (ties broken by column index); the output vectors are
    // the flagged columns, the only ones polished, in descending order of their values
    // (NaN values sort as -inf: ranks and slots stay permutations, every slot is written)
    auto keyd = [](dfr v) { return v.hi == v.hi && v.lo == v.lo ? v : dfr(-INFINITY, 0.f); };
    auto greater = [](dfr x, dfr y) { return x.hi > y.hi || (x.hi == y.hi && x.lo > y.lo); };
    auto same = [](dfr x, dfr y) { return x.hi == y.hi && x.lo == y.lo; };
    for (int c = tid; c < m; c += nt) {
        const dfr s = keyd(nrmd[c]);
        int rank = 0, rank_f = 0;
        for (int c2 = 0; c2 < m; ++c2) {
            const dfr s2 = keyd(nrmd[c2]);
            const bool before = greater(s2, s) || (same(s2, s) && c2 < c);
            rank += before;
            rank_f += before && small_col[c2];
        }
        sigma[rank] = sqrt((double)nrmd[c]) / sc;
        if (small_col[c]) slot_col[rank_f] = c;
    }
    __syncthreads();
    for (int e = tid; e < k * m; e += nt) {
        const int col = min(max(slot_col[e / m], 0), m - 1);
        const dfc v = Vd[(size_t)col * ldv + e % m];
        vs[e] = make_double2((double)v.x, (double)v.y);
    }
    if (tid == 0 && sweeps_out) *sweeps_out = s32 * 1000 + sdf;
}

// ----------------------------------------------------------------- SELL-32 SpMM
// ----------------------------------------------------------------- matrix-free stencil
// Thread (x, y) of a 32 x 8 tile marches over ZC planes, keeping the planes below, at and
// above in registers: each x value comes from memory once for the z direction, the in-plane
// neighbours come from the same or adjacent rows of the tile (L1).  Grid (tiles, z chunks,
// systems).
template <class C> __device__ __forceinline__ C cadd(C a, C b) {
    C r;
    r.x = a.x + b.x;
    r.y = a.y + b.y;
    return r;
}
constexpr int ST_ZC = 8;
template <class R>
__global__ void __launch_bounds__(NT) k_stencil(int nx, int ny, int nz, double2 dd, double2 wxd, double2 wyd,
                                                double2 wzd, const typename CT<R>::t *__restrict__ x0, size_t strideX,
                                                typename CT<R>::t *__restrict__ y0, size_t strideY,
                                                const int *__restrict__ act, const SysState *__restrict__ scale,
                                                typename CT<R>::t *__restrict__ vout0, size_t strideVO) {
    using C = typename CT<R>::t;
    const int sys = act[blockIdx.z];
    const C *x = x0 + (size_t)sys * strideX;
    C *y = y0 + (size_t)sys * strideY;
    // pending normalisation, as in k_spmm: x is w, y = a (A w), vout = a w
    const R al = scale ? (R)scale[sys].alpha : R(1.0);
    const bool brk = scale && scale[sys].broken;
    C *vout = scale ? vout0 + (size_t)sys * strideVO : nullptr;
    const int tilesx = (nx + 31) / 32;
    const int ix = (blockIdx.x % tilesx) * 32 + (threadIdx.x & 31);
    const int iy = (blockIdx.x / tilesx) * 8 + (threadIdx.x >> 5);
    if (ix >= nx || iy >= ny) return;
    const C d = from_d<C>(dd), wx = from_d<C>(wxd), wy = from_d<C>(wyd), wz = from_d<C>(wzd);
    const long plane = (long)nx * ny;
    const int z0 = blockIdx.y * ST_ZC, z1 = min(nz, z0 + ST_ZC);
    long idx = (long)iy * nx + ix + (long)z0 * plane;
    C below = z0 > 0 ? x[idx - plane] : czero<C>();
    C cur = x[idx];
    for (int z = z0; z < z1; ++z, idx += plane) {
        const C above = z + 1 < nz ? x[idx + plane] : czero<C>();
        C sx = czero<C>(), sy = czero<C>();
        if (ix > 0) sx = x[idx - 1];
        if (ix + 1 < nx) sx = cadd(sx, x[idx + 1]);
        if (iy > 0) sy = x[idx - nx];
        if (iy + 1 < ny) sy = cadd(sy, x[idx + nx]);
        C acc = czero<C>();
        cfma(acc, d, cur);
        cfma(acc, wx, sx);
        cfma(acc, wy, sy);
        cfma(acc, wz, cadd(below, above));
        if (vout) {
            C v = cur;
            v.x = v.x * al;
            v.y = v.y * al;
            acc.x = acc.x * al;
            acc.y = acc.y * al;
            if (brk) v = czero<C>();
            vout[idx] = canon(v);
        }
        y[idx] = canon(acc);
        below = cur;
        cur = above;
    }
}

// ----------------------------------------------------------------- structured-grid operator
// The SELL matrix's grid form (coefficient planes, SellMatrix::grid) on the stencil kernel's
// schedule: a CTA is a 32 x 8 tile of (x, y) and a chunk of GR_ZC planes, each thread marches
// up z holding, per system, the x values of the plane below and of its own row in registers;
// in-plane neighbours come from the tile's other rows (L1).  A thread loads its row's
// coefficients once per plane and applies them to SG systems.  Blocks are numbered system group
// fastest, so the groups of one tile run side by side and its coefficients come from DRAM once
// and from L2 for the other groups.  Terms are added in ascending offset order (-P, -Q, -1, 0,
// +1, +Q, +P), the order in which the SELL kernels add a stencil row; a term whose neighbour
// lies outside the grid is left out where the SELL kernels add a stored zero times x.  So both
// forms give the same values for a matrix whose CSR rows are sorted and free of duplicates.
constexpr int GR_ZC = 8;
template <class R, int SG>
__global__ void __launch_bounds__(NT) k_grid_spmm(int nx, int ny, int nz, int ngroups, int ntiles,
                                                  unsigned greal, const typename CT<R>::t *__restrict__ coef,
                                                  const typename CT<R>::t *__restrict__ x0, size_t strideX,
                                                  typename CT<R>::t *__restrict__ y0, size_t strideY,
                                                  const int *__restrict__ act, int nsys,
                                                  const SysState *__restrict__ scale,
                                                  typename CT<R>::t *__restrict__ vout0, size_t strideVO) {
    using C = typename CT<R>::t;
    const int grp = (int)(blockIdx.x % (unsigned)ngroups);
    const int rest = (int)(blockIdx.x / (unsigned)ngroups);
    const int tile = rest % ntiles, zc = rest / ntiles;
    const int tilesx = (nx + 31) / 32;
    const int ix = (tile % tilesx) * 32 + (int)(threadIdx.x & 31);
    const int iy = (tile / tilesx) * 8 + (int)(threadIdx.x >> 5);
    if (ix >= nx || iy >= ny) return;
    const int g0 = grp * SG, ng = min(SG, nsys - g0);
    const long plane = (long)nx * ny, n = plane * nz;
    const bool d3 = nz > 1;
    const C *cf = coef + (d3 ? n : 0);   // the -Q plane (the -P plane precedes it in 3D)
    const int z0 = zc * GR_ZC, z1 = min(nz, z0 + GR_ZC);
    long idx = (long)iy * nx + ix + (long)z0 * plane;
    const C *xs[SG];
    C below[SG], cur[SG];
    R al[SG];      // pending normalisation factors, converted once (a double -> float conversion
    bool bk[SG];   // is an FP64-pipe instruction on GB300)
#pragma unroll
    for (int g = 0; g < SG; ++g) {
        al[g] = R(1.0);
        bk[g] = false;
        if (g < ng) {
            xs[g] = x0 + (size_t)act[g0 + g] * strideX;
            below[g] = z0 > 0 ? xs[g][idx - plane] : czero<C>();
            cur[g] = xs[g][idx];
            if (scale) {
                al[g] = (R)scale[act[g0 + g]].alpha;
                bk[g] = scale[act[g0 + g]].broken != 0;
            }
        }
    }
    const bool xl = ix > 0, xh = ix + 1 < nx, yl = iy > 0, yh = iy + 1 < ny;
    // real planes, in the planes' order (-P first in 3D)
    const int pb = d3 ? 1 : 0;
    const bool rmP = d3 && (greal & 1u), rmQ = (greal >> pb) & 1u, rm1 = (greal >> (pb + 1)) & 1u,
               r00 = (greal >> (pb + 2)) & 1u, rp1 = (greal >> (pb + 3)) & 1u, rpQ = (greal >> (pb + 4)) & 1u,
               rpP = d3 && ((greal >> 6) & 1u);
    for (int z = z0; z < z1; ++z, idx += plane) {
        const bool zl = z > 0, zh = z + 1 < nz;
        const C amP = zl ? coef[idx] : czero<C>();
        const C amQ = cf[idx], am1 = cf[n + idx], a00 = cf[2 * n + idx], ap1 = cf[3 * n + idx], apQ = cf[4 * n + idx];
        const C apP = zh ? cf[5 * n + idx] : czero<C>();
#pragma unroll
        for (int g = 0; g < SG; ++g) {
            if (g < ng) {
                const C *x = xs[g];
                const C above = zh ? x[idx + plane] : czero<C>();
                C acc = czero<C>();
                if (zl) cfma_r(acc, amP, below[g], rmP);
                if (yl) cfma_r(acc, amQ, x[idx - nx], rmQ);
                if (xl) cfma_r(acc, am1, x[idx - 1], rm1);
                cfma_r(acc, a00, cur[g], r00);
                if (xh) cfma_r(acc, ap1, x[idx + 1], rp1);
                if (yh) cfma_r(acc, apQ, x[idx + nx], rpQ);
                if (zh) cfma_r(acc, apP, above, rpP);
                const int sys = act[g0 + g];
                if (scale) {   // pending normalisation, as in k_spmm
                    C v = cur[g];
                    v.x = v.x * al[g];
                    v.y = v.y * al[g];
                    acc.x = acc.x * al[g];
                    acc.y = acc.y * al[g];
                    if (bk[g]) v = czero<C>();
                    vout0[(size_t)sys * strideVO + idx] = canon(v);
                }
                y0[(size_t)sys * strideY + idx] = canon(acc);
                below[g] = cur[g];
                cur[g] = above;
            }
        }
    }
}

// One system: two rows a thread (row r and r + NT of a 2*NT-row chunk), both rows' entries
// loaded before any gather, so the two dependent trips (column index, then x) overlap across
// the rows; rows wider than WMAX take the generic loop.
template <class R>
__global__ void __launch_bounds__(NT, 2) k_spmv2(int n, const int *__restrict__ slice_ptr, const int *__restrict__ cols,
                                              const typename CT<R>::t *__restrict__ vals,
                                              const typename CT<R>::t *__restrict__ x0, size_t strideX,
                                              typename CT<R>::t *__restrict__ y0, size_t strideY,
                                              const int *__restrict__ act, SellPattern pat,
                                              const SysState *__restrict__ scale,
                                              typename CT<R>::t *__restrict__ vout0, size_t strideVO) {
    using C = typename CT<R>::t;
    constexpr int WMAX = SELL_PATTERN;
    const int sys = act[0];
    const C *x = x0 + (size_t)sys * strideX;
    C *y = y0 + (size_t)sys * strideY;
    // pending normalisation, as in k_spmm
    const R al = scale ? (R)scale[sys].alpha : R(1.0);
    const bool brk = scale && scale[sys].broken;
    const long rbase = (long)blockIdx.x * 2 * NT + threadIdx.x;
    C v[2][WMAX];
    int c[2][WMAX], width[2];
    bool ok[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const long row = rbase + (long)h * NT;
        ok[h] = row < n;
        width[h] = 0;
        if (ok[h]) {
            const int slice = (int)(row >> 5), lane = (int)(row & 31);
            const int beg = slice_ptr[slice];
            width[h] = (slice_ptr[slice + 1] - beg) >> 5;
            const bool uni = pat.uniform && pat.uniform[slice];   // columns row + off[e]
#pragma unroll
            for (int e = 0; e < WMAX; ++e) {
                const bool in = e < width[h];
                v[h][e] = in ? vals[beg + e * 32 + lane] : czero<C>();
                c[h][e] = in ? (uni ? (int)row + pat.off[e] : cols[beg + e * 32 + lane]) : (int)row;
            }
        }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        if (!ok[h]) continue;
        const long row = rbase + (long)h * NT;
        C acc = czero<C>();
        if (width[h] <= WMAX) {
            C g[WMAX];
#pragma unroll
            for (int e = 0; e < WMAX; ++e) g[e] = e < width[h] ? x[c[h][e]] : czero<C>();
#pragma unroll
            for (int e = 0; e < WMAX; ++e)
                if (e < width[h]) cfma(acc, v[h][e], g[e]);
        } else {
            const int slice = (int)(row >> 5), lane = (int)(row & 31), beg = slice_ptr[slice];
            for (int e = 0; e < width[h]; ++e) {
                const int idx = beg + e * 32 + lane;
                cfma(acc, vals[idx], x[cols[idx]]);
                acc = canon(acc);
            }
        }
        if (scale) {
            C v = x[row];
            v.x = v.x * al;
            v.y = v.y * al;
            acc.x = acc.x * al;
            acc.y = acc.y * al;
            if (brk) v = czero<C>();
            vout0[(size_t)sys * strideVO + row] = canon(v);
        }
        y[row] = canon(acc);
    }
}

// Grid (system groups, row chunks): the groups of one row chunk run together, so the
// matrix slice is read from HBM once and from L2 for the other groups.
template <class R, int SG>
__global__ void __launch_bounds__(NT) k_spmm(int n, const int *__restrict__ slice_ptr, const int *__restrict__ cols,
                                             const typename CT<R>::t *__restrict__ vals,
                                             const typename CT<R>::t *__restrict__ x0, size_t strideX,
                                             typename CT<R>::t *__restrict__ y0, size_t strideY,
                                             const int *__restrict__ act, int nsys, SellPattern pat,
                                             const SysState *__restrict__ scale, typename CT<R>::t *__restrict__ vout0,
                                             size_t strideVO) {
    using C = typename CT<R>::t;
    constexpr int WMAX = SELL_PATTERN;   // stencil rows (7-point) fit; wider slices take the loop below
    const int g0 = blockIdx.x * SG;
    const int ng = min(SG, nsys - g0);
    // With `scale`, x_s is the unnormalised Krylov vector w_s: y_s = a_s (A w_s) and the row's
    // basis entry v_s = a_s w_s goes to vout_s (a_s = state[s].alpha; zeros after a breakdown),
    // which spares the normalisation kernel its pass over w.  The factors are converted once per
    // CTA: a double -> float conversion per row and system would be an FP64-pipe instruction
    // per element on GB300.
    __shared__ R s_al[SG];
    __shared__ int s_bk[SG];
    if (scale && (int)threadIdx.x < ng) {
        const SysState &stt = scale[act[g0 + threadIdx.x]];
        s_al[threadIdx.x] = (R)stt.alpha;
        s_bk[threadIdx.x] = stt.broken;
    }
    __syncthreads();
    auto fin = [&](int g, int sys, long row, C acc, const C *x) {
        if (scale) {
            const R al = s_al[g];
            C v = x[row];
            v.x = v.x * al;
            v.y = v.y * al;
            acc.x = acc.x * al;
            acc.y = acc.y * al;
            if (s_bk[g]) v = czero<C>();
            vout0[(size_t)sys * strideVO + row] = canon(v);
        }
        y0[(size_t)sys * strideY + row] = canon(acc);
    };
    for (long row = (long)blockIdx.y * NT + threadIdx.x; row < n; row += (long)gridDim.y * NT) {
        const int slice = (int)(row >> 5), lane = (int)(row & 31);
        const int beg = slice_ptr[slice], width = (slice_ptr[slice + 1] - beg) >> 5;
        const bool uni = pat.uniform && pat.uniform[slice];   // columns row + off[e]: no index loads
        if (width <= WMAX) {
            C v[WMAX];
            int c[WMAX];
#pragma unroll
            for (int e = 0; e < WMAX; ++e) {
                if (e < width) {
                    v[e] = vals[beg + e * 32 + lane];
                    c[e] = uni ? (int)row + pat.off[e] : cols[beg + e * 32 + lane];
                } else {
                    v[e] = czero<C>();
                    c[e] = (int)row;
                }
            }
            int g = 0;
            for (; g + 1 < ng; g += 2) {       // two systems: 2*width independent gathers in flight
                const int s0 = act[g0 + g], s1 = act[g0 + g + 1];
                const C *xa = x0 + (size_t)s0 * strideX, *xb = x0 + (size_t)s1 * strideX;
                C a0 = czero<C>(), a1 = czero<C>();
#pragma unroll
                for (int e = 0; e < WMAX; ++e) {
                    if (e < width) {
                        cfma(a0, v[e], xa[c[e]]);
                        cfma(a1, v[e], xb[c[e]]);
                    }
                }
                fin(g, s0, row, a0, xa);
                fin(g + 1, s1, row, a1, xb);
            }
            if (g < ng) {
                const int s0 = act[g0 + g];
                const C *xa = x0 + (size_t)s0 * strideX;
                C a0 = czero<C>();
#pragma unroll
                for (int e = 0; e < WMAX; ++e)
                    if (e < width) cfma(a0, v[e], xa[c[e]]);
                fin(g, s0, row, a0, xa);
            }
        } else {
            for (int g = 0; g < ng; ++g) {
                const int s = act[g0 + g];
                const C *x = x0 + (size_t)s * strideX;
                C acc = czero<C>();
                for (int e = 0; e < width; ++e) {
                    const int idx = beg + e * 32 + lane;
                    cfma(acc, vals[idx], x[cols[idx]]);
                }
                fin(g, s, row, acc, x);
            }
        }
    }
}

// r = b - A x in FP64 with ||r||^2 reduced; last CTA sets true_res and alpha.  The rows of a
// system are split into Gv virtual blocks (row = vb * NT + tid + i * Gv * NT), each with its own
// partial sum; a CTA takes virtual blocks blockIdx.y, blockIdx.y + gridDim.y, ...  So a grid of
// fewer CTAs (to leave room on the SMs for a concurrent stream) adds the same numbers in the
// same order as one CTA per virtual block.
template <int NCX, int WID>
__global__ void __launch_bounds__(NT) k_residual64(int n, const int *__restrict__ slice_ptr, const int *__restrict__ cols,
                                                   const double2 *__restrict__ vals, const double2 *__restrict__ b0,
                                                   size_t strideB, const double2 *__restrict__ x0, size_t strideX,
                                                   double2 *__restrict__ r0, size_t strideR, const int *__restrict__ act,
                                                   double2 *__restrict__ partials, unsigned *tickets, SysState *state,
                                                   ResidPattern rp, int Gv) {
    const int slot = blockIdx.x, s = act[slot], G = gridDim.y, tid = threadIdx.x;
    const double2 *b = b0 + (size_t)s * strideB;
    const double2 *x = x0 + (size_t)s * strideX;
    double2 *r = r0 + (size_t)s * strideR;
    __shared__ double red[1][NW];
    double *part = (double *)partials + (size_t)slot * Gv;
    for (int vb = blockIdx.y; vb < Gv; vb += G) {
        double n2 = 0;
        for (int row = vb * NT + tid; row < n; row += Gv * NT) {
            const double2 acc = resid_row<NCX, WID>(b[row], row, slice_ptr, cols, vals, x, rp);
            r[row] = acc;
            n2 += acc.x * acc.x + acc.y * acc.y;
        }
        double v[1] = {n2};
        block_sum<1>(v, red);
        if (tid == 0) part[vb] = v[0];
        __syncthreads();   // red is reused by the next virtual block
    }
    if (!arrive_last(&tickets[slot], G)) return;
    double tot[1];
    sum_partials<1>(part, Gv, tot, red);
    if (tid == 0) {
        SysState &st = state[s];
        st.nrm2 = tot[0];
        const double nr = sqrt(tot[0]);
        st.true_res = nr;
        st.alpha = nr > 0 ? 1.0 / nr : 0.0;
        if (!isfinite(nr)) st.bad = 1;
        tickets[slot] = 0;
    }
}

template <class R>
__global__ void __launch_bounds__(NT) k_dense_gemv(int n, const typename CT<R>::t *__restrict__ A,
                                                   const typename CT<R>::t *__restrict__ x, typename CT<R>::t *__restrict__ y) {
    using C = typename CT<R>::t;
    __shared__ C xs[NT];
    const int row = blockIdx.x * NT + threadIdx.x;
    C acc = czero<C>();
    for (int j0 = 0; j0 < n; j0 += NT) {
        __syncthreads();
        xs[threadIdx.x] = j0 + threadIdx.x < n ? x[j0 + threadIdx.x] : czero<C>();
        __syncthreads();
        if (row < n) {
            const int lim = min(NT, n - j0);
            for (int j = 0; j < lim; ++j) {
                cfma(acc, A[(size_t)(j0 + j) * n + row], xs[j]);
                acc = canon(acc);
            }
        }
    }
    if (row < n) y[row] = canon(acc);
}

template <class R>
__global__ void __launch_bounds__(NT) k_copy(int n, const typename CT<R>::t *__restrict__ src, size_t strideS,
                                             typename CT<R>::t *__restrict__ dst, size_t strideD, const int *__restrict__ act) {
    const int s = act[blockIdx.y];
    for (long i = (long)blockIdx.x * NT + threadIdx.x; i < n; i += (long)gridDim.x * NT)
        dst[(size_t)s * strideD + i] = src[(size_t)s * strideS + i];
}

template <class R>
__global__ void __launch_bounds__(NT) k_refine_update(int n, double2 *__restrict__ x0, size_t strideX,
                                                      typename CT<R>::t *__restrict__ d0, size_t strideD,
                                                      const int *__restrict__ act, const SysState *__restrict__ state) {
    using C = typename CT<R>::t;
    const int s = act[blockIdx.y];
    const double sc = state[s].true_res;
    double2 *x = x0 + (size_t)s * strideX;
    C *d = d0 + (size_t)s * strideD;
    for (long i = (long)blockIdx.x * NT + threadIdx.x; i < n; i += (long)gridDim.x * NT) {
        C dv = d[i];
        double2 xv = x[i];
        if constexpr (std::is_same<C, float2>::value) {
            // the exact float -> double conversion by integer operations: two FP64 FMAs an
            // element instead of four FP64-pipe instructions
            xv.x = ::fma(sc, f2d_bits(dv.x), xv.x);
            xv.y = ::fma(sc, f2d_bits(dv.y), xv.y);
        } else {
            xv.x += sc * (double)dv.x;
            xv.y += sc * (double)dv.y;
        }
        x[i] = xv;
        d[i] = czero<C>();
    }
}

template <class R>
__global__ void __launch_bounds__(NT) k_demote_unit(int n, const double2 *__restrict__ r0, size_t strideR,
                                                    typename CT<R>::t *__restrict__ h0, size_t strideH,
                                                    typename CT<R>::t *__restrict__ v0, size_t strideV,
                                                    const int *__restrict__ act, const SysState *__restrict__ state) {
    using C = typename CT<R>::t;
    const int s = act[blockIdx.y];
    const double a = state[s].alpha;
    const float af = (float)a;
    for (long i = (long)blockIdx.x * NT + threadIdx.x; i < n; i += (long)gridDim.x * NT) {
        double2 v = r0[(size_t)s * strideR + i];
        C h;
        if constexpr (std::is_same<C, float2>::value) {
            // complex64: the double -> float conversion by integer operations (hi + lo rounds to
            // nearest) and the scaling in FP32; two FP64 multiplies and two conversions per
            // element, all on GB300's FP64 pipe, bounded this kernel
            const dfr xr = d2df_bits(v.x), xi = d2df_bits(v.y);
            h = make_float2((xr.hi + xr.lo) * af, (xi.hi + xi.lo) * af);
        } else {
            h = from_d<C>(make_double2(v.x * a, v.y * a));
        }
        h0[(size_t)s * strideH + i] = h;
        if (v0) v0[(size_t)s * strideV + i] = h;
    }
}

template <class R>
__global__ void __launch_bounds__(NT) k_norm(int n, const typename CT<R>::t *__restrict__ v0, size_t strideV,
                                             const int *__restrict__ act, double2 *__restrict__ partials,
                                             unsigned *tickets, SysState *state, int mode) {
    using C = typename CT<R>::t;
    const int slot = blockIdx.x, s = act[slot], G = gridDim.y, tid = threadIdx.x;
    const C *v = v0 + (size_t)s * strideV;
    __shared__ double red[1][NW];
    double n2 = 0;
    for (long i = (long)blockIdx.y * NT + tid; i < n; i += (long)G * NT) {
        C a = v[i];
        n2 += abs2_d(a);
    }
    double vv[1] = {n2};
    block_sum<1>(vv, red);
    double *part = (double *)partials + (size_t)slot * G;
    if (tid == 0) part[blockIdx.y] = vv[0];
    if (!arrive_last(&tickets[slot], G)) return;
    double tot[1];
    __syncthreads();
    sum_partials<1>(part, G, tot, red);
    if (tid == 0) {
        SysState &st = state[s];
        st.nrm2 = tot[0];
        const double nr = sqrt(tot[0]);
        if (mode == 1) st.bnorm = nr;
        if (mode == 2) { st.rho_abs = nr; st.alpha = nr > 0 ? 1.0 / nr : 0.0; }
        if (!isfinite(nr)) st.bad = 1;
        tickets[slot] = 0;
    }
}

__global__ void k_broadcast_hdef(int m, int kk, const double2 *__restrict__ Hd, double2 *__restrict__ H0, size_t strideH,
                                 const int *__restrict__ act) {
    const int s = act[blockIdx.x], ld = m + 1;
    double2 *H = H0 + (size_t)s * strideH;
    for (int i = threadIdx.x; i < kk * kk; i += blockDim.x) {
        const int c = i / kk, r = i % kk;
        if (r <= c) H[(size_t)c * ld + r] = Hd[(size_t)c * ld + r];
    }
}

inline dim3 grid2(int gx, int gy) { return dim3((unsigned)gx, (unsigned)gy, 1); }

template <class R> int stream_grid(int n, int nsys) {
    int chunks = (n + NT - 1) / NT;
    int target = (num_sms() * 8 + nsys - 1) / (nsys > 0 ? nsys : 1);
    if (target < 1) target = 1;
    return chunks < target ? (chunks > 0 ? chunks : 1) : target;
}

}  // namespace

// ----------------------------------------------------------------- instrumentation
namespace {
std::atomic<long long> g_launches{0};
bool g_prof = false;
struct Pending {
    int kc;
    double bytes;
    cudaEvent_t a, b;
};
std::vector<Pending> g_pending;
std::vector<cudaEvent_t> g_event_pool;
double g_bytes[KC_COUNT], g_ms[KC_COUNT];
long long g_calls[KC_COUNT];
std::mutex g_prof_mu;

cudaEvent_t take_event() {
    if (!g_event_pool.empty()) {
        cudaEvent_t e = g_event_pool.back();
        g_event_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

// RAII bracket around one kernel launch.
struct Launch {
    int kc;
    double bytes;
    cudaStream_t st;
    cudaEvent_t a = nullptr;
    Launch(int kc_, double bytes_, cudaStream_t st_, int nlaunch = 1) : kc(kc_), bytes(bytes_), st(st_) {
        g_launches += nlaunch;
        if (g_prof) {
            std::lock_guard<std::mutex> lk(g_prof_mu);
            a = take_event();
            cudaEventRecord(a, st);
        }
    }
    void add(int k) { g_launches += k; }
    ~Launch() {
        if (a) {
            std::lock_guard<std::mutex> lk(g_prof_mu);
            cudaEvent_t b = take_event();
            cudaEventRecord(b, st);
            g_pending.push_back(Pending{kc, bytes, a, b});
        }
    }
};
}  // namespace

long long launch_count() { return g_launches.load(); }
void profile_enable(bool on) { g_prof = on; }
bool profile_enabled() { return g_prof; }
void profile_flush() {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    for (auto &p : g_pending) {
        float ms = 0;
        cudaEventSynchronize(p.b);
        cudaEventElapsedTime(&ms, p.a, p.b);
        g_ms[p.kc] += ms;
        g_bytes[p.kc] += p.bytes;
        g_calls[p.kc] += 1;
        g_event_pool.push_back(p.a);
        g_event_pool.push_back(p.b);
    }
    g_pending.clear();
}
void profile_read(int kc, double *bytes, double *ms, long long *launches) {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    if (kc < 0 || kc >= KC_COUNT) return;
    if (bytes) *bytes = g_bytes[kc];
    if (ms) *ms = g_ms[kc];
    if (launches) *launches = g_calls[kc];
}
void profile_reset() {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    for (int i = 0; i < KC_COUNT; ++i) g_bytes[i] = g_ms[i] = 0, g_calls[i] = 0;
}

namespace {
// Algorithmic bytes of y_s = A x_s for nsys systems, CSR accounting: every non-zero
// read once (value + 4-byte index), row pointers once, x_s read once, y_s written once.
double spmm_bytes(const SellMatrix &A, size_t vs, int nsys) {
    return (double)A.nnz * (vs + 4.0) + (A.n + 1.0) * 4.0 + (double)nsys * 2.0 * vs * A.n;
}
}  // namespace
size_t scratch_doubles(int qmax, int nsys, int n) {
    // projection partials dominate: qmax coefficients x (re, im) per chunk and system, for the
    // smallest chunk any kernel variant uses (NT elements, one per thread)
    const size_t min_chunks = ((size_t)n + NT - 1) / NT;
    const size_t per_chunk = (size_t)(2 * qmax + 4) * nsys * (min_chunks > 0 ? min_chunks : 1);
    const size_t grid_stride = (size_t)32 * (num_sms() * 8 + nsys);                // norms, residuals, Z update
    return per_chunk + grid_stride;
}

unsigned bulk_timeouts() {
    unsigned v = 0;
    cudaMemcpyFromSymbol(&v, g_bulk_timeouts, sizeof v);
    return v;
}

void enqueue_timeout_read_tc(unsigned *host, cudaStream_t st);   // gdmr_tc.cu
void enqueue_timeout_read(unsigned *host2, cudaStream_t st) {
    enqueue_timeout_read_tc(host2, st);
    cudaMemcpyFromSymbolAsync(host2 + 1, g_bulk_timeouts, sizeof(unsigned), 0, cudaMemcpyDeviceToHost, st);
}

namespace {
constexpr double CYCLES_PER_MS = 2.07e6;   // the GB300's maximum SM clock
std::mutex g_wait_mu;
double g_wait_ms = 2000.0;
std::vector<long long> g_wait_pushed;      // per device: the cycles it holds
}  // namespace

void set_wait_limit_ms(double ms) {
    std::lock_guard<std::mutex> lk(g_wait_mu);
    g_wait_ms = ms < 0 ? 0 : ms;
}
double wait_limit_ms() {
    std::lock_guard<std::mutex> lk(g_wait_mu);
    return g_wait_ms;
}
// 0 on success, -1 if a CUDA call failed
int push_wait_limit() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    std::lock_guard<std::mutex> lk(g_wait_mu);
    const long long cycles = g_wait_ms == 2000.0 ? BK_WAIT_CYCLES : (long long)(g_wait_ms * CYCLES_PER_MS);
    if ((int)g_wait_pushed.size() <= dev) g_wait_pushed.resize(dev + 1, BK_WAIT_CYCLES);
    if (g_wait_pushed[dev] == cycles) return 0;
    if (cudaMemcpyToSymbol(c_wait_cycles, &cycles, sizeof cycles) != cudaSuccess) return -1;
    if (push_wait_limit_tc(cycles) != 0) return -1;
    g_wait_pushed[dev] = cycles;
    return 0;
}

namespace {
// Raises a kernel's dynamic shared-memory limit once per (kernel, device) to the most the
// device allows next to the kernel's static shared memory, so no attribute call happens
// inside a stream capture (the first, eager cycle of an engine makes every call).
std::mutex g_smem_mu;
std::vector<std::pair<const void *, int>> g_smem_done;
template <class K> void allow_smem(K kernel, size_t bytes) {
    if (bytes <= 48 * 1024) return;
    int dev = 0;
    cudaGetDevice(&dev);
    const void *key = (const void *)kernel;
    std::lock_guard<std::mutex> lk(g_smem_mu);
    for (auto &e : g_smem_done)
        if (e.first == key && e.second == dev) return;
    // the opt-in per-block maximum minus the kernel's static shared memory
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa{};
    cudaFuncGetAttributes(&fa, kernel);
    const int dyn = optin - (int)fa.sharedSizeBytes;
    if (dyn > 0 && cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) == cudaSuccess)
        g_smem_done.emplace_back(key, dev);
}
}  // namespace

// ----------------------------------------------------------------- scratch registry
// Engines register their reduction scratch (pointer, doubles); the Gram-Schmidt launchers
// skip any kernel variant whose partial sums would not fit, so no variant can overrun it.
namespace {
std::mutex g_scratch_mu;
std::vector<std::pair<const void *, size_t>> g_scratch;
size_t scratch_capacity(const void *p) {
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    for (auto &e : g_scratch)
        if (e.first == p) return e.second;
    return 0;
}
}  // namespace

void register_scratch(const void *p, size_t doubles) {
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    for (auto &e : g_scratch)
        if (e.first == p) { e.second = doubles; return; }
    g_scratch.emplace_back(p, doubles);
}
void unregister_scratch(const void *p) {
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    for (size_t i = 0; i < g_scratch.size(); ++i)
        if (g_scratch[i].first == p) { g_scratch.erase(g_scratch.begin() + i); return; }
}

// ----------------------------------------------------------------- Gram-Schmidt autotuner
// The projection and update kernels come in (EPT, PU, VEC) variants.  The first launch for a
// (precision, kernel, n) of at least 8 vectors times every variant on the caller's own
// buffers (three runs each, CUDA events on the caller's stream), keeps the fastest, and
// caches the choice for the process, so later launches (and repeat solves) are bitwise
// reproducible.  Re-running a variant is harmless: both kernels are idempotent on their
// inputs (outputs and finishing writes do not alias inputs).
namespace {
struct TuneKey {
    int prec, kernel, n, bucket;
    bool operator==(const TuneKey &o) const {
        return prec == o.prec && kernel == o.kernel && n == o.n && bucket == o.bucket;
    }
};
struct TuneEntry {
    TuneKey key;
    int variant;
    float ms[16];
    int nvar;
};
std::vector<TuneEntry> g_tuned;
std::mutex g_tune_mu;
bool g_tune_enabled = true;
int g_forced[2] = {-1, -1};
int forced_variant(int kernel) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    return g_forced[kernel];
}
thread_local bool t_capturing = false;   // a stream capture is open on this thread: no timing

// One choice per (precision, kernel, n, shape class).  The shape class separates launches
// with and without a shared segment (the deflation vectors W) and single- from multi-system
// launches, because a batch sharing W is limited by re-reading W and favours other tiles.
// Engines run their first two cycles eagerly, so every class they use is settled before a
// cycle is captured into a CUDA graph.
int bucket_of(int nsys, int qa) { return (nsys > 1 ? 1 : 0) + (qa > 0 ? 2 : 0); }

// A class is tuned on its first launch with at least 8 own-basis vectors (mid-cycle Krylov
// steps, where the own part weighs as it does on average), or, for a single system, at least
// 8 shared vectors (the deflation loop, which has no own part).
bool representative(int nsys, int qa, int qb) { return qb >= 8 || (nsys == 1 && qa >= 8); }

template <class F>
int tuned_variant(int prec, int kernel, int n, int nsys, int qa, int nvar, cudaStream_t st, F &&run) {
    const TuneKey key{prec, kernel, n, bucket_of(nsys, qa)};
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        for (auto &e : g_tuned)
            if (e.key == key) return e.variant;
        if (!g_tune_enabled || t_capturing) return 0;
    }
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    TuneEntry ent{key, 0, {0}, nvar};
    float best = 1e30f;
    for (int v = 0; v < nvar; ++v) {
        run(v);   // warm
        float t[3];
        for (int r = 0; r < 3; ++r) {
            cudaEventRecord(a, st);
            run(v);
            cudaEventRecord(b, st);
            cudaEventSynchronize(b);
            cudaEventElapsedTime(&t[r], a, b);
        }
        std::sort(t, t + 3);
        ent.ms[v] = t[1];
        if (t[1] < best) best = t[1];
    }
    // the lowest-numbered variant within 3% of the fastest: variants that close swap places with
    // timing noise from one process to the next, and each choice sums in its own order, so a
    // stable choice keeps a process's results repeatable across runs as well as within one
    for (int v = 0; v < nvar; ++v)
        if (ent.ms[v] >= 0.f && ent.ms[v] <= 1.03f * best) { ent.variant = v; break; }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    for (auto &e : g_tuned)
        if (e.key == key) return e.variant;
    g_tuned.push_back(ent);
    return ent.variant;
}
}  // namespace

void set_capturing(bool on) { t_capturing = on; }

void tune_force(int projection, int update) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_forced[0] = projection;
    g_forced[1] = update;
}

void tune_enable(bool on) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_enabled = on;
}

std::string tune_report() {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    std::string out;
    for (auto &e : g_tuned) {
        char buf[256];
        int len = snprintf(buf, sizeof buf, "%s %s n=%d %s %s: variant %d [",
                           e.key.prec == 4 ? "c64" : e.key.prec == 9 ? "df64" : "c128",
                           e.key.kernel == 0 ? "projection" : "update", e.key.n,
                           (e.key.bucket & 1) ? "batch" : "single", (e.key.bucket & 2) ? "shared" : "own", e.variant);
        out.append(buf, len);
        for (int v = 0; v < e.nvar; ++v) {
            len = snprintf(buf, sizeof buf, "%s%.4f", v ? " " : "", e.ms[v]);
            out.append(buf, len);
        }
        out += " ms]\n";
    }
    return out;
}

// Variant tables: (EPT, PU, VEC), or grp(EPT, SB) for the system-grouped kernels.
//   complex64:  0 (8,2,1)  1 (8,2,2)  2 (16,2,2)  3 (8,4,2)  4 (2,2,1)  5 (1,4,1)  6 grp(4,4)  7 grp(4,2)
//               projection only: 8 split-vector(4); 9 batched shared-W (CUDA cores);
//               10 batched shared-W on the tensor cores (tcgen05, 3xTF32);
//               update only: 8 batched shared-W (CUDA cores), 9 shared part on the tensor cores,
//               10 the whole update in one kernel with the shared part on the tensor cores
//   complex128 and double-float: 0 (4,2,1)  1 (8,2,1)  2 (4,4,1)  3 (1,4,1)  4 (2,2,1)  5 grp(4,2)
//               projection: 6 split-vector(4), 7 batched shared-W (complex128), 8 (4,2,1) prefetching
//               update: 6 batched shared-W (complex128), 7 (4,2,1) prefetching
template <class R, int EPT, int PU, int VEC, bool PF = false>
void mdot_v(int n, const typename CT<R>::t *segA, int qa, const typename CT<R>::t *segB, size_t strideB, int qb,
            const typename CT<R>::t *w, size_t strideW, const int *act, int nsys, double2 *partials, int qmax,
            unsigned *tickets, double2 *coef, size_t strideC, SysState *state, bool skip_broken, cudaStream_t st) {
    const int G = (n + NT * EPT - 1) / (NT * EPT);
    k_mdot<R, EPT, PU, VEC, PF><<<grid2(nsys, G > 0 ? G : 1), NT, 0, st>>>(n, segA, qa, segB, strideB, qb, w, strideW,
                                                                         act, partials, qmax, tickets, coef, strideC,
                                                                         state, skip_broken ? 1 : 0);
}
template <class R, int EPT, int PU, int VEC, bool PF = false>
void update_v(int n, const typename CT<R>::t *segA, int qa, const typename CT<R>::t *segB, size_t strideB, int qb,
              const typename CT<R>::t *w, size_t strideW, typename CT<R>::t *out, size_t strideO, const int *act,
              int nsys, const double2 *coef, size_t strideC, double2 *partials, unsigned *tickets, SysState *state,
              FinishArgs fin, bool skip_broken, cudaStream_t st) {
    const int G = (n + NT * EPT - 1) / (NT * EPT);
    k_update<R, EPT, PU, VEC, PF><<<grid2(nsys, G > 0 ? G : 1), NT, 0, st>>>(n, segA, qa, segB, strideB, qb, w,
                                                                           strideW, out, strideO, act, coef, strideC,
                                                                           partials, tickets, state, fin,
                                                                           skip_broken ? 1 : 0);
}

template <class R, int VPG>
void mdot_s(int n, const typename CT<R>::t *segA, int qa, const typename CT<R>::t *segB, size_t strideB, int qb,
            const typename CT<R>::t *w, size_t strideW, const int *act, int nsys, double2 *partials, int qmax,
            unsigned *tickets, double2 *coef, size_t strideC, SysState *state, bool skip_broken, cudaStream_t st) {
    const int G = (n + NT - 1) / NT, groups = (qa + qb + VPG - 1) / VPG;
    k_mdot_vs<R, VPG><<<dim3((unsigned)nsys, (unsigned)(G > 0 ? G : 1), (unsigned)groups), NT, 0, st>>>(
        n, segA, qa, segB, strideB, qb, w, strideW, act, partials, qmax, tickets, coef, strideC, state,
        skip_broken ? 1 : 0);
}

template <class R, int EPT, int SB>
void mdot_g(int n, const typename CT<R>::t *segA, int qa, const typename CT<R>::t *segB, size_t strideB, int qb,
            const typename CT<R>::t *w, size_t strideW, const int *act, int nsys, double2 *partials, int qmax,
            unsigned *tickets, double2 *coef, size_t strideC, cudaStream_t st) {
    const int G = (n + NT * EPT - 1) / (NT * EPT);
    const size_t smem = sizeof(typename CT<R>::t) * NW * SB * (size_t)qmax;
    allow_smem(k_mdot_grp<R, EPT, SB>, smem);
    k_mdot_grp<R, EPT, SB><<<grid2((nsys + SB - 1) / SB, G > 0 ? G : 1), NT, smem, st>>>(
        n, segA, qa, segB, strideB, qb, w, strideW, act, nsys, partials, qmax, tickets, coef, strideC);
}
template <class R, int EPT, int SB>
void update_g(int n, const typename CT<R>::t *segA, int qa, const typename CT<R>::t *segB, size_t strideB, int qb,
              const typename CT<R>::t *w, size_t strideW, typename CT<R>::t *out, size_t strideO, const int *act,
              int nsys, const double2 *coef, size_t strideC, double2 *partials, unsigned *tickets, SysState *state,
              FinishArgs fin, bool skip_broken, cudaStream_t st) {
    const int G = (n + NT * EPT - 1) / (NT * EPT);
    const size_t smem = sizeof(typename CT<R>::t) * SB * (size_t)(qa + qb > 0 ? qa + qb : 1);
    allow_smem(k_update_grp<R, EPT, SB>, smem);
    k_update_grp<R, EPT, SB><<<grid2((nsys + SB - 1) / SB, G > 0 ? G : 1), NT, smem, st>>>(
        n, segA, qa, segB, strideB, qb, w, strideW, out, strideO, act, nsys, coef, strideC, partials, tickets, state,
        fin, skip_broken ? 1 : 0);
}

// 16-byte packets need every vector base 16-byte aligned: n even (complex64).
inline bool vec2_ok(int n, size_t strideB, size_t strideW) { return (n % 2 == 0) && strideB % 2 == 0 && strideW % 2 == 0; }

bool batched_w_ok(int kk, int nsys) { return kk > 0 && kk <= WP_KMAX && nsys >= 8 && nsys <= WP_SMAX; }

int wproj_grid(int n, int rt) {
    const long nrt = (n + rt - 1) / rt;
    long G = (long)num_sms() * 2;
    if (G > nrt) G = nrt;
    return G < 1 ? 1 : (int)G;
}

// Shared-W projection for a batch: two launches, no profiling bracket of its own (the
// caller's covers it).
template <class R>
void wproj_run(int n, int kk, const typename CT<R>::t *W, const typename CT<R>::t *Y, size_t strideY, const int *act,
               int nsys, double2 *partials, double2 *coef, size_t strideC, cudaStream_t st) {
    const int G = wproj_grid(n, wp_rt<R>());
    const size_t smem = wproj_smem<R>(kk, nsys);
    allow_smem(k_wproj<R>, smem);
    k_wproj<R><<<G, NT, smem, st>>>(n, kk, W, Y, strideY, act, nsys, (double *)partials);
    const int outs = kk * nsys;
    k_wproj_reduce<<<(outs + NW - 1) / NW, NT, 0, st>>>(kk, nsys, G, (const double *)partials, act, coef, strideC);
}

// W rows held in registers: complex64 up to 32 vectors, complex128 up to 16.
template <class R> constexpr int wreg_max() { return sizeof(R) == 4 ? 32 : 16; }

template <class R>
void update_wreg_run(int n, int kk, const typename CT<R>::t *W, const typename CT<R>::t *V, size_t strideV, int qb,
                     const typename CT<R>::t *w, size_t strideW, typename CT<R>::t *out, size_t strideO,
                     const int *act, int nsys, const double2 *coef, size_t strideC, double2 *partials,
                     unsigned *tickets, SysState *state, FinishArgs fin, bool skip_broken, cudaStream_t st) {
    constexpr int SGU = 16;
    const int G = (n + NT - 1) / NT;
    const size_t smem = sizeof(typename CT<R>::t) * (size_t)SGU * (kk + qb);
    const dim3 grid((nsys + SGU - 1) / SGU, G);
    if (kk <= 16) {
        allow_smem(k_update_wreg<R, 16, SGU>, smem);
        k_update_wreg<R, 16, SGU><<<grid, NT, smem, st>>>(n, kk, W, V, strideV, qb, w, strideW, out, strideO, act,
                                                          nsys, coef, strideC, partials, tickets, state, fin,
                                                          skip_broken ? 1 : 0);
    } else {
        constexpr int KW = wreg_max<R>() > 16 ? wreg_max<R>() : 16;
        allow_smem(k_update_wreg<R, KW, SGU>, smem);
        k_update_wreg<R, KW, SGU><<<grid, NT, smem, st>>>(n, kk, W, V, strideV, qb, w, strideW, out, strideO, act,
                                                          nsys, coef, strideC, partials, tickets, state, fin,
                                                          skip_broken ? 1 : 0);
    }
}

// k_update_rows over about two CTAs a SM, each on a contiguous range of chunks; false (nothing
// launched) when the batch or the partials do not fit.
inline bool update_rows_run(int n, int kk, const float2 *W, const float2 *V, size_t strideV, int qb,
                            const float2 *w, size_t strideW, float2 *out, size_t strideO, const int *act, int nsys,
                            const double2 *coef, size_t strideC, double2 *partials, unsigned *tickets,
                            SysState *state, FinishArgs fin, bool skip_broken, cudaStream_t st) {
    if (kk <= 0 || kk > 32 || nsys <= 0 || nsys > 128 || (qb > 0 && !V)) return false;
    const long nch = ((long)n + NT - 1) / NT;
    long target = 2L * num_sms();
    if (target > nch) target = nch;
    const int cpb = (int)((nch + target - 1) / target);
    const int G = (int)((nch + cpb - 1) / cpb);
    if ((size_t)nsys * 3 * G > scratch_capacity(partials)) return false;
    const size_t smem = update_rows_smem(nsys, kk + qb);
    if (smem > 200 * 1024) return false;
    auto go = [&](auto kernel) {
        allow_smem(kernel, smem);
        kernel<<<G, NT, smem, st>>>(n, kk, W, V, strideV, qb, w, strideW, out, strideO, act, nsys, coef, strideC, cpb,
                                    (double *)partials, tickets, state, fin, skip_broken ? 1 : 0);
    };
    if (kk <= 8) go(k_update_rows<8, 8>);
    else if (kk <= 16) go(k_update_rows<16, 8>);
    else if (kk <= 24) go(k_update_rows<24, 8>);
    else go(k_update_rows<32, 4>);
    return true;
}

// The projection variants; returns the number of kernels launched.
template <class R>
int mdot_dispatch(int v, int n, const typename CT<R>::t *segA, int qa, const typename CT<R>::t *segB, size_t strideB,
                  int qb, const typename CT<R>::t *w, size_t strideW, const int *act, int nsys, double2 *partials,
                  int qmax, unsigned *tickets, double2 *coef, size_t strideC, SysState *state, bool skip_broken,
                  cudaStream_t st) {
    const size_t cap = scratch_capacity(partials);
    auto fits = [&](int ept) { return (size_t)nsys * qmax * 2 * (((size_t)n + NT * ept - 1) / (NT * ept)) <= cap; };
    constexpr int VW = sizeof(R) == 4 ? 9 : 7;   // batched shared-W variant
    if constexpr (sizeof(R) == 4) {
        if (v == 10) {   // batched shared-W projection on the tensor cores
            if (qa > 0 && wproj_tc_ok(n, qa, nsys, segA, w, strideW) &&
                (size_t)qa * nsys * 2 * wproj_tc_grid(n) <= cap) {
                launch_wproj_tc(n, qa, segA, w, strideW, act, nsys, (double *)partials, coef, strideC, st);
                if (qb == 0) return 2;
                int vown = 0;
                {
                    std::lock_guard<std::mutex> lk(g_tune_mu);
                    for (auto &e : g_tuned)
                        if (e.key == TuneKey{prec_key<R>(), 0, n, bucket_of(nsys, 0)}) vown = e.variant;
                }
                if (vown >= VW) vown = 0;
                return 2 + mdot_dispatch<R>(vown, n, nullptr, 0, segB, strideB, qb, w, strideW, act, nsys, partials,
                                            qmax, tickets, coef + qa, strideC, state, skip_broken, st);
            }
            v = 0;
        }
    }
    if (v == VW && !std::is_same<R, dfr>::value) {
        if constexpr (!std::is_same<R, dfr>::value) {
          if (qa > 0 && batched_w_ok(qa, nsys) && (size_t)qa * nsys * 2 * wproj_grid(n, wp_rt<R>()) <= cap) {
            wproj_run<R>(n, qa, segA, w, strideW, act, nsys, partials, coef, strideC, st);
            if (qb == 0) return 2;
            // own-basis part: the tuned choice for a batch without a shared segment
            int vown = 0;
            {
                std::lock_guard<std::mutex> lk(g_tune_mu);
                for (auto &e : g_tuned)
                    if (e.key == TuneKey{prec_key<R>(), 0, n, bucket_of(nsys, 0)}) vown = e.variant;
            }
            if (vown >= VW) vown = 0;
            return 2 + mdot_dispatch<R>(vown, n, nullptr, 0, segB, strideB, qb, w, strideW, act, nsys, partials, qmax,
                                        tickets, coef + qa, strideC, state, skip_broken, st);
          }
        }
        v = 0;
    }
    if constexpr (sizeof(R) != 4) {
        if (v == 8) {   // (4, 2, 1) with the next group prefetched
            mdot_v<R, 4, 2, 1, true>(n, segA, qa, segB, strideB, qb, w, strideW, act, nsys, partials, qmax, tickets,
                                     coef, strideC, state, skip_broken, st);
            return 1;
        }
        if constexpr (std::is_same<R, dfr>::value) {
            if (v == 11) {   // bulk-copy pipeline, one CTA per SM
                const long ntiles = ((long)n + BK_TILE - 1) / BK_TILE;
                long G = num_sms() / nsys;
                if (G > ntiles) G = ntiles;
                if (G < 1) G = 1;
                if ((size_t)nsys * qmax * 2 * G <= cap) {
                    allow_smem(k_mdot_bulk, bk_mdot_smem());
                    k_mdot_bulk<<<grid2(nsys, (int)G), BK_THREADS, bk_mdot_smem(), st>>>(
                        n, segA, qa, segB, strideB, qb, w, strideW, act, partials, qmax, tickets, coef, strideC, state,
                        skip_broken ? 1 : 0);
                    return 1;
                }
                v = 0;
            }
        }
        if (v == 12 || v == 13) {   // persistent with the next chunk prefetched: (1, 4) or (2, 2)
            const int ept = v == 12 ? 1 : 2, G = persist_grid(n, ept, nsys);
            if ((size_t)nsys * qmax * 2 * G <= cap) {
                if (v == 12)
                    k_mdot_persist<R, 1, 4, true><<<grid2(nsys, G), NT, 0, st>>>(n, segA, qa, segB, strideB, qb, w,
                                                                                 strideW, act, partials, qmax, tickets,
                                                                                 coef, strideC, state,
                                                                                 skip_broken ? 1 : 0);
                else
                    k_mdot_persist<R, 2, 2, true><<<grid2(nsys, G), NT, 0, st>>>(n, segA, qa, segB, strideB, qb, w,
                                                                                 strideW, act, partials, qmax, tickets,
                                                                                 coef, strideC, state,
                                                                                 skip_broken ? 1 : 0);
                return 1;
            }
            v = 0;
        }
        if (v == 9 || v == 10) {   // persistent: (4 elements, 2 vectors) or (2, 4)
            const int ept = v == 9 ? 4 : 2, G = persist_grid(n, ept, nsys);
            if ((size_t)nsys * qmax * 2 * G <= cap) {
                if (v == 9)
                    k_mdot_persist<R, 4, 2><<<grid2(nsys, G), NT, 0, st>>>(n, segA, qa, segB, strideB, qb, w, strideW,
                                                                           act, partials, qmax, tickets, coef, strideC,
                                                                           state, skip_broken ? 1 : 0);
                else
                    k_mdot_persist<R, 2, 4><<<grid2(nsys, G), NT, 0, st>>>(n, segA, qa, segB, strideB, qb, w, strideW,
                                                                           act, partials, qmax, tickets, coef, strideC,
                                                                           state, skip_broken ? 1 : 0);
                return 1;
            }
            v = 0;
        }
    }
    if constexpr (sizeof(R) == 4) {
        static const int ept_of[9] = {8, 8, 16, 8, 2, 1, 4, 4, 1};
        if (v < 0 || v > 8 || !fits(ept_of[v])) v = 0;
    } else {
        static const int ept_of[7] = {4, 8, 4, 1, 2, 4, 1};
        if (v < 0 || v > 6 || !fits(ept_of[v])) v = 0;
    }
    if constexpr (sizeof(R) == 4) {
        const bool v2 = vec2_ok(n, strideB, strideW);
        if (v == 8) { mdot_s<R, 4>(n, segA, qa, segB, strideB, qb, w, strideW, act, nsys, partials, qmax, tickets, coef, strideC, state, skip_broken, st); return 1; }
        if (v == 1 && v2) mdot_v<R, 8, 2, 2>(n, segA, qa, segB, strideB, qb, w, strideW, act, nsys, partials, qmax, tickets, coef, strideC, state, skip_broken, st);
        else if (v == 2 && v2) mdot_v<R, 16, 2, 2>(n, segA, qa, segB, strideB, qb, w, strideW, act, nsys, partials, qmax, tickets, coef, strideC, state, skip_broken, st);
        else if (v == 3 && v2) mdot_v<R, 8, 4, 2>(n, segA, qa, segB, strideB, qb, w, strideW, act, nsys, partials, qmax, tickets, coef, strideC, state, skip_broken, st);
        else if (v == 4) mdot_v<R, 2, 2, 1>(n, segA, qa, segB, strideB, qb, w, strideW, act, nsys, partials, qmax, tickets, coef, strideC, state, skip_broken, st);
        else if (v == 5) mdot_v<R, 1, 4, 1>(n, segA, qa, segB, strideB, qb, w, strideW, act, nsys, partials, qmax, tickets, coef, strideC, state, skip_broken, st);
        else if (v == 6) mdot_g<R, 4, 4>(n, segA, qa, segB, strideB, qb, w, strideW, act, nsys, partials, qmax, tickets, coef, strideC, st);
        else if (v == 7) mdot_g<R, 4, 2>(n, segA, qa, segB, strideB, qb, w, strideW, act, nsys, partials, qmax, tickets, coef, strideC, st);
        else mdot_v<R, 8, 2, 1>(n, segA, qa, segB, strideB, qb, w, strideW, act, nsys, partials, qmax, tickets, coef, strideC, state, skip_broken, st);
    } else {
        if (v == 6) { mdot_s<R, 4>(n, segA, qa, segB, strideB, qb, w, strideW, act, nsys, partials, qmax, tickets, coef, strideC, state, skip_broken, st); return 1; }
        if (v == 1) mdot_v<R, 8, 2, 1>(n, segA, qa, segB, strideB, qb, w, strideW, act, nsys, partials, qmax, tickets, coef, strideC, state, skip_broken, st);
        else if (v == 2) mdot_v<R, 4, 4, 1>(n, segA, qa, segB, strideB, qb, w, strideW, act, nsys, partials, qmax, tickets, coef, strideC, state, skip_broken, st);
        else if (v == 3) mdot_v<R, 1, 4, 1>(n, segA, qa, segB, strideB, qb, w, strideW, act, nsys, partials, qmax, tickets, coef, strideC, state, skip_broken, st);
        else if (v == 4) mdot_v<R, 2, 2, 1>(n, segA, qa, segB, strideB, qb, w, strideW, act, nsys, partials, qmax, tickets, coef, strideC, state, skip_broken, st);
        else if (v == 5) mdot_g<R, 4, 2>(n, segA, qa, segB, strideB, qb, w, strideW, act, nsys, partials, qmax, tickets, coef, strideC, st);
        else mdot_v<R, 4, 2, 1>(n, segA, qa, segB, strideB, qb, w, strideW, act, nsys, partials, qmax, tickets, coef, strideC, state, skip_broken, st);
    }
    return 1;
}

template <class R>
void launch_mdot(int n, const typename CT<R>::t *segA, int qa, const typename CT<R>::t *segB, size_t strideB, int qb,
                 const typename CT<R>::t *w, size_t strideW, const int *act, int nsys, double2 *partials, int qmax,
                 unsigned *tickets, double2 *coef, size_t strideC, SysState *state, bool skip_broken, cudaStream_t st) {
    if (nsys <= 0 || qa + qb <= 0) return;
    Launch L_(KC_MDOT, (double)sizeof(typename CT<R>::t) * n * ((double)qa + (double)nsys * (qb + 1)), st, 0);
    int launched = 0;
    auto run = [&](int v) {
        launched = mdot_dispatch<R>(v, n, segA, qa, segB, strideB, qb, w, strideW, act, nsys, partials, qmax, tickets,
                                    coef, strideC, state, skip_broken, st);
    };
    int v = 0;
    if (forced_variant(0) >= 0) v = forced_variant(0);
    else if (representative(nsys, qa, qb) && !profile_enabled()) v = tuned_variant(prec_key<R>(), 0, n, nsys, qa, sizeof(R) == 4 ? 11 : 14, st, run);
    else {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        for (auto &e : g_tuned)
            if (e.key == TuneKey{prec_key<R>(), 0, n, bucket_of(nsys, qa)}) v = e.variant;
    }
    run(v);
    L_.add(launched);
}

// The update variants; returns the number of kernels launched.
template <class R>
int update_dispatch(int v, int n, const typename CT<R>::t *segA, int qa, const typename CT<R>::t *segB,
                    size_t strideB, int qb, const typename CT<R>::t *w, size_t strideW, typename CT<R>::t *out,
                    size_t strideO, const int *act, int nsys, const double2 *coef, size_t strideC, double2 *partials,
                    unsigned *tickets, SysState *state, FinishArgs fin, bool skip_broken, cudaStream_t st) {
    const size_t cap = scratch_capacity(partials);
    auto fits = [&](int ept) { return (size_t)nsys * 3 * (((size_t)n + NT * ept - 1) / (NT * ept)) <= cap; };
    constexpr int VW = sizeof(R) == 4 ? 8 : 6;   // batched shared-W variant
    if constexpr (sizeof(R) == 4) {
        // 11: every system of the batch per CTA, W rows in registers (k_update_rows)
        if (v == 11) {
            if (qa > 0 && update_rows_run(n, qa, segA, segB, strideB, qb, w, strideW, out, strideO, act, nsys, coef,
                                          strideC, partials, tickets, state, fin, skip_broken, st))
                return 1;
            v = 0;
        }
        // 10: the whole update in one kernel, the shared part W c on the tensor cores and
        // subtracted from TMEM by the epilogue that streams w_s and V_s
        if (v == 10) {
            if (qa > 0 && wupdate_tc_ok(n, qa, qb, nsys) && (qb == 0 || segB) &&
                (size_t)nsys * 3 * wupdate_tc_grid(n) <= cap) {
                launch_wupdate_tc(n, qa, segA, segB, strideB, qb, w, strideW, out, strideO, act, nsys, coef, strideC,
                                  (double *)partials, tickets, state, fin, skip_broken, st);
                return 1;
            }
            v = 0;
        }
        // 9: the shared part W c on the tensor cores into the free slot segB_s[qb] (the next
        // Krylov vector's), then the per-system update with that slot as one more basis vector
        // of coefficient 1 (written by the apply kernel at coef_s[qa + qb])
        if (v == 9) {
            if (qa > 0 && qb > 0 && segB && wapply_tc_ok(n, qa, nsys) && fits(8)) {
                launch_wapply_tc(n, qa, segA, const_cast<double2 *>(coef), strideC, act, nsys,
                                 const_cast<typename CT<R>::t *>(segB) + (size_t)qb * n, strideB, qa + qb, st);
                int vown = 0;
                {
                    std::lock_guard<std::mutex> lk(g_tune_mu);
                    for (auto &e : g_tuned)
                        if (e.key == TuneKey{prec_key<R>(), 1, n, bucket_of(nsys, 0)}) vown = e.variant;
                }
                if (vown >= VW) vown = 0;
                return 1 + update_dispatch<R>(vown, n, nullptr, 0, segB, strideB, qb + 1, w, strideW, out, strideO,
                                              act, nsys, coef + qa, strideC, partials, tickets, state, fin,
                                              skip_broken, st);
            }
            v = 0;
        }
    }
    if (v == VW && std::is_same<R, dfr>::value) v = 0;   // no double-float form of the batched pair
    if constexpr (!std::is_same<R, dfr>::value) {
        if (v == VW) {
            if (qa > 0 && batched_w_ok(qa, nsys) && qa <= wreg_max<R>() && fits(1) && (n + NT - 1) / NT <= 65535) {
                update_wreg_run<R>(n, qa, segA, segB, strideB, qb, w, strideW, out, strideO, act, nsys, coef, strideC,
                                   partials, tickets, state, fin, skip_broken, st);
                return 1;
            }
            v = 0;
        }
    }
    if constexpr (sizeof(R) != 4) {
        if (v == 7) {   // (4, 2, 1) with the next group prefetched
            update_v<R, 4, 2, 1, true>(n, segA, qa, segB, strideB, qb, w, strideW, out, strideO, act, nsys, coef,
                                       strideC, partials, tickets, state, fin, skip_broken, st);
            return 1;
        }
        if constexpr (std::is_same<R, dfr>::value) {
            if (v == 10) {   // bulk-copy pipeline, one CTA per SM
                const long ntiles = ((long)n + BK_TILE - 1) / BK_TILE;
                long G = num_sms() / nsys;
                if (G > ntiles) G = ntiles;
                if (G < 1) G = 1;
                if ((size_t)nsys * 3 * G <= cap) {
                    allow_smem(k_update_bulk, bk_update_smem());
                    k_update_bulk<<<grid2(nsys, (int)G), BK_THREADS, bk_update_smem(), st>>>(
                        n, segA, qa, segB, strideB, qb, w, strideW, out, strideO, act, coef, strideC, partials, tickets,
                        state, fin, skip_broken ? 1 : 0);
                    return 1;
                }
                v = 0;
            }
        }
        if (v == 11 || v == 12) {   // persistent with the next group prefetched: (2, 2) or (1, 4)
            const int ept = v == 11 ? 2 : 1, G = persist_grid(n, ept, nsys);
            if ((size_t)nsys * 3 * G <= cap) {
                if (v == 11)
                    k_update_persist<R, 2, 2, true><<<grid2(nsys, G), NT, 0, st>>>(n, segA, qa, segB, strideB, qb, w,
                                                                                   strideW, out, strideO, act, coef,
                                                                                   strideC, partials, tickets, state, fin,
                                                                                   skip_broken ? 1 : 0);
                else
                    k_update_persist<R, 1, 4, true><<<grid2(nsys, G), NT, 0, st>>>(n, segA, qa, segB, strideB, qb, w,
                                                                                   strideW, out, strideO, act, coef,
                                                                                   strideC, partials, tickets, state, fin,
                                                                                   skip_broken ? 1 : 0);
                return 1;
            }
            v = 0;
        }
        if (v == 8 || v == 9) {   // persistent: (4 elements, 2 vectors) or (2, 4)
            const int ept = v == 8 ? 4 : 2, G = persist_grid(n, ept, nsys);
            if ((size_t)nsys * 3 * G <= cap) {
                if (v == 8)
                    k_update_persist<R, 4, 2><<<grid2(nsys, G), NT, 0, st>>>(n, segA, qa, segB, strideB, qb, w,
                                                                             strideW, out, strideO, act, coef, strideC,
                                                                             partials, tickets, state, fin,
                                                                             skip_broken ? 1 : 0);
                else
                    k_update_persist<R, 2, 4><<<grid2(nsys, G), NT, 0, st>>>(n, segA, qa, segB, strideB, qb, w,
                                                                             strideW, out, strideO, act, coef, strideC,
                                                                             partials, tickets, state, fin,
                                                                             skip_broken ? 1 : 0);
                return 1;
            }
            v = 0;
        }
    }
    if constexpr (sizeof(R) == 4) {
        static const int ept_of[8] = {8, 8, 16, 8, 2, 1, 4, 4};
        if (v < 0 || v > 7 || !fits(ept_of[v])) v = 0;
    } else {
        static const int ept_of[6] = {4, 8, 4, 1, 2, 4};
        if (v < 0 || v > 5 || !fits(ept_of[v])) v = 0;
    }
    if constexpr (sizeof(R) == 4) {
        const bool v2 = vec2_ok(n, strideB, strideW) && strideO % 2 == 0;
        if (v == 1 && v2) update_v<R, 8, 2, 2>(n, segA, qa, segB, strideB, qb, w, strideW, out, strideO, act, nsys, coef, strideC, partials, tickets, state, fin, skip_broken, st);
        else if (v == 2 && v2) update_v<R, 16, 2, 2>(n, segA, qa, segB, strideB, qb, w, strideW, out, strideO, act, nsys, coef, strideC, partials, tickets, state, fin, skip_broken, st);
        else if (v == 3 && v2) update_v<R, 8, 4, 2>(n, segA, qa, segB, strideB, qb, w, strideW, out, strideO, act, nsys, coef, strideC, partials, tickets, state, fin, skip_broken, st);
        else if (v == 4) update_v<R, 2, 2, 1>(n, segA, qa, segB, strideB, qb, w, strideW, out, strideO, act, nsys, coef, strideC, partials, tickets, state, fin, skip_broken, st);
        else if (v == 5) update_v<R, 1, 4, 1>(n, segA, qa, segB, strideB, qb, w, strideW, out, strideO, act, nsys, coef, strideC, partials, tickets, state, fin, skip_broken, st);
        else if (v == 6) update_g<R, 4, 4>(n, segA, qa, segB, strideB, qb, w, strideW, out, strideO, act, nsys, coef, strideC, partials, tickets, state, fin, skip_broken, st);
        else if (v == 7) update_g<R, 4, 2>(n, segA, qa, segB, strideB, qb, w, strideW, out, strideO, act, nsys, coef, strideC, partials, tickets, state, fin, skip_broken, st);
        else update_v<R, 8, 2, 1>(n, segA, qa, segB, strideB, qb, w, strideW, out, strideO, act, nsys, coef, strideC, partials, tickets, state, fin, skip_broken, st);
    } else {
        if (v == 1) update_v<R, 8, 2, 1>(n, segA, qa, segB, strideB, qb, w, strideW, out, strideO, act, nsys, coef, strideC, partials, tickets, state, fin, skip_broken, st);
        else if (v == 2) update_v<R, 4, 4, 1>(n, segA, qa, segB, strideB, qb, w, strideW, out, strideO, act, nsys, coef, strideC, partials, tickets, state, fin, skip_broken, st);
        else if (v == 3) update_v<R, 1, 4, 1>(n, segA, qa, segB, strideB, qb, w, strideW, out, strideO, act, nsys, coef, strideC, partials, tickets, state, fin, skip_broken, st);
        else if (v == 4) update_v<R, 2, 2, 1>(n, segA, qa, segB, strideB, qb, w, strideW, out, strideO, act, nsys, coef, strideC, partials, tickets, state, fin, skip_broken, st);
        else if (v == 5) update_g<R, 4, 2>(n, segA, qa, segB, strideB, qb, w, strideW, out, strideO, act, nsys, coef, strideC, partials, tickets, state, fin, skip_broken, st);
        else update_v<R, 4, 2, 1>(n, segA, qa, segB, strideB, qb, w, strideW, out, strideO, act, nsys, coef, strideC, partials, tickets, state, fin, skip_broken, st);
    }
    return 1;
}

template <class R>
void launch_update(int n, const typename CT<R>::t *segA, int qa, const typename CT<R>::t *segB, size_t strideB, int qb,
                   const typename CT<R>::t *w, size_t strideW, typename CT<R>::t *out, size_t strideO, const int *act,
                   int nsys, const double2 *coef, size_t strideC, double2 *partials, unsigned *tickets,
                   SysState *state, FinishArgs fin, bool skip_broken, cudaStream_t st) {
    if (nsys <= 0) return;
    Launch L_(KC_UPDATE, (double)sizeof(typename CT<R>::t) * n * ((double)qa + (double)nsys * (qb + 2)), st, 0);
    int launched = 0;
    auto run = [&](int v) {
        launched = update_dispatch<R>(v, n, segA, qa, segB, strideB, qb, w, strideW, out, strideO, act, nsys, coef,
                                      strideC, partials, tickets, state, fin, skip_broken, st);
    };
    int v = 0;
    if (forced_variant(1) >= 0) v = forced_variant(1);
    else if (representative(nsys, qa, qb) && !profile_enabled())
        v = tuned_variant(prec_key<R>(), 1, n, nsys, qa, sizeof(R) == 4 ? 12 : 13, st, run);
    else {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        for (auto &e : g_tuned)
            if (e.key == TuneKey{prec_key<R>(), 1, n, bucket_of(nsys, qa)}) v = e.variant;
    }
    run(v);
    L_.add(launched);
}

template <class R>
void launch_scale(int n, const typename CT<R>::t *in, size_t strideI, typename CT<R>::t *out1, size_t strideO1,
                  typename CT<R>::t *out2, size_t strideO2, const int *act, int nsys, const SysState *state,
                  bool honour_broken, cudaStream_t st) {
    if (nsys <= 0) return;
    Launch L_(KC_OTHER, (double)sizeof(typename CT<R>::t) * n * nsys * (out2 ? 3.0 : 2.0), st, 1);
    k_scale<R><<<grid2(stream_grid<R>(n, nsys), nsys), NT, 0, st>>>(n, in, strideI, out1, strideO1, out2, strideO2,
                                                                      act, state, honour_broken ? 1 : 0);
}

template <class R>
void launch_combine(int n, int kk, int m, const typename CT<R>::t *W, const typename CT<R>::t *Z,
                    const typename CT<R>::t *V, size_t strideV, typename CT<R>::t *r, size_t strideR,
                    typename CT<R>::t *x, size_t strideX, const double2 *t, const double2 *y, size_t strideC,
                    const int *act, int nsys, double2 *partials, unsigned *tickets, SysState *state, cudaStream_t st) {
    if (nsys <= 0) return;
    Launch L_(KC_COMBINE, (double)sizeof(typename CT<R>::t) * n * (2.0 * kk + (double)nsys * (m + 1 - kk + 4)), st, 1);
    if (kk > 0 && nsys >= 4 && combine_group() > 0) {
        // the grouped form: the shared W and Z loaded once for four systems
        constexpr int EPT = sizeof(R) == 4 ? 2 : 1;
        const int G = (n + NT * EPT - 1) / (NT * EPT);
        k_combine_grp<R, 4, EPT><<<dim3((unsigned)((nsys + 3) / 4), (unsigned)G), NT, 0, st>>>(
            n, kk, m, W, Z, V, strideV, r, strideR, x, strideX, t, y, strideC, act, nsys, partials, tickets, state);
        return;
    }
    k_combine<R><<<grid2(nsys, nchunks<R>(n)), NT, 0, st>>>(n, kk, m, W, Z, V, strideV, r, strideR, x, strideX, t, y, strideC, act,
                                                 partials, tickets, state);
}

template <class R>
void launch_zupdate(int n, int kk, int m, int k, const typename CT<R>::t *Z, const typename CT<R>::t *V,
                    size_t strideV, const int *lead, const double2 *vs, typename CT<R>::t *Znew, double2 *partials,
                    unsigned *ticket, double *znorm2, cudaStream_t st) {
    using C = typename CT<R>::t;
    int chunks = (n + NT - 1) / NT;
    int G = num_sms() * 4;
    if (G > chunks) G = chunks;
    // complex64: every output in one pass over [Z V] (blocks of 24 or 32 outputs in registers),
    // so the basis is read once; the double-float forms keep 8 outputs a pass (registers)
    if constexpr (sizeof(R) == 4) {
        if (k <= 32) {
            Launch L_(KC_ZUPDATE, (double)sizeof(C) * n * ((double)m + k), st, 1);
            auto run = [&](auto kb) {
                constexpr int KB = decltype(kb)::value;
                const size_t smem = (size_t)m * KB * sizeof(typename ZW<C>::t);
                k_zupdate<R, KB><<<G, NT, smem, st>>>(n, kk, m, k, 0, Z, V, strideV, lead, vs, Znew, partials, ticket,
                                                      znorm2);
            };
            if (k <= 16) run(std::integral_constant<int, 16>{});
            else if (k <= 24) run(std::integral_constant<int, 24>{});
            else run(std::integral_constant<int, 32>{});
            return;
        }
    }
    if constexpr (sizeof(R) != 4) {
        // double-float accumulators (four FP32 words an output): 12 outputs a pass, so k = 24
        // reads [Z V] twice instead of three times
        if (k <= 24) {
            constexpr int KB = 12;
            Launch L_(KC_ZUPDATE, (double)sizeof(C) * n * ((double)m + k), st, (k + KB - 1) / KB);
            for (int t0 = 0; t0 < k; t0 += KB) {
                const size_t smem = (size_t)m * KB * sizeof(typename ZW<C>::t);
                k_zupdate<R, KB><<<G, NT, smem, st>>>(n, kk, m, k, t0, Z, V, strideV, lead, vs, Znew, partials,
                                                      ticket, znorm2);
            }
            return;
        }
    }
    constexpr int KB = sizeof(R) == 4 ? 16 : 8;
    Launch L_(KC_ZUPDATE, (double)sizeof(C) * n * ((double)m + k), st, (k + KB - 1) / KB);
    for (int t0 = 0; t0 < k; t0 += KB) {
        size_t smem = (size_t)m * KB * sizeof(typename ZW<C>::t);
        k_zupdate<R, KB><<<G, NT, smem, st>>>(n, kk, m, k, t0, Z, V, strideV, lead, vs, Znew, partials, ticket,
                                              znorm2);
    }
}

template <class R>
void launch_znormalise(int n, int k, const typename CT<R>::t *Znew, const double *znorm2, typename CT<R>::t *Z,
                       cudaStream_t st) {
    if (k <= 0) return;
    Launch L_(KC_ZUPDATE, (double)sizeof(typename CT<R>::t) * n * 2.0 * k, st, 1);
    k_znormalise<R><<<grid2(stream_grid<R>(n, k), k), NT, 0, st>>>(n, Znew, znorm2, Z);
}

void launch_ls(int m, const double2 *H, size_t strideH, const double2 *g, double2 *y, double2 *t, size_t strideC,
               const int *act, int nsys, cudaStream_t st) {
    if (nsys <= 0) return;
    Launch L_(KC_LS, (double)sizeof(double2) * nsys * (m + 1.0) * m, st, 1);
    size_t smem = sizeof(double2) * ((size_t)m * (m + 3) / 2 + (m + 1) + m + m) + sizeof(double) * (m + 1);
    allow_smem(k_ls, smem);
    k_ls<<<nsys, 128, smem, st>>>(m, H, strideH, g, y, t, strideC, act);
}

size_t svd_smem_bytes(int m) { return svd_work_bytes(m); }

void launch_svd_smallest(int m, int k, const double2 *H, size_t strideH, const int *lead, double2 *vs, double *sigma,
                         double2 *work, int *sweeps,
                         cudaStream_t st) {
    Launch L_(KC_SVD, (double)sizeof(double2) * (m + 1.0) * m, st, 1);
    size_t smem = svd_smem_bytes(m);
    int use_smem = smem <= 200 * 1024;
    if (use_smem) allow_smem(k_svd, smem);
    const int pairs = (m + 1) / 2;
    int threads = 32 * (pairs < 32 ? (pairs > 4 ? pairs : 4) : 32);
    k_svd<<<1, threads, use_smem ? smem : 0, st>>>(m, k, H, strideH, lead, vs, sigma, work, use_smem, sweeps);
}

// Algorithmic bytes of the fused Krylov loop: per step the operator product, the projection
// against kk + j vectors (and y), the update (the same vectors, y, w) and the scaling.
double krylov_small_bytes(const SellMatrix &A, size_t vs, int kk, int m);

int krylov_multi_resident() {
    static std::mutex mu;
    static std::vector<int> per_dev;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    if ((int)per_dev.size() <= dev) per_dev.resize(dev + 1, -1);
    if (per_dev[dev] < 0) {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_krylov_multi<float>, KM_THREADS, 0) != cudaSuccess)
            per_sm = 0;
        int per_sm2 = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm2, k_krylov_multi<double>, KM_THREADS, 0) !=
            cudaSuccess)
            per_sm2 = 0;
        int per_sm3 = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm3, k_krylov_multi<dfr>, KM_THREADS, 0) != cudaSuccess)
            per_sm3 = 0;
        per_dev[dev] = std::min(per_sm, std::min(per_sm2, per_sm3)) * num_sms();
    }
    return per_dev[dev];
}

template <class R>
int launch_krylov_multi(const KrylovJob<R> *jobs, const int *cta_job, int ctas, int *abort, double algorithmic_bytes,
                        cudaStream_t st) {
    if (ctas < 1) return 0;
    Launch L_(KC_UPDATE, algorithmic_bytes, st, 1);
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)ctas);
    cfg.blockDim = dim3(KM_THREADS);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_krylov_multi<R>, jobs, cta_job, abort) == cudaSuccess ? 1 : -1;
}

double krylov_loop_bytes(const SellMatrix &A, size_t vs, int kk, int m) { return krylov_small_bytes(A, vs, kk, m); }

double krylov_small_bytes(const SellMatrix &A, size_t vs, int kk, int m) {
    double b = 0;
    for (int j = 1; j <= m - kk; ++j)
        b += spmm_bytes(A, vs, 1) + (double)vs * A.n * ((kk + j + 1.0) + (kk + j + 2.0) + 2.0);
    return b;
}

// The fused Krylov loop for one system (k_krylov_small); false when it does not apply: n above
// 32 x (CTAs resident at once), the scratch too small, or the launch refused.
template <class R>
bool launch_krylov_small(int n, int kk, int m, const SellMatrix &A, const typename CT<R>::t *W,
                         typename CT<R>::t *V, size_t strideV, const int *act, SysState *state, double2 *H,
                         size_t strideH, double2 *coef, size_t strideC, double *partials, int qmax, unsigned *bar,
                         double tol, bool compat_eye, cudaStream_t st) {
    if constexpr (sizeof(R) == 4) {
        return false;
    } else {
        const int G = A.nslices;
        if (G < 1 || m - kk < 1 || qmax > QMAX) return false;
        static int resident = -1;
        if (resident < 0) {
            int per_sm = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_krylov_small<R>, KS_THREADS, 0) != cudaSuccess)
                per_sm = 0;
            resident = per_sm * num_sms();
        }
        if (G > resident) return false;
        const size_t need = (size_t)G * qmax * 2 + (size_t)G * 3;
        if (need > scratch_capacity(partials)) return false;
        KrylovSmallArgs<R> a{};
        a.n = n; a.kk = kk; a.m = m; a.compat_eye = compat_eye ? 1 : 0; a.qmax = qmax; a.tol = tol;
        a.slice_ptr = A.slice_ptr; a.cols = A.cols; a.vals = (const typename CT<R>::t *)A.vals;
        a.W = W; a.V0 = V; a.strideV = strideV; a.act = act; a.state = state;
        a.H0 = H; a.strideH = strideH; a.coef0 = coef; a.strideC = strideC;
        a.part = partials; a.npart = partials + (size_t)G * qmax * 2; a.bar = bar;
        Launch L_(KC_UPDATE, krylov_small_bytes(A, sizeof(typename CT<R>::t), kk, m), st, 1);
        if (cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), st) != cudaSuccess) return false;
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3((unsigned)G);
        cfg.blockDim = dim3(KS_THREADS);
        cfg.dynamicSmemBytes = 0;
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        return cudaLaunchKernelEx(&cfg, k_krylov_small<R>, a) == cudaSuccess;
    }
}

static std::atomic<int> g_combine_group{1};
void set_combine_group(int on) { g_combine_group.store(on ? 1 : 0); }
int combine_group() { return g_combine_group.load(); }
static std::atomic<int> g_overlap_residual{0};
int set_overlap_residual(int ctas_per_sm) {
    const int prev = g_overlap_residual.load();
    if (ctas_per_sm >= 0) g_overlap_residual.store(std::min(ctas_per_sm, 8));
    return prev;
}
int overlap_residual() { return g_overlap_residual.load(); }
static std::atomic<int> g_grid_operator{1};
static std::atomic<int> g_grid_batch{0};
void set_grid_operator(int enable) { g_grid_operator.store(enable ? 1 : 0); }
int grid_operator() { return g_grid_operator.load(); }
void set_grid_batch(int sg) { g_grid_batch.store(sg == 1 || sg == 2 || sg == 4 ? sg : 0); }
int grid_batch() { return g_grid_batch.load(); }

SellPattern sell_pattern(const SellMatrix &A) {
    SellPattern p{};
    p.uniform = A.npat > 0 ? A.uniform : nullptr;
    for (int e = 0; e < SELL_PATTERN; ++e) p.off[e] = A.pat[e];
    return p;
}

template <class R>
void launch_spmm(const SellMatrix &A, const typename CT<R>::t *x, size_t strideX, typename CT<R>::t *y, size_t strideY,
                 const int *act, int nsys, cudaStream_t st, const SysState *scale, typename CT<R>::t *vout,
                 size_t strideVO) {
    if (nsys <= 0) return;
    // with the normalisation folded in, the kernel also writes v_s: one more vector a system
    Launch L_(KC_SPMM, spmm_bytes(A, sizeof(typename CT<R>::t), nsys) +
                           (scale ? (double)sizeof(typename CT<R>::t) * A.n * nsys : 0.0), st, 1);
    const int sg = nsys == 1 ? 1 : grid_batch();
    if (A.grid && grid_operator() && sg > 0) {
        const int ntiles = ((A.gx + 31) / 32) * ((A.gy + 7) / 8), nzc = (A.gz + GR_ZC - 1) / GR_ZC;
        const int ngroups = (nsys + sg - 1) / sg;
        const long blocks = (long)ngroups * ntiles * nzc;
        if (blocks <= 0x7fffffffL) {
            const auto *cf = (const typename CT<R>::t *)A.grid;
#define GRID_LAUNCH_(SGV)                                                                                              \
    k_grid_spmm<R, SGV><<<(unsigned)blocks, NT, 0, st>>>(A.gx, A.gy, A.gz, ngroups, ntiles, A.greal, cf, x, strideX, y, \
                                                         strideY, act, nsys, scale, vout, strideVO)
            if (sg == 1)
                GRID_LAUNCH_(1);
            else if (sg == 2)
                GRID_LAUNCH_(2);
            else
                GRID_LAUNCH_(4);
#undef GRID_LAUNCH_
            return;
        }
    }
    if (nsys == 1) {
        const long chunks = ((long)A.n + 2 * NT - 1) / (2 * NT);
        k_spmv2<R><<<(unsigned)chunks, NT, 0, st>>>(A.n, A.slice_ptr, A.cols, (const typename CT<R>::t *)A.vals, x,
                                                    strideX, y, strideY, act, sell_pattern(A), scale, vout,
                                                    strideVO);
        return;
    }
    constexpr int SG = 8;
    int rows = (A.n + NT - 1) / NT;
    dim3 grid((nsys + SG - 1) / SG, rows < 65535 ? rows : 65535);
    k_spmm<R, SG><<<grid, NT, 0, st>>>(A.n, A.slice_ptr, A.cols, (const typename CT<R>::t *)A.vals, x, strideX, y,
                                       strideY, act, nsys, sell_pattern(A), scale, vout, strideVO);
}

template <class R>
void launch_stencil(const Stencil7 &S, const typename CT<R>::t *x, size_t strideX, typename CT<R>::t *y,
                    size_t strideY, const int *act, int nsys, cudaStream_t st, const SysState *scale,
                    typename CT<R>::t *vout, size_t strideVO) {
    if (nsys <= 0) return;
    const double n = (double)S.nx * S.ny * S.nz;
    // x read once, y written (and v = a x written with the normalisation folded in)
    Launch L_(KC_SPMM, (scale ? 3.0 : 2.0) * nsys * n * sizeof(typename CT<R>::t), st, 1);
    const int tiles = ((S.nx + 31) / 32) * ((S.ny + 7) / 8);
    const dim3 grid(tiles, (S.nz + ST_ZC - 1) / ST_ZC, nsys);
    k_stencil<R><<<grid, NT, 0, st>>>(S.nx, S.ny, S.nz, S.d, S.wx, S.wy, S.wz, x, strideX, y, strideY, act, scale,
                                      vout, strideVO);
}

int resid_pattern(const SellMatrix &A, ResidPattern &rp) {
    rp = ResidPattern{};
    if (A.npat <= 0 || !A.uniform || !A.preal) return -1;
    rp.uniform = A.uniform;
    int j = 0;
    for (int e = 0; e < A.npat; ++e)
        if (!(A.preal >> e & 1u)) rp.idx[j++] = e;
    const int ncx = j;
    for (int e = 0; e < A.npat; ++e)
        if (A.preal >> e & 1u) rp.idx[j++] = e;
    for (int q = 0; q < A.npat; ++q) rp.off[q] = A.pat[rp.idx[q]];
    return ncx;
}

void launch_residual64(const SellMatrix &A, const double2 *b, size_t strideB, const double2 *x, size_t strideX,
                       double2 *r, size_t strideR, const int *act, int nsys, double2 *partials, unsigned *tickets,
                       SysState *state, cudaStream_t st, int per_sm) {
    if (nsys <= 0) return;
    Launch L_(KC_RESID64, spmm_bytes(A, sizeof(double2), nsys) + (double)sizeof(double2) * A.n * nsys, st, 1);
    ResidPattern rp{};
    const int ncx = resid_pattern(A, rp);
    const int Gv = capped_grid(A.n, nsys, 8);
    const int G = per_sm > 0 ? std::min(Gv, capped_grid(A.n, nsys, per_sm)) : Gv;
    const dim3 grid = grid2(nsys, G);
    resid_dispatch(A.npat, ncx, [&](auto ncx_c, auto wid_c) {
        k_residual64<decltype(ncx_c)::value, decltype(wid_c)::value><<<grid, NT, 0, st>>>(
            A.n, A.slice_ptr, A.cols, (const double2 *)A.vals, b, strideB, x, strideX, r, strideR, act, partials,
            tickets, state, rp, Gv);
    });
}

template <class R>
void launch_dense_gemv(int n, const typename CT<R>::t *A, const typename CT<R>::t *x, typename CT<R>::t *y,
                       cudaStream_t st) {
    Launch L_(KC_SPMM, (double)sizeof(typename CT<R>::t) * ((double)n * n + 2.0 * n), st, 1);
    k_dense_gemv<R><<<(n + NT - 1) / NT, NT, 0, st>>>(n, A, x, y);
}

template <class R>
void launch_copy_vec(int n, const typename CT<R>::t *src, size_t strideS, typename CT<R>::t *dst, size_t strideD,
                     const int *act, int nsys, cudaStream_t st) {
    if (nsys <= 0) return;
    Launch L_(KC_OTHER, (double)sizeof(typename CT<R>::t) * n * nsys * 2.0, st, 1);
    k_copy<R><<<grid2(stream_grid<R>(n, nsys), nsys), NT, 0, st>>>(n, src, strideS, dst, strideD, act);
}

template <class R>
void launch_refine_update(int n, double2 *x, size_t strideX, typename CT<R>::t *d, size_t strideD, const int *act,
                          int nsys, const SysState *state, cudaStream_t st) {
    if (nsys <= 0) return;
    Launch L_(KC_OTHER, (double)(sizeof(typename CT<R>::t) * 2 + sizeof(double2) * 2) * n * nsys, st, 1);
    k_refine_update<R><<<grid2(stream_grid<R>(n, nsys), nsys), NT, 0, st>>>(n, x, strideX, d, strideD, act, state);
}

template <class R>
void launch_demote_unit(int n, const double2 *r64, size_t strideR, typename CT<R>::t *rhat, size_t strideH,
                        typename CT<R>::t *v0, size_t strideV, const int *act, int nsys, const SysState *state,
                        cudaStream_t st) {
    if (nsys <= 0) return;
    Launch L_(KC_OTHER, (double)((v0 ? 2 : 1) * sizeof(typename CT<R>::t) + sizeof(double2)) * n * nsys, st, 1);
    k_demote_unit<R><<<grid2(stream_grid<R>(n, nsys), nsys), NT, 0, st>>>(n, r64, strideR, rhat, strideH, v0, strideV,
                                                                          act, state);
}

template <class R>
void launch_norm(int n, const typename CT<R>::t *v, size_t strideV, const int *act, int nsys, double2 *partials,
                 unsigned *tickets, SysState *state, int mode, cudaStream_t st) {
    if (nsys <= 0) return;
    Launch L_(KC_OTHER, (double)sizeof(typename CT<R>::t) * n * nsys, st, 1);
    k_norm<R><<<grid2(nsys, capped_grid(n, nsys, 8)), NT, 0, st>>>(n, v, strideV, act, partials, tickets, state, mode);
}

void launch_broadcast_hdef(int m, int kk, const double2 *Hd, double2 *H, size_t strideH, const int *act, int nsys,
                           cudaStream_t st) {
    if (nsys <= 0 || kk <= 0) return;
    Launch L_(KC_OTHER, 0.0, st, 1);
    k_broadcast_hdef<<<nsys, 256, 0, st>>>(m, kk, Hd, H, strideH, act);
}

#define GDMR_INST(R)                                                                                                   \
    template void launch_mdot<R>(int, const CT<R>::t *, int, const CT<R>::t *, size_t, int, const CT<R>::t *, size_t,  \
                                 const int *, int, double2 *, int, unsigned *, double2 *, size_t, SysState *, bool,   \
                                 cudaStream_t);                                                                        \
    template void launch_update<R>(int, const CT<R>::t *, int, const CT<R>::t *, size_t, int, const CT<R>::t *,        \
                                   size_t, CT<R>::t *, size_t, const int *, int, const double2 *, size_t, double2 *,   \
                                   unsigned *, SysState *, FinishArgs, bool, cudaStream_t);                            \
    template void launch_scale<R>(int, const CT<R>::t *, size_t, CT<R>::t *, size_t, CT<R>::t *, size_t, const int *, \
                                  int, const SysState *, bool, cudaStream_t);                                          \
    template void launch_combine<R>(int, int, int, const CT<R>::t *, const CT<R>::t *, const CT<R>::t *, size_t,       \
                                    CT<R>::t *, size_t, CT<R>::t *, size_t, const double2 *, const double2 *, size_t, \
                                    const int *, int, double2 *, unsigned *, SysState *, cudaStream_t);                \
    template void launch_zupdate<R>(int, int, int, int, const CT<R>::t *, const CT<R>::t *, size_t, const int *,       \
                                    const double2 *, CT<R>::t *, double2 *, unsigned *, double *, cudaStream_t);       \
    template void launch_znormalise<R>(int, int, const CT<R>::t *, const double *, CT<R>::t *, cudaStream_t);          \
    template void launch_spmm<R>(const SellMatrix &, const CT<R>::t *, size_t, CT<R>::t *, size_t, const int *, int,  \
                                 cudaStream_t, const SysState *, CT<R>::t *, size_t);                                 \
    template void launch_stencil<R>(const Stencil7 &, const CT<R>::t *, size_t, CT<R>::t *, size_t, const int *, int, \
                                    cudaStream_t, const SysState *, CT<R>::t *, size_t);                               \
    template void launch_dense_gemv<R>(int, const CT<R>::t *, const CT<R>::t *, CT<R>::t *, cudaStream_t);             \
    template void launch_copy_vec<R>(int, const CT<R>::t *, size_t, CT<R>::t *, size_t, const int *, int,              \
                                     cudaStream_t);                                                                    \
    template void launch_refine_update<R>(int, double2 *, size_t, CT<R>::t *, size_t, const int *, int,                \
                                          const SysState *, cudaStream_t);                                             \
    template void launch_demote_unit<R>(int, const double2 *, size_t, CT<R>::t *, size_t, CT<R>::t *, size_t,         \
                                        const int *, int, const SysState *, cudaStream_t);                             \
    template void launch_norm<R>(int, const CT<R>::t *, size_t, const int *, int, double2 *, unsigned *, SysState *,   \
                                 int, cudaStream_t);                                                                   \
    template int launch_krylov_multi<R>(const KrylovJob<R> *, const int *, int, int *, double, cudaStream_t);         \
    template bool launch_krylov_small<R>(int, int, int, const SellMatrix &, const CT<R>::t *, CT<R>::t *, size_t,      \
                                         const int *, SysState *, double2 *, size_t, double2 *, size_t, double *, int, \
                                         unsigned *, double, bool, cudaStream_t);

GDMR_INST(float)
GDMR_INST(double)
GDMR_INST(dfr)

}  // namespace gdmr
