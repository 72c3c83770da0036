// Tensor-core (tcgen05) projection of a batch onto the shared deflation basis.
//
// In a batched restart cycle every system orthogonalises its Krylov vector y_s against the
// same kk deflation vectors W (the deflator of the reference, gDMR.cu:1710-1787, applied to
// many right-hand sides at once).  The kk x nsys coefficients W^H Y are a GEMM with a huge
// K (= n) and tiny M, N, so this kernel runs it split-K on the 5th-generation tensor cores:
//
//   * complex -> real: with y, w viewed as interleaved real vectors of length 2n,
//       Re <w, y> = (wr, wi) . (yr, yi)      Im <w, y> = (-wi, wr) . (yr, yi)
//     so A has 2kk rows: w_p and its twin w'_p = (-wi, wr), and B has the nsys rows y_s;
//   * FP32 accuracy from TF32 inputs (3xTF32 with the fourth product for free): every
//     operand x is split into big = tf32(x) and small = x - big.  A is M = 128 rows:
//     rows 0-31 big(w), 32-63 big(w'), 64-95 small(w), 96-127 small(w'), and B has 2 np
//     rows: big(y) then small(y).  One MMA per K step (N = 2 np) forms all four products
//     big/small x big/small; coef is the sum of the four blocks of D;
//   * persistent CTAs (one per SM) walk K tiles of 32 complex elements in a warp-specialised
//     pipeline synchronised by mbarriers only: warps 0-15 load the raw tiles three tiles ahead
//     into registers (about 66 KB in flight per SM at 64 systems), split them into big/small
//     TF32 parts and store them in the 128-byte-swizzled K-major layout (coalesced 256-byte
//     row loads, conflict-free 16-byte stores) in one of three operand buffers, then arrive on
//     its "full" mbarrier;
//     warp 16 issues the MMAs and commits them to the buffer's "empty" mbarrier.  (Staging the
//     raw tiles with 256-byte bulk copies instead measured slower: 88 copies per tile.)
//   * tile i accumulates into TMEM region i mod 4 (4 x 128 columns), so no FP32 accumulation
//     chain is longer than a quarter of the CTA's tiles; at the end the regions are read
//     back (tcgen05.ld) and summed in double-float, the CTA's partials are written as doubles
//     and k_wproj_tc_reduce sums them over CTAs in a fixed order (deterministic).
//
// Every wait on an mbarrier is bounded: the pipeline's stage waits by the process's wait limit
// (about two seconds of clock by default), the final wait for every issued MMA by a fixed two
// seconds.  A timeout is counted in g_tc_timeouts; the kernel skips its remaining work, waits
// for the MMAs it issued and still frees its TMEM.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <type_traits>
#include <vector>

#include "gdmr_kernels.cuh"

namespace gdmr {
namespace {

constexpr int TC_PRODUCERS = 512;              // warps 0-15 load, split and store operand tiles
constexpr int TC_MMA_WARP = TC_PRODUCERS / 32; // warp 16 issues the MMAs
constexpr int TC_THREADS = TC_PRODUCERS + 32;
constexpr int TC_KT = 32;                      // complex elements per K tile
constexpr int TC_KCH = 2 * TC_KT / 4;          // 16-byte chunks per operand row per tile (2 swizzle atoms)
constexpr int TC_ROW = 128;                    // bytes per operand row inside a 128-byte swizzle atom
constexpr int TC_SBO = 1024;                   // 8-row swizzle atoms
constexpr int TC_M = 128;
constexpr int TC_NMAX = 64;
constexpr int TC_KMAX = 32;
constexpr int TC_NB = 3;                       // operand buffers
constexpr int TC_AHEAD = 3;                    // tiles whose loads are in flight ahead of the one stored
constexpr int TC_REGIONS = 4;                  // TMEM accumulators, 128 columns each, tiles round-robin
constexpr int TC_REGION_COLS = 128;            // [A big(y) | A small(y)], 2 x np <= 128 columns
constexpr int TC_TMEM_COLS = 512;
constexpr int TC_ITEMS = (TC_KMAX + TC_NMAX) * TC_KCH / TC_PRODUCERS;   // chunks per producer per tile
constexpr int TC_A_FLOATS = TC_M * 2 * TC_KT;
constexpr long long TC_WAIT_CYCLES = 4000000000LL;                       // ~2 s at 2 GHz

__device__ unsigned g_tc_timeouts = 0;
// bound of the pipeline stage waits: the process's wait limit in clock cycles; the waits on
// `done` (every MMA issued has finished, before TMEM is read and freed) keep TC_WAIT_CYCLES
__constant__ long long c_tc_wait_cycles = TC_WAIT_CYCLES;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor, K-major with 128-byte swizzle: rows of 128 bytes (32 tf32),
// 8-row atoms of 1024 bytes, the 16-byte chunk index of a row XOR-ed with (row & 7).
__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;                          // leading byte offset: unused for swizzled K-major
    d |= (uint64_t)((TC_SBO >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;                          // descriptor version of the sm_100 family
    d |= (uint64_t)2 << 61;                          // SWIZZLE_128B
    return d;
}

// kind::tf32 instruction descriptor: D f32, A and B tf32, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_tf32(int m, int n) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// Float offset of (row r, 16-byte chunk c of the tile's 256-byte row) in a 128-byte-swizzled
// K-major operand of `rows` rows: atom column c / 8, chunk (c % 8) XOR (r & 7).
__device__ __forceinline__ int sw_ofs(int r, int c, int rows) {
    return ((c >> 3) * rows * TC_ROW + r * TC_ROW + (((c & 7) ^ (r & 7)) << 4)) >> 2;
}

__device__ __forceinline__ float tf32_big(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t parity, volatile int *abort,
                                          long long limit = c_tc_wait_cycles) {
    const long long t0 = clock64();
    while (true) {
        uint32_t ok;
        // the thread may sleep in the instruction up to the hint (ns) until the phase completes
        asm volatile("{\n.reg .pred P;\nmbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2, %3;\nselp.b32 %0, 1, 0, P;\n}\n"
                     : "=r"(ok) : "r"(addr), "r"(parity), "r"(20000) : "memory");
        if (ok) return true;
        if ((abort && *abort) || clock64() - t0 > limit) return false;
    }
}

__device__ __forceinline__ void mbar_arrive(uint32_t addr) {
    asm volatile("{\n.reg .b64 st;\nmbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(addr) : "memory");
}

__device__ __forceinline__ void st4(float *p, float a, float b, float c, float d) {
    *reinterpret_cast<float4 *>(p) = make_float4(a, b, c, d);
}

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Double-float accumulate: (hi, lo) += v with the rounding error of the add kept in lo.
__device__ __forceinline__ void df_add(float &hi, float &lo, float v) {
    const float s = hi + v;
    const float bb = s - hi;
    const float err = (hi - (s - bb)) + (v - bb);
    hi = s;
    lo += err;
}

__device__ __forceinline__ void tmem_ld16(uint32_t addr, uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(addr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

// Lane 0 waits on an mbarrier phase and the warp follows its verdict (warp-uniform).
__device__ __forceinline__ bool warp_wait(uint32_t addr, uint32_t parity, volatile int *abort, int lane) {
    int ok = 1;
    if (lane == 0) {
        ok = mbar_wait(addr, parity, abort);
        if (!ok && !*abort) {
            atomicAdd(&g_tc_timeouts, 1u);
            *abort = 1;
        }
    }
    return __shfl_sync(0xffffffffu, ok, 0) != 0;
}

__global__ void __launch_bounds__(TC_THREADS, 1)
    k_wproj_tc(int n, int kk, const float2 *__restrict__ W, const float2 *__restrict__ Y0, size_t strideY,
               const int *__restrict__ act, int nsys, int np, double *__restrict__ part) {
    extern __shared__ __align__(1024) unsigned char tc_sm[];
    // operand buffer b: A (128 rows), then B = [big(y) rows; small(y) rows] (2 np rows); the
    // swizzle atoms need 1024-byte alignment, so the buffers start at the next 1 KB boundary
    float *ops = reinterpret_cast<float *>(tc_sm + ((1024u - (smem_u32(tc_sm) & 1023u)) & 1023u));
    const int b_floats = np * 2 * TC_KT, buf_floats = TC_A_FLOATS + 2 * b_floats;
    __shared__ __align__(8) uint64_t full[TC_NB], empty[TC_NB], done;
    __shared__ uint32_t tmem_base;
    __shared__ int s_act[TC_NMAX];
    __shared__ volatile int s_abort;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, G = gridDim.x;
    const long ntiles = ((long)n + TC_KT - 1) / TC_KT;
    const int my_tiles = (int)((ntiles - blockIdx.x + G - 1) / G);

    // zero the operand rows that are never written: A rows of p >= kk (all four row sets),
    // B rows of s >= nsys (big and small); 16 float4 per row (both swizzle atom columns)
    {
        const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
        const int arows = 32 - kk, brows = np - nsys;
        const int per_buf = (4 * arows + 2 * brows) * TC_KCH;
        for (int e = tid; e < TC_NB * per_buf; e += TC_THREADS) {
            const int b = e / per_buf, le = e % per_buf, c = le % TC_KCH, rr = le / TC_KCH;
            float *base = ops + (size_t)b * buf_floats;
            int r, rows;
            if (rr < 4 * arows) {
                r = (rr / arows) * 32 + kk + rr % arows;
                rows = TC_M;
            } else {
                const int q = rr - 4 * arows;
                base += TC_A_FLOATS;
                r = (q / brows) * np + nsys + q % brows;
                rows = 2 * np;
            }
            *reinterpret_cast<float4 *>(base + sw_ofs(r, c, rows)) = z;
        }
    }
    if (tid < nsys) s_act[tid] = act[tid];
    if (tid == 0) {
        s_abort = 0;
        for (int b = 0; b < TC_NB; ++b) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(&full[b])), "r"(TC_PRODUCERS / 32));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&empty[b])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&done)));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_base)),
                     "n"(TC_TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t taddr = tmem_base;

    if (warp < TC_MMA_WARP) {
        // ---- producers.  Chunk items of a tile: the kk W rows, then the nsys Y rows, 16 chunks
        // of 16 bytes each, chunk fastest: a warp loads two rows' 256-byte segments (coalesced)
        // and the eight lanes of a 16-byte store phase fill one swizzled 128-byte row (distinct banks).
        const int witems = kk * TC_KCH, items = witems + nsys * TC_KCH;
        const float2 *gp[TC_ITEMS];
        int so[TC_ITEMS], c2[TC_ITEMS], kind[TC_ITEMS];   // kind: 0 none, 1 W row, 2 Y row
#pragma unroll
        for (int u = 0; u < TC_ITEMS; ++u) {
            const int e = tid + u * TC_PRODUCERS;
            kind[u] = 0;
            gp[u] = W;
            so[u] = c2[u] = 0;
            if (e < items) {
                const bool isw = e < witems;
                const int le = isw ? e : e - witems;
                const int r = le / TC_KCH, c = le % TC_KCH;
                c2[u] = 2 * c;
                if (isw) {
                    kind[u] = 1;
                    so[u] = sw_ofs(r, c, TC_M);
                    gp[u] = W + (size_t)r * n + 2 * c;
                } else {
                    kind[u] = 2;
                    so[u] = TC_A_FLOATS + sw_ofs(r, c, 2 * np);
                    gp[u] = Y0 + (size_t)s_act[r] * strideY + 2 * c;
                }
            }
        }
        auto load_tile = [&](long t, float4(&dst)[TC_ITEMS]) {
#pragma unroll
            for (int u = 0; u < TC_ITEMS; ++u) {
                float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                if (kind[u] && t * TC_KT + c2[u] < n) v = *reinterpret_cast<const float4 *>(gp[u] + t * TC_KT);
                dst[u] = v;
            }
        };
        auto store_tile = [&](float *buf0, const float4(&src)[TC_ITEMS]) {
#pragma unroll
            for (int u = 0; u < TC_ITEMS; ++u) {
                if (!kind[u]) continue;
                const float4 v = src[u];
                const float b0 = tf32_big(v.x), b1 = tf32_big(v.y), b2 = tf32_big(v.z), b3 = tf32_big(v.w);
                const float s0 = v.x - b0, s1 = v.y - b1, s2 = v.z - b2, s3 = v.w - b3;
                float *a = buf0 + so[u];
                if (kind[u] == 1) {   // rows r, 32+r, 64+r, 96+r: same swizzle, 32 rows apart
                    st4(a, b0, b1, b2, b3);
                    st4(a + 32 * TC_ROW / 4, -b1, b0, -b3, b2);
                    st4(a + 64 * TC_ROW / 4, s0, s1, s2, s3);
                    st4(a + 96 * TC_ROW / 4, -s1, s0, -s3, s2);
                } else {              // big(y) row s and small(y) row np + s (np a multiple of 8)
                    st4(a, b0, b1, b2, b3);
                    st4(a + np * TC_ROW / 4, s0, s1, s2, s3);
                }
            }
        };
        // register ring of TC_AHEAD + 1 tiles; the loop is unrolled by four so every slot is a
        // fixed set of registers (slot i % 4 is stored while slot (i + 3) % 4 is being loaded)
        float4 R0[TC_ITEMS], R1[TC_ITEMS], R2[TC_ITEMS], R3[TC_ITEMS];
        static_assert(TC_AHEAD == 3, "the ring below has four slots");
        const long t0 = blockIdx.x;
        if (my_tiles > 0) load_tile(t0, R0);
        if (my_tiles > 1) load_tile(t0 + G, R1);
        if (my_tiles > 2) load_tile(t0 + 2 * G, R2);
        auto step = [&](auto S, int i) -> bool {
            constexpr int sl = decltype(S)::value;
            float4(&cur)[TC_ITEMS] = sl == 0 ? R0 : sl == 1 ? R1 : sl == 2 ? R2 : R3;
            float4(&fut)[TC_ITEMS] = sl == 0 ? R3 : sl == 1 ? R0 : sl == 2 ? R1 : R2;
            const int buf = i % TC_NB;
            if (i + TC_AHEAD < my_tiles) load_tile(t0 + (long)(i + TC_AHEAD) * G, fut);
            if (i >= TC_NB && !warp_wait(smem_u32(&empty[buf]), ((i / TC_NB) - 1) & 1, &s_abort, lane)) return false;
            store_tile(ops + (size_t)buf * buf_floats, cur);
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&full[buf]));
            return true;
        };
        for (int i = 0; i < my_tiles; i += 4) {
            if (!step(std::integral_constant<int, 0>{}, i)) break;
            if (i + 1 >= my_tiles || !step(std::integral_constant<int, 1>{}, i + 1)) break;
            if (i + 2 >= my_tiles || !step(std::integral_constant<int, 2>{}, i + 2)) break;
            if (i + 3 >= my_tiles || !step(std::integral_constant<int, 3>{}, i + 3)) break;
        }
    } else if (warp == TC_MMA_WARP) {
        if (lane == 0) {
            // ---- MMA issuer: one MMA per K step with N = 2 np, B = [big(y) rows; small(y) rows];
            // tile i accumulates into TMEM region i % TC_REGIONS.  K step ks reads swizzle atom
            // column ks / 4 at byte offset (ks % 4) * 32 inside the 128-byte rows; only the
            // start-address field of the descriptors changes (no carry below 256 KB).
            const uint32_t idesc = idesc_tf32(TC_M, 2 * np);
            const uint64_t adesc0 = sdesc(smem_u32(ops)), bdesc0 = sdesc(smem_u32(ops) + TC_A_FLOATS * 4);
            const uint64_t buf_step = (uint64_t)(buf_floats * 4) >> 4;   // start-address units per buffer
            const uint64_t acol = (uint64_t)(TC_M * TC_ROW) >> 4, bcol = (uint64_t)(2 * np * TC_ROW) >> 4;
            for (int i = 0; i < my_tiles; ++i) {
                const int buf = i % TC_NB;
                if (!mbar_wait(smem_u32(&full[buf]), (i / TC_NB) & 1, &s_abort)) {
                    if (!s_abort) { atomicAdd(&g_tc_timeouts, 1u); s_abort = 1; }
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint64_t ad0 = adesc0 + buf * buf_step, bd0 = bdesc0 + buf * buf_step;
                const uint32_t d = taddr + (uint32_t)((i % TC_REGIONS) * TC_REGION_COLS);
                asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                             "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
                             "l"(ad0), "l"(bd0), "r"(idesc), "r"(i >= TC_REGIONS ? 1u : 0u));
#pragma unroll
                for (int ks = 1; ks < 2 * TC_KT / 8; ++ks) {
                    const uint64_t koff = (uint64_t)((ks & 3) * 32) >> 4;
                    const uint64_t ad = ad0 + (ks >> 2) * acol + koff, bd = bd0 + (ks >> 2) * bcol + koff;
                    asm volatile("tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, 1;\n" ::"r"(d), "l"(ad),
                                 "l"(bd), "r"(idesc));
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                                 smem_u32(&empty[buf]))
                             : "memory");
            }
            // completes when every MMA issued above has finished (also after an abort)
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             smem_u32(&done))
                         : "memory");
        }
    }
    __syncthreads();
    if (!mbar_wait(smem_u32(&done), 0, nullptr, TC_WAIT_CYCLES) && tid == 0) {
        atomicAdd(&g_tc_timeouts, 1u);
        s_abort = 1;
    }
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    __syncthreads();
    // ---- sum the regions (double-float), then big + small rows, through shared memory
    float *acc_hi = ops, *acc_lo = ops + nsys * 2 * 32;   // [s][re|im][32]; operand buffers are free now
    const int used = my_tiles < TC_REGIONS ? my_tiles : TC_REGIONS;
    for (int phase = 0; phase < 2; ++phase) {
        if (warp < 4 && (warp >> 1) == phase && !s_abort) {
            const int m = warp * 32 + lane, p = m & 31, ri = (m >> 5) & 1;
            for (int c0 = 0; c0 < np; c0 += 16) {
                float hi[16], lo[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) hi[j] = lo[j] = 0.f;
                for (int rg = 0; rg < used; ++rg)
                    for (int half = 0; half < 2; ++half) {   // columns of big(y), then of small(y)
                        uint32_t v[16];
                        tmem_ld16(taddr + ((uint32_t)(warp * 32) << 16) +
                                      (uint32_t)(rg * TC_REGION_COLS + half * np + c0),
                                  v);
#pragma unroll
                        for (int j = 0; j < 16; ++j) df_add(hi[j], lo[j], __uint_as_float(v[j]));
                    }
                if (p < kk) {
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const int s = c0 + j;
                        if (s >= nsys) break;
                        const int o = (s * 2 + ri) * 32 + p;
                        if (phase == 0) {
                            acc_hi[o] = hi[j];
                            acc_lo[o] = lo[j];
                        } else {
                            df_add(acc_hi[o], acc_lo[o], hi[j]);
                            acc_lo[o] += lo[j];
                        }
                    }
                }
            }
        }
        __syncthreads();
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "n"(TC_TMEM_COLS));
    // this CTA's partials, contiguous: part[blockIdx.x][p*nsys + s][re|im]
    double *pc = part + (size_t)blockIdx.x * kk * nsys * 2;
    for (int e = tid; e < kk * nsys * 2; e += TC_THREADS) {
        const int o = e >> 1, p = o / nsys, s = o % nsys, ri = e & 1;
        const int idx = (s * 2 + ri) * 32 + p;
        pc[e] = s_abort ? 0.0 : (double)acc_hi[idx] + (double)acc_lo[idx];
    }
}

// coef_s[p] = sum over the G CTAs of part[g][p*nsys + s]: 32 outputs per CTA, lane = output
// (coalesced reads across outputs), warp w sums the CTAs g = w, w + 8, ... in order, and the
// eight warp sums are added in warp order (deterministic).
__global__ void __launch_bounds__(256) k_wproj_tc_reduce(int kk, int nsys, int G, const double *__restrict__ part,
                                                         const int *__restrict__ act, double2 *__restrict__ coef0,
                                                         size_t strideC) {
    __shared__ double2 red[8][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int o = blockIdx.x * 32 + lane, O = kk * nsys;
    double re = 0, im = 0;
    if (o < O) {
#pragma unroll 4
        for (int g = warp; g < G; g += 8) {
            const double2 v = *reinterpret_cast<const double2 *>(part + ((size_t)g * O + o) * 2);
            re += v.x;
            im += v.y;
        }
    }
    red[warp][lane] = make_double2(re, im);
    __syncthreads();
    if (warp == 0 && o < O) {
        double2 t = red[0][lane];
#pragma unroll
        for (int w = 1; w < 8; ++w) {
            t.x += red[w][lane].x;
            t.y += red[w][lane].y;
        }
        coef0[(size_t)act[o % nsys] * strideC + o / nsys] = t;
    }
}

// ================================================================ batched shared-basis apply
// P_s = W c_s for every active system s (c_s = coef_s[0:kk], the projection onto the shared
// deflation vectors), written into the caller's slot for s (the next Krylov vector's slot),
// so that the update out_s = y_s - P_s - V_s c_s^V runs as a per-system update with P_s as one
// more basis vector of coefficient 1 (written here at coef_s[unit_idx]).
//
// Real GEMM on the tensor cores (kind::tf32), one 128-element tile of W per step:
//   A (M = 128 rows = elements, K = 2kk reals (wr_p, wi_p)), split big/small into two operands;
//   B (N = 4 NSp rows, K = 2kk): rows [big | small] x system x (re, im output) with
//     re row: (cr_p, -ci_p), im row: (ci_p, cr_p), so D[i][(s,re)] = Re(w_i c_s), D[i][(s,im)] = Im;
//   per K step: A_big x B (N = 4 NSp) and A_small x B_big (N = 2 NSp) into one TMEM tile, and
//   P = D[:, big block] + D[:, small block].
// Warp roles: warps 0 .. WA_EPI-1 epilogue (warp w reads TMEM lane quarter w % 4, the tile's
// elements 32 (w % 4) .. + 31, and stores P for every (WA_EPI / 4)-th group of 8 systems from
// group w / 4; four warps of stores ran the kernel at about half the HBM rate), the next WA_PROD
// warps producers (W tile -> split, swizzled A operands), the last warp issues the MMAs.  A and
// the TMEM tile are double-buffered; mbarriers only.
constexpr int WA_EPI = 8, WA_PROD = 8;
constexpr int WA_MMA_WARP = WA_EPI + WA_PROD;
constexpr int WA_THREADS = (WA_MMA_WARP + 1) * 32;
constexpr int WA_TILE = 128;                      // elements per tile (MMA M)
constexpr int WA_AOP = WA_TILE * 2 * TC_ROW;      // bytes of one A operand (2 swizzle atom columns)
constexpr int WA_ITEMS = TC_KMAX * WA_TILE / (WA_PROD * 32);   // W values per producer per tile

__device__ __forceinline__ int swz(int r, int kf, int rows) {   // float offset of (row, K float)
    return ((kf >> 5) * rows * TC_ROW + r * TC_ROW + ((((kf >> 2) & 7) ^ (r & 7)) << 4) + ((kf & 3) << 2)) >> 2;
}

__global__ void __launch_bounds__(WA_THREADS, 1)
    k_wapply_tc(int n, int kk, const float2 *__restrict__ W, double2 *__restrict__ coef0, size_t strideC,
                const int *__restrict__ act, int nsys, int nsp, float2 *__restrict__ P0, size_t strideP,
                int unit_idx) {
    extern __shared__ __align__(1024) unsigned char wa_sm[];
    unsigned char *base = wa_sm + ((1024u - (smem_u32(wa_sm) & 1023u)) & 1023u);
    float *A = reinterpret_cast<float *>(base);                       // [buf][big|small] operands
    float *B = reinterpret_cast<float *>(base + 4 * WA_AOP);          // 4 nsp rows x 2 atom columns
    const int brows = 4 * nsp;
    __shared__ __align__(8) uint64_t full[2], mdone[2], tempty[2], done;
    __shared__ uint32_t tmem_base;
    __shared__ int s_act[TC_NMAX];
    __shared__ volatile int s_abort;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, G = gridDim.x;
    const long ntiles = ((long)n + WA_TILE - 1) / WA_TILE;
    const int my_tiles = (int)((ntiles - blockIdx.x + G - 1) / G);

    // zero both A buffers (padded K stays zero) and B, then fill B from the coefficients
    for (int e = tid; e < (4 * WA_AOP + brows * 2 * TC_ROW) / 16; e += WA_THREADS)
        reinterpret_cast<float4 *>(base)[e] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (tid < nsys) s_act[tid] = act[tid];
    if (tid == 0) {
        s_abort = 0;
        for (int b = 0; b < 2; ++b) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(&full[b])), "r"(WA_PROD));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mdone[b])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(&tempty[b])), "r"(WA_EPI));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&done)));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_base)),
                     "n"(TC_TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    __syncthreads();
    for (int e = tid; e < nsys * kk; e += WA_THREADS) {
        const int sl = e / kk, p = e % kk;
        const double2 c = coef0[(size_t)s_act[sl] * strideC + p];
        const float cr = (float)c.x, ci = (float)c.y;
        const float vals[2][2] = {{cr, -ci}, {ci, cr}};   // [output re|im][K 2p, 2p+1]
#pragma unroll
        for (int o = 0; o < 2; ++o)
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const float v = vals[o][q], big = tf32_big(v);
                B[swz(2 * sl + o, 2 * p + q, brows)] = big;
                B[swz(2 * nsp + 2 * sl + o, 2 * p + q, brows)] = v - big;
            }
    }
    if (blockIdx.x == 0 && tid < nsys) coef0[(size_t)s_act[tid] * strideC + unit_idx] = make_double2(1.0, 0.0);
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t taddr = tmem_base;

    if (warp >= WA_EPI && warp < WA_MMA_WARP) {
        // ---- producers: W tile (kk vectors x 128 elements, lane = element: coalesced) ->
        // big/small A operands, K position 2p (re) and 2p + 1 (im) of row = element
        const int ptid = tid - WA_EPI * 32;
        float2 cur[WA_ITEMS], nxt[WA_ITEMS];
        auto load = [&](long t, float2(&dst)[WA_ITEMS]) {
#pragma unroll
            for (int u = 0; u < WA_ITEMS; ++u) {
                const int e = ptid + u * WA_PROD * 32, p = e / WA_TILE, i = e % WA_TILE;
                const long g = t * WA_TILE + i;
                dst[u] = (p < kk && g < n) ? W[(size_t)p * n + g] : make_float2(0.f, 0.f);
            }
        };
        const long t0 = blockIdx.x;
        if (my_tiles > 0) load(t0, cur);
        for (int i = 0; i < my_tiles; ++i) {
            const int buf = i & 1;
            if (i + 1 < my_tiles) load(t0 + (long)(i + 1) * G, nxt);
            if (i >= 2) {   // the MMAs of tile i - 2 read this A buffer
                int ok = 1;
                if (lane == 0) {
                    ok = mbar_wait(smem_u32(&mdone[buf]), ((i >> 1) - 1) & 1, &s_abort);
                    if (!ok && !s_abort) { atomicAdd(&g_tc_timeouts, 1u); s_abort = 1; }
                }
                if (!__shfl_sync(0xffffffffu, ok, 0)) break;
            }
            float *Ab = A + (size_t)buf * 2 * (WA_AOP / 4), *As = Ab + WA_AOP / 4;
#pragma unroll
            for (int u = 0; u < WA_ITEMS; ++u) {
                const int e = ptid + u * WA_PROD * 32, p = e / WA_TILE, r = e % WA_TILE;
                if (p >= kk) continue;
                const float br = tf32_big(cur[u].x), bi = tf32_big(cur[u].y);
                const int o = swz(r, 2 * p, WA_TILE);   // 2p and 2p + 1 share a 16-byte chunk
                *reinterpret_cast<float2 *>(Ab + o) = make_float2(br, bi);
                *reinterpret_cast<float2 *>(As + o) = make_float2(cur[u].x - br, cur[u].y - bi);
            }
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&full[buf]));
#pragma unroll
            for (int u = 0; u < WA_ITEMS; ++u) cur[u] = nxt[u];
        }
    } else if (warp == WA_MMA_WARP) {
        if (lane == 0) {
            const int ksteps = (2 * kk + 7) / 8;
            const uint32_t id_all = idesc_tf32(TC_M, 4 * nsp), id_big = idesc_tf32(TC_M, 2 * nsp);
            const uint64_t a0 = sdesc(smem_u32(A)), b0 = sdesc(smem_u32(B));
            const uint64_t abuf = (uint64_t)(2 * WA_AOP) >> 4, asmall = (uint64_t)WA_AOP >> 4;
            const uint64_t acol = (uint64_t)(WA_TILE * TC_ROW) >> 4, bcol = (uint64_t)(brows * TC_ROW) >> 4;
            for (int i = 0; i < my_tiles; ++i) {
                const int buf = i & 1;
                if (!mbar_wait(smem_u32(&full[buf]), (i >> 1) & 1, &s_abort) ||
                    (i >= 2 && !mbar_wait(smem_u32(&tempty[buf]), ((i >> 1) - 1) & 1, &s_abort))) {
                    if (!s_abort) { atomicAdd(&g_tc_timeouts, 1u); s_abort = 1; }
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t d = taddr + (uint32_t)(buf * 256);
                for (int ks = 0; ks < ksteps; ++ks) {
                    const uint64_t koff = (uint64_t)((ks & 3) * 32) >> 4;
                    const uint64_t ab = a0 + buf * abuf + (ks >> 2) * acol + koff;
                    const uint64_t bd = b0 + (ks >> 2) * bcol + koff;
                    asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                                 "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
                                 "l"(ab), "l"(bd), "r"(id_all), "r"(ks > 0 ? 1u : 0u));
                    asm volatile("tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, 1;\n" ::"r"(d),
                                 "l"(ab + asmall), "l"(bd), "r"(id_big));
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                                 smem_u32(&mdone[buf]))
                             : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             smem_u32(&done))
                         : "memory");
        }
    } else {
        // ---- epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 = elements of the tile, sums
        // the big and small blocks and stores P_s (lanes = consecutive elements) for the systems
        // of every other group of 16 columns (8 systems), starting at group w / 4
        const int quarter = warp & 3, part = warp >> 2;
        for (int i = 0; i < my_tiles; ++i) {
            const int buf = i & 1;
            int ok = 1;
            if (lane == 0) {
                ok = mbar_wait(smem_u32(&mdone[buf]), (i >> 1) & 1, &s_abort);
                if (!ok && !s_abort) { atomicAdd(&g_tc_timeouts, 1u); s_abort = 1; }
            }
            if (!__shfl_sync(0xffffffffu, ok, 0)) break;
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const long g = ((long)blockIdx.x + (long)i * G) * WA_TILE + quarter * 32 + lane;
            const uint32_t row = taddr + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(buf * 256);
            for (int c0 = 16 * part; c0 < 2 * nsp; c0 += 16 * (WA_EPI / 4)) {
                uint32_t vb[16], vs[16];
                tmem_ld16(row + (uint32_t)c0, vb);
                tmem_ld16(row + (uint32_t)(2 * nsp + c0), vs);
                if (g < n) {
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        const int sl = c0 / 2 + j;
                        if (sl < nsys)
                            P0[(size_t)s_act[sl] * strideP + g] =
                                make_float2(__uint_as_float(vb[2 * j]) + __uint_as_float(vs[2 * j]),
                                            __uint_as_float(vb[2 * j + 1]) + __uint_as_float(vs[2 * j + 1]));
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&tempty[buf]));
        }
    }
    __syncthreads();
    if (!mbar_wait(smem_u32(&done), 0, nullptr, TC_WAIT_CYCLES) && tid == 0) atomicAdd(&g_tc_timeouts, 1u);
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "n"(TC_TMEM_COLS));
}

// ================================================================ fused shared-basis update
// The whole batched Gram-Schmidt update of a Krylov step in one kernel:
//   out_s = w_s - V_s c_s^V - W c_s^W,   ||out_s||^2 and <out_s, w_s> reduced, then the update's
//   finish (Hessenberg column, breakdown test and identity tail, normalisation factor) per system,
// the classical Gram-Schmidt step of arnoldiDMR against [W V] with the deflator (gDMR.cu:1710-1787,
// 2115-2310) for a batch of systems that share W.  The shared part W c_s^W of every system comes
// from the tensor cores with the operands and MMAs of k_wapply_tc, and the epilogue warps take it
// straight from TMEM while they stream w_s and V_s, so it never goes through memory (the split
// form writes P_s = W c_s^W and the per-system update reads it back: two extra vectors a system).
//   * warps 0-15 epilogue: warp w reads TMEM lane quarter w % 4 (the tile's elements 32 (w % 4) ..
//     + 31, one a lane) and handles the systems 16 (w / 4) .. + 15; per element and system it
//     subtracts the own basis in the order of the per-system update kernel, then P, stores out and
//     accumulates the two reductions (warp sums per tile, FP64 slots per lane quarter and system);
//   * warps 16-23 produce the big/small TF32 A operands of each 128-element W tile;
//   * warp 24 issues the MMAs into one of two TMEM tiles (256 columns each).
// After the last tile every CTA writes its partial sums per system and arrives on the system's
// ticket; the last CTA of a system sums the partials over the CTAs in order (deterministic) and
// runs the finish.  Systems flagged broken are skipped when skip_broken is set, as in k_update.
constexpr int WU_EPI = 16, WU_PROD = 8;
constexpr int WU_MMA_WARP = WU_EPI + WU_PROD;
constexpr int WU_THREADS = (WU_MMA_WARP + 1) * 32;
constexpr int WU_QB = 32;                                      // own basis vectors at most
constexpr int WU_ITEMS = TC_KMAX * WA_TILE / (WU_PROD * 32);   // W values per producer per tile

__device__ __forceinline__ void tmem_ld8(uint32_t addr, uint32_t (&v)[8]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
                 : "r"(addr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

__device__ __forceinline__ void cfms2(float2 &acc, float2 c, float2 v) {   // acc -= c * v (k_update's order)
    acc.x = fmaf(-c.x, v.x, acc.x);
    acc.x = fmaf(c.y, v.y, acc.x);
    acc.y = fmaf(-c.x, v.y, acc.y);
    acc.y = fmaf(-c.y, v.x, acc.y);
}

__global__ void __launch_bounds__(WU_THREADS, 1)
    k_wupdate_tc(int n, int kk, const float2 *__restrict__ W, const float2 *__restrict__ V0, size_t strideV, int qb,
                 const float2 *__restrict__ w0, size_t strideW, float2 *__restrict__ out0, size_t strideO,
                 const int *__restrict__ act, int nsys, int nsp, const double2 *__restrict__ coef0, size_t strideC,
                 double *__restrict__ partials, unsigned *tickets, SysState *state, FinishArgs fin, int skip_broken) {
    extern __shared__ __align__(1024) unsigned char wu_sm[];
    unsigned char *base = wu_sm + ((1024u - (smem_u32(wu_sm) & 1023u)) & 1023u);
    const int brows = 4 * nsp;
    float *A = reinterpret_cast<float *>(base);                        // [buf][big|small]
    float *B = reinterpret_cast<float *>(base + 4 * WA_AOP);           // 4 nsp rows x 2 atom columns
    float2 *cv = reinterpret_cast<float2 *>(base + 4 * WA_AOP + (size_t)brows * 2 * TC_ROW);   // [sys][WU_QB]
    // per lane quarter and system: the tiles' warp sums in FP32 (an FP64 add per system, tile and
    // warp was about the epilogue's memory time on GB300's FP64 pipe); FP64 once per CTA
    float *sacc = reinterpret_cast<float *>(cv + (size_t)TC_NMAX * WU_QB);                     // [quarter][sys][3]
    __shared__ __align__(8) uint64_t full[2], mdone[2], tempty[2], done;
    __shared__ uint32_t tmem_base;
    __shared__ int s_act[TC_NMAX], s_skip[TC_NMAX];
    __shared__ volatile int s_abort;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, G = gridDim.x;
    const long ntiles = ((long)n + WA_TILE - 1) / WA_TILE;
    const int my_tiles = (int)((ntiles - blockIdx.x + G - 1) / G);

    for (int e = tid; e < (4 * WA_AOP + brows * 2 * TC_ROW) / 16; e += WU_THREADS)
        reinterpret_cast<float4 *>(base)[e] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int e = tid; e < 4 * TC_NMAX * 3; e += WU_THREADS) sacc[e] = 0.f;
    if (tid < nsys) {
        const int sy = act[tid];
        s_act[tid] = sy;
        s_skip[tid] = skip_broken && state[sy].broken;
    }
    if (tid == 0) {
        s_abort = 0;
        for (int b = 0; b < 2; ++b) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(&full[b])), "r"(WU_PROD));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mdone[b])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(&tempty[b])), "r"(WU_EPI));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&done)));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_base)),
                     "n"(TC_TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    __syncthreads();
    // B from the shared coefficients (as k_wapply_tc), cv from the own coefficients
    for (int e = tid; e < nsys * kk; e += WU_THREADS) {
        const int sl = e / kk, p = e % kk;
        const double2 c = coef0[(size_t)s_act[sl] * strideC + p];
        const float cr = (float)c.x, ci = (float)c.y;
        const float vals[2][2] = {{cr, -ci}, {ci, cr}};
#pragma unroll
        for (int o = 0; o < 2; ++o)
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const float v = vals[o][q], big = tf32_big(v);
                B[swz(2 * sl + o, 2 * p + q, brows)] = big;
                B[swz(2 * nsp + 2 * sl + o, 2 * p + q, brows)] = v - big;
            }
    }
    for (int e = tid; e < nsys * qb; e += WU_THREADS) {
        const int sl = e / qb, p = e % qb;
        const double2 c = coef0[(size_t)s_act[sl] * strideC + kk + p];
        cv[sl * WU_QB + p] = make_float2((float)c.x, (float)c.y);
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t taddr = tmem_base;

    if (warp >= WU_EPI && warp < WU_MMA_WARP) {
        // ---- producers (as k_wapply_tc, without its register prefetch of the next tile: 800
        // threads leave 80 registers a thread, and a tile's W loads take a small part of the
        // epilogue's time for the same tile)
        const int ptid = tid - WU_EPI * 32;
        float2 cur[WU_ITEMS];
        const long t0 = blockIdx.x;
        for (int i = 0; i < my_tiles; ++i) {
            const int buf = i & 1;
#pragma unroll
            for (int u = 0; u < WU_ITEMS; ++u) {
                const int e = ptid + u * WU_PROD * 32, p = e / WA_TILE, r = e % WA_TILE;
                const long g = (t0 + (long)i * G) * WA_TILE + r;
                cur[u] = (p < kk && g < n) ? W[(size_t)p * n + g] : make_float2(0.f, 0.f);
            }
            if (i >= 2) {   // the MMAs of tile i - 2 read this A buffer
                int ok = 1;
                if (lane == 0) {
                    ok = mbar_wait(smem_u32(&mdone[buf]), ((i >> 1) - 1) & 1, &s_abort);
                    if (!ok && !s_abort) { atomicAdd(&g_tc_timeouts, 1u); s_abort = 1; }
                }
                if (!__shfl_sync(0xffffffffu, ok, 0)) break;
            }
            float *Ab = A + (size_t)buf * 2 * (WA_AOP / 4), *As = Ab + WA_AOP / 4;
#pragma unroll
            for (int u = 0; u < WU_ITEMS; ++u) {
                const int e = ptid + u * WU_PROD * 32, p = e / WA_TILE, r = e % WA_TILE;
                if (p >= kk) continue;
                const float br = tf32_big(cur[u].x), bi = tf32_big(cur[u].y);
                const int o = swz(r, 2 * p, WA_TILE);
                *reinterpret_cast<float2 *>(Ab + o) = make_float2(br, bi);
                *reinterpret_cast<float2 *>(As + o) = make_float2(cur[u].x - br, cur[u].y - bi);
            }
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&full[buf]));
        }
    } else if (warp == WU_MMA_WARP) {
        if (lane == 0) {
            // ---- MMA issuer (as k_wapply_tc)
            const int ksteps = (2 * kk + 7) / 8;
            const uint32_t id_all = idesc_tf32(TC_M, 4 * nsp), id_big = idesc_tf32(TC_M, 2 * nsp);
            const uint64_t a0 = sdesc(smem_u32(A)), b0 = sdesc(smem_u32(B));
            const uint64_t abuf = (uint64_t)(2 * WA_AOP) >> 4, asmall = (uint64_t)WA_AOP >> 4;
            const uint64_t acol = (uint64_t)(WA_TILE * TC_ROW) >> 4, bcol = (uint64_t)(brows * TC_ROW) >> 4;
            for (int i = 0; i < my_tiles; ++i) {
                const int buf = i & 1;
                if (!mbar_wait(smem_u32(&full[buf]), (i >> 1) & 1, &s_abort) ||
                    (i >= 2 && !mbar_wait(smem_u32(&tempty[buf]), ((i >> 1) - 1) & 1, &s_abort))) {
                    if (!s_abort) { atomicAdd(&g_tc_timeouts, 1u); s_abort = 1; }
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t d = taddr + (uint32_t)(buf * 256);
                for (int ks = 0; ks < ksteps; ++ks) {
                    const uint64_t koff = (uint64_t)((ks & 3) * 32) >> 4;
                    const uint64_t ab = a0 + buf * abuf + (ks >> 2) * acol + koff;
                    const uint64_t bd = b0 + (ks >> 2) * bcol + koff;
                    asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                                 "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
                                 "l"(ab), "l"(bd), "r"(id_all), "r"(ks > 0 ? 1u : 0u));
                    asm volatile("tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, 1;\n" ::"r"(d),
                                 "l"(ab + asmall), "l"(bd), "r"(id_big));
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                                 smem_u32(&mdone[buf]))
                             : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             smem_u32(&done))
                         : "memory");
        }
    } else {
        // ---- epilogue: the update proper
        const int quarter = warp & 3, group = warp >> 2;
        const int s_lo = group * 16, s_hi = min(nsys, s_lo + 16);
        float *myacc = sacc + (size_t)quarter * TC_NMAX * 3;
        for (int i = 0; i < my_tiles; ++i) {
            const int buf = i & 1;
            int ok = 1;
            if (lane == 0) {
                ok = mbar_wait(smem_u32(&mdone[buf]), (i >> 1) & 1, &s_abort);
                if (!ok && !s_abort) { atomicAdd(&g_tc_timeouts, 1u); s_abort = 1; }
            }
            if (!__shfl_sync(0xffffffffu, ok, 0)) break;
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const long e = ((long)blockIdx.x + (long)i * G) * WA_TILE + quarter * 32 + lane;
            const bool in = e < n;
            const uint32_t row = taddr + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(buf * 256);
            for (int s0 = s_lo; s0 < s_hi; s0 += 4) {
                uint32_t vb[8], vs[8];
                tmem_ld8(row + (uint32_t)(2 * s0), vb);
                tmem_ld8(row + (uint32_t)(2 * nsp + 2 * s0), vs);
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int sl = s0 + u;
                    if (sl >= s_hi || s_skip[sl]) continue;   // warp-uniform
                    const int sy = s_act[sl];
                    const float2 P = make_float2(__uint_as_float(vb[2 * u]) + __uint_as_float(vs[2 * u]),
                                                 __uint_as_float(vb[2 * u + 1]) + __uint_as_float(vs[2 * u + 1]));
                    float2 org = make_float2(0.f, 0.f), acc = org;
                    if (in) {
                        org = w0[(size_t)sy * strideW + e];
                        acc = org;
                        const float2 *vp = V0 + (size_t)sy * strideV + e;
                        const float2 *cs = cv + sl * WU_QB;
                        int p = 0;
                        for (; p + 8 <= qb; p += 8) {   // eight loads in flight before their use
                            float2 v[8];
#pragma unroll
                            for (int q = 0; q < 8; ++q) v[q] = vp[(size_t)(p + q) * n];
#pragma unroll
                            for (int q = 0; q < 8; ++q) cfms2(acc, cs[p + q], v[q]);
                        }
                        for (; p < qb; ++p) cfms2(acc, cs[p], vp[(size_t)p * n]);
                        cfms2(acc, make_float2(1.f, 0.f), P);
                        out0[(size_t)sy * strideO + e] = acc;
                    }
                    // ||out||^2 and <out, w> = sum conj(out) w, summed over the warp, into the
                    // lane quarter's FP64 slot of the system
                    float ln = acc.x * acc.x + acc.y * acc.y;
                    float cr = acc.x * org.x + acc.y * org.y, ci = acc.x * org.y - acc.y * org.x;
                    ln = warp_sum_f(ln);
                    cr = warp_sum_f(cr);
                    ci = warp_sum_f(ci);
                    if (lane == 0) {
                        myacc[sl * 3] += ln;
                        myacc[sl * 3 + 1] += cr;
                        myacc[sl * 3 + 2] += ci;
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&tempty[buf]));
        }
    }
    __syncthreads();
    if (!mbar_wait(smem_u32(&done), 0, nullptr, TC_WAIT_CYCLES) && tid == 0) {
        atomicAdd(&g_tc_timeouts, 1u);
        s_abort = 1;
    }
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "n"(TC_TMEM_COLS));
    // per system: this CTA's partials, then the ticket; the last CTA sums over the CTAs in order and
    // runs the finish.  Every CTA arrives (with zeros after an abort) so the tickets stay balanced.
    if (tid < nsys && !s_skip[tid]) {
        const int sl = tid;
        double *part = partials + (size_t)sl * 3 * G;
        for (int v = 0; v < 3; ++v) {
            double t = 0;
            for (int q = 0; q < 4; ++q) t += (double)sacc[(size_t)q * TC_NMAX * 3 + sl * 3 + v];
            part[(size_t)v * G + blockIdx.x] = s_abort ? 0.0 : t;
        }
        __threadfence();
        if (atomicAdd(&tickets[sl], 1u) == (unsigned)G - 1) {
            __threadfence();
            double tot[3];
            for (int v = 0; v < 3; ++v) {
                double t = 0;
                for (int g = 0; g < G; ++g) t += __ldcg(part + (size_t)v * G + g);
                tot[v] = t;
            }
            const int sy = s_act[sl];
            run_finish(fin, sy, state[sy], tot[0], tot[1], tot[2]);
            tickets[sl] = 0;
        }
    }
}

std::mutex g_tc_mu;
std::vector<int> g_tc_sms;       // per device
std::vector<char> g_tc_smem_set;

int device_sms(int dev) {
    std::lock_guard<std::mutex> lk(g_tc_mu);
    if ((int)g_tc_sms.size() <= dev) g_tc_sms.resize(dev + 1, 0), g_tc_smem_set.resize(dev + 1, 0);
    if (!g_tc_sms[dev]) cudaDeviceGetAttribute(&g_tc_sms[dev], cudaDevAttrMultiProcessorCount, dev);
    return g_tc_sms[dev];
}

size_t tc_smem_bytes(int np) { return sizeof(float) * (size_t)TC_NB * (TC_A_FLOATS + 2 * np * 2 * TC_KT) + 1024; }

}  // namespace

bool wproj_tc_ok(int n, int kk, int nsys, const void *W, const void *Y, size_t strideY) {
    return kk > 0 && kk <= TC_KMAX && nsys >= 8 && nsys <= TC_NMAX && n % 2 == 0 && strideY % 2 == 0 &&
           ((uintptr_t)W & 15) == 0 && ((uintptr_t)Y & 15) == 0;
}

int wproj_tc_grid(int n) {
    int dev = 0;
    cudaGetDevice(&dev);
    const long ntiles = ((long)n + TC_KT - 1) / TC_KT;
    const int sms = device_sms(dev);
    return (int)(ntiles < sms ? ntiles : sms);
}

int launch_wproj_tc(int n, int kk, const float2 *W, const float2 *Y, size_t strideY, const int *act, int nsys,
                    double *part, double2 *coef, size_t strideC, cudaStream_t st) {
    int dev = 0;
    cudaGetDevice(&dev);
    const int G = wproj_tc_grid(n);
    const int np = ((nsys + 15) / 16) * 16;
    const size_t smem = tc_smem_bytes(np);
    {
        std::lock_guard<std::mutex> lk(g_tc_mu);
        if (!g_tc_smem_set[dev]) {
            cudaFuncSetAttribute(k_wproj_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)tc_smem_bytes(TC_NMAX));
            g_tc_smem_set[dev] = 1;
        }
    }
    k_wproj_tc<<<G, TC_THREADS, smem, st>>>(n, kk, W, Y, strideY, act, nsys, np, part);
    const int O = kk * nsys;
    k_wproj_tc_reduce<<<(O + 31) / 32, 256, 0, st>>>(kk, nsys, G, part, act, coef, strideC);
    return 2;
}

size_t wapply_smem_bytes(int nsp) { return (size_t)4 * WA_AOP + (size_t)4 * nsp * 2 * TC_ROW + 1024; }

bool wapply_tc_ok(int n, int kk, int nsys) { return kk > 0 && kk <= TC_KMAX && nsys >= 8 && nsys <= TC_NMAX && n > 0; }

int launch_wapply_tc(int n, int kk, const float2 *W, double2 *coef, size_t strideC, const int *act, int nsys,
                     float2 *P, size_t strideP, int unit_idx, cudaStream_t st) {
    int dev = 0;
    cudaGetDevice(&dev);
    const long ntiles = ((long)n + WA_TILE - 1) / WA_TILE;
    const int sms = device_sms(dev);
    const int G = (int)(ntiles < sms ? ntiles : sms);
    const int nsp = ((nsys + 7) / 8) * 8;
    static std::vector<char> set;
    {
        std::lock_guard<std::mutex> lk(g_tc_mu);
        if ((int)set.size() <= dev) set.resize(dev + 1, 0);
        if (!set[dev]) {
            cudaFuncSetAttribute(k_wapply_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)wapply_smem_bytes(TC_NMAX));
            set[dev] = 1;
        }
    }
    k_wapply_tc<<<G, WA_THREADS, wapply_smem_bytes(nsp), st>>>(n, kk, W, coef, strideC, act, nsys, nsp, P, strideP,
                                                               unit_idx);
    return 1;
}

size_t wupdate_smem_bytes(int nsp) {
    return (size_t)4 * WA_AOP + (size_t)4 * nsp * 2 * TC_ROW + sizeof(float2) * TC_NMAX * WU_QB +
           sizeof(float) * 4 * TC_NMAX * 3 + 1024;
}

bool wupdate_tc_ok(int n, int kk, int qb, int nsys) {
    return n > 0 && kk > 0 && kk <= TC_KMAX && qb >= 0 && qb <= WU_QB && nsys >= 8 && nsys <= TC_NMAX;
}

int wupdate_tc_grid(int n) {
    int dev = 0;
    cudaGetDevice(&dev);
    const long ntiles = ((long)n + WA_TILE - 1) / WA_TILE;
    const int sms = device_sms(dev);
    return (int)(ntiles < sms ? ntiles : sms);
}

int launch_wupdate_tc(int n, int kk, const float2 *W, const float2 *V, size_t strideV, int qb, const float2 *w,
                      size_t strideW, float2 *out, size_t strideO, const int *act, int nsys, const double2 *coef,
                      size_t strideC, double *partials, unsigned *tickets, SysState *state, FinishArgs fin,
                      bool skip_broken, cudaStream_t st) {
    int dev = 0;
    cudaGetDevice(&dev);
    const int G = wupdate_tc_grid(n);
    const int nsp = ((nsys + 7) / 8) * 8;
    static std::vector<char> set;
    {
        std::lock_guard<std::mutex> lk(g_tc_mu);
        if ((int)set.size() <= dev) set.resize(dev + 1, 0);
        if (!set[dev]) {
            cudaFuncSetAttribute(k_wupdate_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)wupdate_smem_bytes(TC_NMAX));
            set[dev] = 1;
        }
    }
    k_wupdate_tc<<<G, WU_THREADS, wupdate_smem_bytes(nsp), st>>>(n, kk, W, V, strideV, qb, w, strideW, out, strideO,
                                                                  act, nsys, nsp, coef, strideC, partials, tickets,
                                                                  state, fin, skip_broken ? 1 : 0);
    return 1;
}

unsigned wproj_tc_timeouts() {
    unsigned v = 0;
    cudaMemcpyFromSymbol(&v, g_tc_timeouts, sizeof v);
    return v;
}

void enqueue_timeout_read_tc(unsigned *host, cudaStream_t st) {
    cudaMemcpyFromSymbolAsync(host, g_tc_timeouts, sizeof(unsigned), 0, cudaMemcpyDeviceToHost, st);
}

int push_wait_limit_tc(long long cycles) {
    return cudaMemcpyToSymbol(c_tc_wait_cycles, &cycles, sizeof cycles) == cudaSuccess ? 0 : -1;
}

}  // namespace gdmr
