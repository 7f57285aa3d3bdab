// qr_reduce.cu -- FP64 reductions over state vectors on sm_103a:
//   * <a, b> per state (qr_vdot, and <psi|H|psi> through qr_expect),
//   * per-string coefficient gradients R_m = sum_r (-1)^popc(r & z_m)
//     conj(psi[r ^ x_m]) g[r] (qr_term_grad).
// Partial sums are written per block into stream-ordered scratch and summed
// by a second kernel in a fixed order, so results are deterministic.
#include <cstdio>
#include <mutex>
#include <type_traits>

#include "../../include/qrusty_gpu.h"
#include "qr_common.cuh"

namespace qr {

constexpr int kRedThreads = 256;

__device__ __forceinline__ bool parity_of(uint32_t v) { return (__popc(v) & 1) != 0; }
__device__ __forceinline__ bool parity_of(uint64_t v) { return (__popcll(v) & 1) != 0; }

// Block-wide FP64 complex sum; result valid in thread 0.
__device__ __forceinline__ double2 block_sum(double re, double im, double2 *sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, o);
        im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = make_double2(re, im);
    __syncthreads();
    double2 r = make_double2(0.0, 0.0);
    if (threadIdx.x == 0) {
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
            r.x += sh[i].x;
            r.y += sh[i].y;
        }
    }
    __syncthreads();
    return r;
}

// partial[s * nblk + blk] = sum over this block's slice of conj(a) b.
// c64 inputs: FP32 products, FP64 accumulation.  c128: FP64 throughout.
template <bool F32>
__global__ void __launch_bounds__(kRedThreads) vdot_partial_kernel(uint64_t N, const void *a_,
                                                                   const void *b_, uint32_t nblk,
                                                                   double2 *partial) {
    __shared__ double2 sh[kRedThreads / 32];
    const uint32_t s = blockIdx.y;
    double re = 0.0, im = 0.0;
    const uint64_t stride = (uint64_t)nblk * blockDim.x;
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < N; r += stride) {
        if constexpr (F32) {
            const float2 a = static_cast<const float2 *>(a_)[s * N + r];
            const float2 b = static_cast<const float2 *>(b_)[s * N + r];
            re += (double)fmaf(a.x, b.x, a.y * b.y);
            im += (double)fmaf(a.x, b.y, -a.y * b.x);
        } else {
            const double2 a = static_cast<const double2 *>(a_)[s * N + r];
            const double2 b = static_cast<const double2 *>(b_)[s * N + r];
            re = fma(a.x, b.x, fma(a.y, b.y, re));
            im = fma(a.x, b.y, fma(-a.y, b.x, im));
        }
    }
    const double2 t = block_sum(re, im, sh);
    if (threadIdx.x == 0) partial[(size_t)s * nblk + blockIdx.x] = t;
}

// out[s] = sum_i partial[s * nblk + i] (fixed order: thread-strided, then
// the block sum).
__global__ void __launch_bounds__(kRedThreads) sum_partials_kernel(const double2 *partial,
                                                                   uint32_t nblk, double2 *out) {
    __shared__ double2 sh[kRedThreads / 32];
    const uint32_t s = blockIdx.x;
    double re = 0.0, im = 0.0;
    for (uint32_t i = threadIdx.x; i < nblk; i += blockDim.x) {
        re += partial[(size_t)s * nblk + i].x;
        im += partial[(size_t)s * nblk + i].y;
    }
    const double2 t = block_sum(re, im, sh);
    if (threadIdx.x == 0) out[s] = t;
}

uint32_t vdot_blocks(uint64_t N, int nsm) {
    uint64_t b = (N + (uint64_t)kRedThreads * 16 - 1) / ((uint64_t)kRedThreads * 16);
    const uint64_t cap = (uint64_t)nsm * 4;
    if (b > cap) b = cap;
    if (b == 0) b = 1;
    return (uint32_t)b;
}

cudaError_t launch_vdot(int dtype, uint64_t N, const void *a, const void *b, int nstates,
                        double2 *partial, uint32_t nblk, double2 *out, cudaStream_t st) {
    const dim3 grid(nblk, (unsigned)nstates);
    if (dtype == 1)
        vdot_partial_kernel<true><<<grid, kRedThreads, 0, st>>>(N, a, b, nblk, partial);
    else
        vdot_partial_kernel<false><<<grid, kRedThreads, 0, st>>>(N, a, b, nblk, partial);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    sum_partials_kernel<<<(unsigned)nstates, kRedThreads, 0, st>>>(partial, nblk, out);
    count_launch();
    return cudaGetLastError();
}

// ---------------------------------------------------------------- term grads
// One block per (string m, chunk c): sum over the chunk's rows r of
// (-1)^popc(r & z_m) conj(psi[r ^ x_m]) g[r], over all states.  c64 inputs:
// FP32 products and per-thread FP32 sums over <= kGradPerThread rows, then
// FP64 across threads and chunks.  partial[m * nchunk + c].
constexpr int kGradPerThread = 32;

constexpr int kGradK = 4;  // strings per block: they share each g load

template <bool F32> struct GradT;
template <> struct GradT<true> {
    using V = float2;
    using A = float;
};
template <> struct GradT<false> {
    using V = double2;
    using A = double;
};

// Accumulate (-1)^popc(r & z) conj(p) g into (ar, ai).
template <typename A, typename V>
__device__ __forceinline__ void grad_acc(A &ar, A &ai, V p, V gg, bool neg) {
    A pr = p.x * gg.x + p.y * gg.y;
    A pi = p.x * gg.y - p.y * gg.x;
    ar += neg ? -pr : pr;
    ai += neg ? -pi : pi;
}

// partial[m * gridDim.x + blockIdx.x] = the chunk's sum over rows r and states
// of (-1)^popc(r & z_m) conj(psi[r ^ x_m]) g[r], for the kGradK strings of
// this block (g read once for all of them).  complex64: FP32 products and
// per-thread FP32 sums over at most kGradPerThread rows, then FP64.
template <bool F32, bool WIDE>
__global__ void __launch_bounds__(kRedThreads) term_grad_partial_kernel(
    uint64_t N, int nstates, const uint64_t *sx, const uint64_t *sz, uint32_t nstr,
    const void *psi_, const void *g_, uint64_t chunk, uint32_t nchunk, double2 *partial) {
    using W = typename std::conditional<WIDE, uint64_t, uint32_t>::type;
    using V = typename GradT<F32>::V;
    using A = typename GradT<F32>::A;
    __shared__ double2 sh[kRedThreads / 32];
    const uint32_t nbatch = (nstr + kGradK - 1) / kGradK;
    for (uint32_t bm = blockIdx.y; bm < nbatch; bm += gridDim.y) {
        const uint32_t m0 = bm * kGradK;
        const uint32_t kv = nstr - m0 < (uint32_t)kGradK ? nstr - m0 : (uint32_t)kGradK;
        W x[kGradK], z[kGradK];
#pragma unroll
        for (int k = 0; k < kGradK; ++k) {
            x[k] = (uint32_t)k < kv ? (W)sx[m0 + k] : (W)0;
            z[k] = (uint32_t)k < kv ? (W)sz[m0 + k] : (W)0;
        }
        double re[kGradK], im[kGradK];
#pragma unroll
        for (int k = 0; k < kGradK; ++k) re[k] = im[k] = 0.0;
        for (uint32_t c = blockIdx.x; c < nchunk; c += gridDim.x) {
            const uint64_t r0 = (uint64_t)c * chunk, r1 = (r0 + chunk < N) ? r0 + chunk : N;
            for (int s = 0; s < nstates; ++s) {
                const V *psi = static_cast<const V *>(psi_) + (size_t)s * N;
                const V *g = static_cast<const V *>(g_) + (size_t)s * N;
                A fr[kGradK], fi[kGradK];
#pragma unroll
                for (int k = 0; k < kGradK; ++k) fr[k] = fi[k] = A(0);
                int cnt = 0;
                W r = (W)(r0 + threadIdx.x);
                // two rows per step (independent loads in flight)
                for (; (uint64_t)r + kRedThreads < r1; r += 2 * kRedThreads) {
                    const W r2 = r + kRedThreads;
                    const V g1 = g[r], g2 = g[r2];
#pragma unroll
                    for (int k = 0; k < kGradK; ++k) {
                        if ((uint32_t)k < kv) {
                            const V p1 = psi[r ^ x[k]], p2 = psi[r2 ^ x[k]];
                            grad_acc<A, V>(fr[k], fi[k], p1, g1, parity_of(r & z[k]));
                            grad_acc<A, V>(fr[k], fi[k], p2, g2, parity_of(r2 & z[k]));
                        }
                    }
                    if (F32 && ++cnt == kGradPerThread / 2) {  // 2 rows per step
#pragma unroll
                        for (int k = 0; k < kGradK; ++k) {
                            re[k] += (double)fr[k];
                            im[k] += (double)fi[k];
                            fr[k] = fi[k] = A(0);
                        }
                        cnt = 0;
                    }
                }
                if ((uint64_t)r < r1) {
                    const V g1 = g[r];
#pragma unroll
                    for (int k = 0; k < kGradK; ++k)
                        if ((uint32_t)k < kv)
                            grad_acc<A, V>(fr[k], fi[k], psi[r ^ x[k]], g1, parity_of(r & z[k]));
                }
#pragma unroll
                for (int k = 0; k < kGradK; ++k) {
                    re[k] += (double)fr[k];
                    im[k] += (double)fi[k];
                }
            }
        }
#pragma unroll
        for (int k = 0; k < kGradK; ++k) {
            const double2 t = block_sum(re[k], im[k], sh);
            if (threadIdx.x == 0 && (uint32_t)k < kv)
                partial[(size_t)(m0 + k) * gridDim.x + blockIdx.x] = t;
        }
    }
}

__global__ void __launch_bounds__(kRedThreads) term_grad_scatter_kernel(uint64_t T,
                                                                        const uint32_t *map,
                                                                        const uint8_t *phase,
                                                                        const double2 *R,
                                                                        double2 *out) {
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < T;
         k += (uint64_t)gridDim.x * blockDim.x) {
        const double2 v = R[map[k]];
        double2 o;
        switch (phase[k] & 3) {
            case 0: o = v; break;                                   // conj(1) = 1
            case 1: o = make_double2(-v.y, v.x); break;             // conj(-i) = i
            case 2: o = make_double2(-v.x, -v.y); break;            // -1
            default: o = make_double2(v.y, -v.x); break;            // conj(i) = -i
        }
        out[k] = o;
    }
}

// ---------------------------------------------------------------- term grads, tiled (complex64)
// The merged strings are sorted by partner tile h = x >> 12 and cut into
// batches of <= kTgB strings with one h.  A work item is (batch, chunk of
// output tiles); per output tile (4,096 rows of one state) the CTA stages
// the tile of g and the batch's partner tile of psi (tile ^ h) in shared
// memory (cp.async, kTgStages stages), and thread i takes rows i + 512 j
// (j < 8).  For string (x, z), row r = tile * 4096 + i + 512 j:
//   psi[r ^ x] = partner row (i ^ (x & 511)) + 512 (j ^ l),  l = (x >> 9) & 7,
//   (-1)^popc(r & z) = (-1)^popc(tile & (z >> 12)) (-1)^popc(i & z & 511)
//                      (-1)^popc(j & w),                     w = (z >> 9) & 7,
// so l is a compile-time case (shared-memory loads at immediate offsets) and
// the register-bit signs are one three-level butterfly.  Packed FP32:
// A = sum s gx p, B = sum s gy p with p = (px, py) give conj(p) g summed as
// (A.x + B.y, B.x - A.y).  Every kTgFlush tiles a warp transpose-reduce sums
// the 8 strings' FP32 values over the warp's lanes (16 shuffles for 16
// values) and lane 2m adds value m to its FP64 sum; at the item's end the 16
// warps' sums are added in warp order.  Deterministic: fixed order
// everywhere, one partial per (string, chunk).
constexpr int kTgThreads = 512;
constexpr int kTgStages = 3;
constexpr int kTgB = 8;        // strings per batch
constexpr int kTgFlush = 4;    // tiles per FP32 window (32 rows per thread)
constexpr uint32_t kTgTileBytes = 4096 * 8;
constexpr uint32_t kTgStageBytes = 2 * kTgTileBytes;
constexpr uint32_t kTgAlign = 32768;
constexpr size_t kTgSmem = (size_t)kTgStages * kTgStageBytes + kTgAlign;

__device__ __forceinline__ uint32_t tg_saddr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void tg_cp16(uint32_t dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void tg_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int K>
__device__ __forceinline__ void tg_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(K) : "memory");
}
constexpr int tg_par3(int v) { return (v ^ (v >> 1) ^ (v >> 2)) & 1; }

__device__ __forceinline__ float2 tg_lds(uint32_t a) {
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a));
    return v;
}

// Row J of g into the plus or minus chain of a string whose register-bit z
// pattern is W: plus rows (even popc(J & W)) start at J = 0, minus rows at
// the lowest set bit of W.  q = shared address of the string's partner row
// for J = 0 with the partner tile 32 KB-aligned, so row J is at q ^ (J << 12).
template <int J, int W>
__device__ __forceinline__ void tg_row(uint32_t q, const float2 (&GX)[8], const float2 (&GY)[8],
                                       float2 &aP, float2 &bP, float2 &aM, float2 &bM) {
    const float2 p = tg_lds(q ^ (uint32_t)(J << 12));
    if constexpr (tg_par3(J & W) == 0) {
        if constexpr (J == 0) {
            aP = __fmul2_rn(GX[J], p);
            bP = __fmul2_rn(GY[J], p);
        } else {
            aP = __ffma2_rn(GX[J], p, aP);
            bP = __ffma2_rn(GY[J], p, bP);
        }
    } else {
        if constexpr (J == (W & -W)) {
            aM = __fmul2_rn(GX[J], p);
            bM = __fmul2_rn(GY[J], p);
        } else {
            aM = __ffma2_rn(GX[J], p, aM);
            bM = __ffma2_rn(GY[J], p, bM);
        }
    }
}

// One string on one staged tile; sg = (tile sign, tile sign, -tile sign,
// -tile sign).  The thread's own sign (-1)^popc(i & z & 511) is applied at
// the flush.
template <int W>
__device__ __forceinline__ void tg_string(uint32_t q, const float2 (&GX)[8],
                                          const float2 (&GY)[8], float4 sg, float2 &accA,
                                          float2 &accB) {
    float2 aP, bP, aM, bM;
    tg_row<0, W>(q, GX, GY, aP, bP, aM, bM);
    tg_row<1, W>(q, GX, GY, aP, bP, aM, bM);
    tg_row<2, W>(q, GX, GY, aP, bP, aM, bM);
    tg_row<3, W>(q, GX, GY, aP, bP, aM, bM);
    tg_row<4, W>(q, GX, GY, aP, bP, aM, bM);
    tg_row<5, W>(q, GX, GY, aP, bP, aM, bM);
    tg_row<6, W>(q, GX, GY, aP, bP, aM, bM);
    tg_row<7, W>(q, GX, GY, aP, bP, aM, bM);
    const float2 ST = make_float2(sg.x, sg.y);
    accA = __ffma2_rn(ST, aP, accA);
    accB = __ffma2_rn(ST, bP, accB);
    if constexpr (W != 0) {
        const float2 NST = make_float2(sg.z, sg.w);
        accA = __ffma2_rn(NST, aM, accA);
        accB = __ffma2_rn(NST, bM, accB);
    }
}

// Sum of v[m] over the warp's 32 lanes for m < 16, by recursive halving:
// returns the sum of value (lane >> 1) & 15.
__device__ __forceinline__ float tg_transpose_reduce(float (&v)[16]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int h = 8, o = 16; h >= 1; h >>= 1, o >>= 1) {
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int q = 0; q < h; ++q) {
            const float send = up ? v[q] : v[q + h];
            const float keep = up ? v[q + h] : v[q];
            v[q] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
    }
    return v[0] + __shfl_xor_sync(0xffffffffu, v[0], 1);
}

__global__ void __launch_bounds__(kTgThreads, 1) term_grad_tiles_kernel(
    uint64_t ntiles, int tbits, int nstates, const uint64_t *sx, const uint64_t *sz,
    const uint32_t *perm, const uint2 *batches, uint32_t nbatch, const float2 *psi,
    const float2 *g, uint32_t nchunk, uint64_t chunk_tiles, double *partial,
    unsigned long long *next_item) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ uint64_t s_x[kTgB], s_z[kTgB];
    __shared__ float4 s_sign[2][kTgB];  // per tile parity: (s, s, -s, -s), two tiles in flight
    __shared__ double s_red[kTgThreads / 32][16];
    __shared__ unsigned long long s_item;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // stages from the first 32 KB boundary of the dynamic window (kTgAlign
    // bytes of slack), so that a partner row's address has the row's
    // register bits at bits 12-14 alone
    const uint32_t raw = tg_saddr(smem_raw);
    const uint32_t sbase = (raw + kTgAlign - 1) & ~(kTgAlign - 1);
    unsigned char *const smem = smem_raw + (sbase - raw);
    const uint64_t TT = ntiles * (uint64_t)nstates;
    const uint64_t nitems = (uint64_t)nbatch * nchunk;
    // items = (batch, chunk), batch-major with the batches largest first:
    // taken from a counter, so the CTAs stay balanced whatever the batch sizes
    // (each item's sums are formed in a fixed order, whichever CTA runs it)
    for (;;) {
        if (tid == 0) s_item = atomicAdd(next_item, 1ull);
        __syncthreads();
        const uint64_t item = s_item;
        if (item >= nitems) break;
        const uint32_t bi = (uint32_t)(item / nchunk), c = (uint32_t)(item % nchunk);
        const uint2 bt = batches[bi];
        const uint32_t kv = bt.y;
        const uint64_t t0 = (uint64_t)c * chunk_tiles;
        const uint64_t t1 = t0 + chunk_tiles < TT ? t0 + chunk_tiles : TT;
        if (tid < kTgB) {
            s_x[tid] = (uint32_t)tid < kv ? sx[bt.x + tid] : 0ull;
            s_z[tid] = (uint32_t)tid < kv ? sz[bt.x + tid] : 0ull;
        }
        __syncthreads();
        const uint64_t hpart = s_x[0] >> 12;  // one partner tile for the batch
        // per string: offset of its partner row for j = 0 within the 32 KB
        // partner tile, (i ^ (x & 511)) * 8 | ((x >> 9) & 7) << 12 (bits
        // 0-14), and w = (z >> 9) & 7 (bits 15-17); per thread the parities
        // of i & z & 511
        uint32_t info[kTgB], tpar = 0;
#pragma unroll
        for (int k = 0; k < kTgB; ++k) {
            const uint32_t x = (uint32_t)s_x[k], z = (uint32_t)s_z[k];
            info[k] = ((((uint32_t)tid ^ x) & 511u) << 3) | (((x >> 9) & 7u) << 12) |
                      (((z >> 9) & 7u) << 15);
            tpar |= (__popc((uint32_t)tid & z & 511u) & 1u) << k;
        }
        auto issue = [&](uint64_t gt, int stage) {
            const uint64_t st = gt >> tbits, t = gt & (ntiles - 1);
            const unsigned char *gsrc = reinterpret_cast<const unsigned char *>(g + (gt << 12));
            const unsigned char *psrc =
                reinterpret_cast<const unsigned char *>(psi + (((st << tbits) | (t ^ hpart)) << 12));
            const uint32_t dst = tg_saddr(smem + (size_t)stage * kTgStageBytes);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint32_t off = (uint32_t)(q * kTgThreads + tid) * 16u;
                tg_cp16(dst + off, psrc + off);
                tg_cp16(dst + kTgTileBytes + off, gsrc + off);
            }
        };
#pragma unroll
        for (int q = 0; q < kTgStages - 1; ++q) {
            if (t0 + q < t1) issue(t0 + q, q);
            tg_commit();
        }
        float2 accA[kTgB], accB[kTgB];
#pragma unroll
        for (int k = 0; k < kTgB; ++k) accA[k] = accB[k] = make_float2(0.f, 0.f);
        double acc64 = 0.0;
        int win = 0, stage = 0;
        for (uint64_t gt = t0; gt < t1; ++gt) {
            if (tid < kTgB) {
                // (-1)^popc(tile & (z >> 12)) of string tid for this tile; the
                // entry written two tiles ago was last read before the
                // previous barrier
                const float sgn =
                    (__popcll((gt & (ntiles - 1)) & (s_z[tid] >> 12)) & 1) ? -1.f : 1.f;
                s_sign[gt & 1][tid] = make_float4(sgn, sgn, -sgn, -sgn);
            }
            tg_wait<kTgStages - 2>();
            __syncthreads();  // tile gt staged by every thread; the oldest stage is free
            {
                const uint64_t nx = gt + kTgStages - 1;
                if (nx < t1) issue(nx, (stage + kTgStages - 1) % kTgStages);
                tg_commit();
            }
            const unsigned char *sb = smem + (size_t)stage * kTgStageBytes;
            float2 GX[8], GY[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const float2 gv =
                    *reinterpret_cast<const float2 *>(sb + kTgTileBytes + (tid + 512 * j) * 8);
                GX[j] = make_float2(gv.x, gv.x);
                GY[j] = make_float2(gv.y, gv.y);
            }
            const uint32_t qs = tg_saddr(sb);  // 32 KB-aligned partner tile
#pragma unroll
            for (int k = 0; k < kTgB; ++k) {
                if ((uint32_t)k < kv) {
                    const uint32_t inf = info[k];
                    const float4 sg = s_sign[gt & 1][k];
                    const uint32_t q = qs | (inf & 0x7fffu);
                    switch ((inf >> 15) & 7u) {
                        case 0: tg_string<0>(q, GX, GY, sg, accA[k], accB[k]); break;
                        case 1: tg_string<1>(q, GX, GY, sg, accA[k], accB[k]); break;
                        case 2: tg_string<2>(q, GX, GY, sg, accA[k], accB[k]); break;
                        case 3: tg_string<3>(q, GX, GY, sg, accA[k], accB[k]); break;
                        case 4: tg_string<4>(q, GX, GY, sg, accA[k], accB[k]); break;
                        case 5: tg_string<5>(q, GX, GY, sg, accA[k], accB[k]); break;
                        case 6: tg_string<6>(q, GX, GY, sg, accA[k], accB[k]); break;
                        default: tg_string<7>(q, GX, GY, sg, accA[k], accB[k]); break;
                    }
                }
            }
            stage = (stage + 1) % kTgStages;
            if (++win == kTgFlush || gt + 1 == t1) {
                float v[16];
#pragma unroll
                for (int k = 0; k < kTgB; ++k) {
                    const float re = accA[k].x + accB[k].y, im = accB[k].x - accA[k].y;
                    const bool neg = (tpar >> k) & 1u;
                    v[2 * k] = neg ? -re : re;
                    v[2 * k + 1] = neg ? -im : im;
                    accA[k] = accB[k] = make_float2(0.f, 0.f);
                }
                acc64 += (double)tg_transpose_reduce(v);
                win = 0;
            }
        }
        tg_wait<0>();
        if (!(lane & 1)) s_red[warp][lane >> 1] = acc64;
        __syncthreads();
        if (tid < 16) {
            double v = 0.0;
            for (int w = 0; w < kTgThreads / 32; ++w) v += s_red[w][tid];
            const uint32_t k = (uint32_t)tid >> 1;
            if (k < kv) partial[2 * ((uint64_t)perm[bt.x + k] * nchunk + c) + (tid & 1)] = v;
        }
        __syncthreads();  // s_x, s_z, s_red and the stages are reused by the next item
    }
}

cudaError_t launch_term_grad_tiles(uint64_t N, int nstates, const uint64_t *sx, const uint64_t *sz,
                                   const uint32_t *perm, const uint2 *batches, uint32_t nbatch,
                                   uint32_t nstr, const void *psi, const void *g,
                                   double2 *partial, uint32_t nchunk, double2 *R, uint64_t T,
                                   const uint32_t *map, const uint8_t *phase, double2 *out,
                                   unsigned long long *counter, int nsm, cudaStream_t st) {
    const uint64_t ntiles = N >> 12;
    int tbits = 0;
    while ((1ull << tbits) < ntiles) ++tbits;
    const uint64_t TT = ntiles * (uint64_t)nstates;
    const uint64_t chunk = (TT + nchunk - 1) / nchunk;
    cudaError_t e = ensure_dyn_smem(reinterpret_cast<const void *>(term_grad_tiles_kernel), kTgSmem);
    if (e != cudaSuccess) return e;
    const uint64_t nitems = (uint64_t)nbatch * nchunk;
    const unsigned grid = (unsigned)(nitems < (uint64_t)nsm ? nitems : (uint64_t)nsm);
    e = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    term_grad_tiles_kernel<<<grid, kTgThreads, kTgSmem, st>>>(
        ntiles, tbits, nstates, sx, sz, perm, batches, nbatch, static_cast<const float2 *>(psi),
        static_cast<const float2 *>(g), nchunk, chunk, reinterpret_cast<double *>(partial),
        counter);
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    sum_partials_kernel<<<nstr, kRedThreads, 0, st>>>(partial, nchunk, R);
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    uint64_t gb = (T + kRedThreads - 1) / kRedThreads;
    if (gb > 4096) gb = 4096;
    term_grad_scatter_kernel<<<(unsigned)gb, kRedThreads, 0, st>>>(T, map, phase, R, out);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_term_grad(int dtype, uint64_t N, int nstates, const uint64_t *sx,
                             const uint64_t *sz, uint32_t nstr, const void *psi, const void *g,
                             double2 *partial, uint32_t nchunk, uint64_t chunk, double2 *R,
                             uint64_t T, const uint32_t *map, const uint8_t *phase, double2 *out,
                             cudaStream_t st) {
    const uint32_t nbatch = (nstr + kGradK - 1) / kGradK;
    const unsigned gy = nbatch < 65535u ? nbatch : 65535u;
    const dim3 grid(nchunk, gy);
    const bool wide = N >= (1ull << 32);  // 32-bit rows need r + 2 * 256 < 2^32
    if (dtype == 1) {
        if (wide)
            term_grad_partial_kernel<true, true><<<grid, kRedThreads, 0, st>>>(
                N, nstates, sx, sz, nstr, psi, g, chunk, nchunk, partial);
        else
            term_grad_partial_kernel<true, false><<<grid, kRedThreads, 0, st>>>(
                N, nstates, sx, sz, nstr, psi, g, chunk, nchunk, partial);
    } else {
        if (wide)
            term_grad_partial_kernel<false, true><<<grid, kRedThreads, 0, st>>>(
                N, nstates, sx, sz, nstr, psi, g, chunk, nchunk, partial);
        else
            term_grad_partial_kernel<false, false><<<grid, kRedThreads, 0, st>>>(
                N, nstates, sx, sz, nstr, psi, g, chunk, nchunk, partial);
    }
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    sum_partials_kernel<<<nstr, kRedThreads, 0, st>>>(partial, nchunk, R);
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    uint64_t gb = (T + kRedThreads - 1) / kRedThreads;
    if (gb > 4096) gb = 4096;
    term_grad_scatter_kernel<<<(unsigned)gb, kRedThreads, 0, st>>>(T, map, phase, R, out);
    count_launch();
    return cudaGetLastError();
}

}  // namespace qr

namespace qr {

// ---------------------------------------------------------------- no-alloc vdot
// Fixed scratch of the allocation-free inner product: one FP64 complex
// partial sum per (state, block).  A file-scope __device__ array, so every
// GPU that loads this library holds these 256 KiB until the process exits.
constexpr uint32_t kNoAllocPartials = QR_VDOT_NOALLOC_MAX_PARTIALS;
static __device__ __align__(256) double2 g_vdot_scratch[kNoAllocPartials];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
double2 *g_scratch_ptr[kMaxDevices] = {};
int g_scratch_nsm[kMaxDevices] = {};

// Device address of g_vdot_scratch on the current device.  In host code the
// array's name is only a host-side stand-in, so the address is looked up
// once per device with cudaGetSymbolAddress (device current) and cached.
int noalloc_scratch(double2 **out, int *nsm) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(QR_ECUDA, "qr_vdot_noalloc: cudaGetDevice failed");
    if (dev < 0 || dev >= kMaxDevices)
        return set_error(QR_ESTATE, "qr_vdot_noalloc: device index out of range");
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_vdot_scratch);
        if (e != cudaSuccess || p == nullptr) {
            char buf[256];
            snprintf(buf, sizeof(buf), "qr_vdot_noalloc: cudaGetSymbolAddress failed: %s",
                     cudaGetErrorString(e));
            return set_error(QR_ECUDA, buf);
        }
        int n = 0;
        e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return set_error(QR_ECUDA, "qr_vdot_noalloc: device attribute");
        g_scratch_ptr[dev] = static_cast<double2 *>(p);
        g_scratch_nsm[dev] = n;
    }
    *out = g_scratch_ptr[dev];
    *nsm = g_scratch_nsm[dev];
    return QR_OK;
}
}  // namespace

}  // namespace qr

extern "C" int qr_vdot_noalloc(int32_t n, int32_t dtype, const void *a, const void *b,
                               int32_t nstates, double *out, void *stream) {
    using namespace qr;
    if (!a || !b || !out) return set_error(QR_EINVAL, "qr_vdot_noalloc: null argument");
    if (n < 1 || n > 40) return set_error(QR_EINVAL, "qr_vdot_noalloc: n outside [1, 40]");
    if (dtype != QR_C128 && dtype != QR_C64C)
        return set_error(QR_EINVAL, "qr_vdot_noalloc: dtype must be QR_C128 or QR_C64C");
    if (nstates < 1) return set_error(QR_EINVAL, "qr_vdot_noalloc: nstates < 1");
    if ((uint32_t)nstates > kNoAllocPartials)
        return set_error(QR_EINVAL,
                         "qr_vdot_noalloc: nstates exceeds QR_VDOT_NOALLOC_MAX_PARTIALS (16384); "
                         "use qr_vdot");
    double2 *scratch = nullptr;
    int nsm = 0;
    int rc = noalloc_scratch(&scratch, &nsm);
    if (rc) return rc;
    const uint64_t N = 1ull << n;
    uint32_t nblk = vdot_blocks(N, nsm);
    const uint32_t cap = kNoAllocPartials / (uint32_t)nstates;  // >= 1 by the check above
    if (nblk > cap) nblk = cap;
    // Every (state, block) slot used below is written by the partial-sum
    // kernel before the second kernel reads it, so nothing is cleared.
    cudaError_t e = launch_vdot(dtype, N, a, b, nstates, scratch, nblk,
                                reinterpret_cast<double2 *>(out),
                                static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return set_error(QR_ECUDA, "qr_vdot_noalloc: kernel launch failed");
    return QR_OK;
}
