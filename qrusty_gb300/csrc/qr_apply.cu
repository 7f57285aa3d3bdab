// qr_apply.cu -- matrix-free Pauli-sum product y = H psi on sm_103a.
//
// Replaces "build the CSR, then spmat_dot_densevec" of qrusty
// (qrusty/src/accel.rs:171-210 row semantics, :338-370 SpMV): row r of H has
// one entry per distinct x mask g, at column r ^ x_g, with value
// D_g(r) = sum_{k in g} c'_k (-1)^popc(r & z_k).  So
//     y[r] = sum_g D_g(r) * psi[r ^ x_g].
//
// Layout and schedule.  The state is cut into tiles of 2^b contiguous
// amplitudes.  Output tile q needs, for every group g, the partner tile
// q ^ (x_g >> b), permuted inside by XOR with lo_g = x_g & (2^b - 1).  Groups
// are bucketed by partner tile ("blocks"); a persistent CTA walks its output
// tiles and, per tile, every block: the partner tile is staged into shared
// memory by a 1-D TMA bulk copy (cp.async.bulk + mbarrier, STAGES-deep ring)
// and all groups of the block are applied from shared memory.  Thread t of
// the CTA owns amplitudes r_lo = t + threads * m, m < AMPS, so a warp's XOR
// partners stay inside one aligned 32-element run (conflict-free LDS).
//
// Diagonal factor per group: D_g(r) = (-1)^popc(r & z0) * T_g[pi(r)], with
// pi(r) the parities of r against a GF(2) basis of the group's z
// differences (rank d <= kDMax, table of 2^d entries precomputed in FP64 on
// the host).  The parities split into a per-thread constant and a per-m part
// read from a 32-entry Walsh table, so the common case costs one sign select
// per amplitude.  The x = 0 group with a large z span is a precomputed
// diagonal vector (FP64 Walsh-Hadamard transform per tile, diag_wht below).
//
// Precision.  QR_C128: double2 amplitudes, FP64 arithmetic.  QR_C64C: float2
// amplitudes, FP32 products, each block's contributions summed in FP32 and
// folded into the row's running sum with a two-sum (error-free transform):
// the running value is an unevaluated (hi + lo) pair per component.
#include "qr_common.cuh"

namespace qr {

// Walsh words: bit m of walsh_word(v) is popc(m & v) & 1, for m, v < 32.
constexpr uint32_t walsh_word(uint32_t v) {
    uint32_t w = 0;
    for (uint32_t m = 0; m < 32; ++m) {
        uint32_t x = m & v, p = 0;
        while (x) { p ^= x & 1u; x >>= 1; }
        if (p) w |= 1u << m;
    }
    return w;
}
__constant__ uint32_t c_walsh[32] = {
    walsh_word(0),  walsh_word(1),  walsh_word(2),  walsh_word(3),  walsh_word(4),
    walsh_word(5),  walsh_word(6),  walsh_word(7),  walsh_word(8),  walsh_word(9),
    walsh_word(10), walsh_word(11), walsh_word(12), walsh_word(13), walsh_word(14),
    walsh_word(15), walsh_word(16), walsh_word(17), walsh_word(18), walsh_word(19),
    walsh_word(20), walsh_word(21), walsh_word(22), walsh_word(23), walsh_word(24),
    walsh_word(25), walsh_word(26), walsh_word(27), walsh_word(28), walsh_word(29),
    walsh_word(30), walsh_word(31)};

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t saddr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(saddr(dst)),
        "l"(src), "r"(bytes), "r"(saddr(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(saddr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ uint64_t gtimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}
// Bounded wait: gives up after ~limit_ns and reports false.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity,
                                                  uint64_t limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = gtimer_ns();
    while (!mbar_try_wait(bar, parity)) {
        if (gtimer_ns() - t0 > limit_ns) return false;
    }
    return true;
}

constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s per stage
constexpr int kMaxStages = 4;

// ---------------------------------------------------------------- arithmetic
template <typename Real>
__device__ __forceinline__ void cmac(Cplx<Real> &acc, const Cplx<Real> &d, const Cplx<Real> &p) {
    acc.re = fma(d.re, p.re, fma(-d.im, p.im, acc.re));
    acc.im = fma(d.re, p.im, fma(d.im, p.re, acc.im));
}
__device__ __forceinline__ void two_sum_into(float &hi, float &lo, float b) {
    const float s = __fadd_rn(hi, b);
    const float bb = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    hi = s;
    lo = __fadd_rn(lo, e);
}
// The same error-free transformation on (re, im) at once with packed FP32
// operations; x - y is formed as fma(y, -1, x) (y * -1 is exact, so the one
// rounding is that of x - y): bit-identical to two_sum_into per component.
__device__ __forceinline__ float2 sub2_rn(float2 x, float2 y) {
    return __ffma2_rn(y, make_float2(-1.f, -1.f), x);
}
__device__ __forceinline__ void two_sum_into2(float2 &hi, float2 &lo, float2 b) {
    const float2 s = __fadd2_rn(hi, b);
    const float2 bb = sub2_rn(s, hi);
    const float2 e = __fadd2_rn(sub2_rn(hi, sub2_rn(s, bb)), sub2_rn(b, bb));
    hi = s;
    lo = __fadd2_rn(lo, e);
}
// hi += b with the same error-free transformation; returns the error term
// instead of accumulating it
__device__ __forceinline__ float2 two_sum_carry2(float2 &hi, float2 b) {
    const float2 s = __fadd2_rn(hi, b);
    const float2 bb = sub2_rn(s, hi);
    const float2 e = __fadd2_rn(sub2_rn(hi, sub2_rn(s, bb)), sub2_rn(b, bb));
    hi = s;
    return e;
}
template <typename Real>
__device__ __forceinline__ Cplx<Real> cneg_if(const Cplx<Real> &d, uint32_t s) {
    Cplx<Real> r;
    r.re = s ? -d.re : d.re;
    r.im = s ? -d.im : d.im;
    return r;
}

// ---------------------------------------------------------------- c128 kernel
// Plain complex128: AMPS amplitudes per thread, one (amplitude, group) = 4
// DFMA.  Warps run decoupled, as in the compensated-c64 kernels: each waits on
// the stage's full mbarrier, applies the block's groups, and counts itself
// out on a per-stage counter; the last warp out refills the stage with the
// partner tile a ring length ahead.  No CTA-wide barrier sits between
// partner blocks, so the FP64 pipe does not drain at every block.
template <int AMPS>
__global__ void __launch_bounds__(512, 1) apply_c128(const ApplyArgs a, int stages) {
    using C = Cplx<double>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const uint32_t threads = blockDim.x;
    const uint32_t nwarps = threads >> 5;
    const uint32_t t = threadIdx.x;
    const uint32_t lane = t & 31;
    const uint32_t tile = 1u << a.b;
    const uint32_t tile_bytes = tile * (uint32_t)sizeof(C);
    C *bufs = reinterpret_cast<C *>(smem_raw);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem_raw + (size_t)stages * tile_bytes);
    uint32_t *cnt = reinterpret_cast<uint32_t *>(full + kMaxStages);
    volatile uint32_t *s_abort = cnt + kMaxStages;
    uint32_t *s_iss = cnt + kMaxStages + 1;  // copies issued per stage (drain)

    const C *psi = static_cast<const C *>(a.psi);
    C *y = static_cast<C *>(a.y);
    const C *tables = static_cast<const C *>(a.tables);
    const C *fat_c = static_cast<const C *>(a.fat_c);
    const C *diag = static_cast<const C *>(a.diag);
    const uint32_t nb = a.nblocks;

    const uint64_t first = blockIdx.x;
    const uint64_t my_items =
        a.nitems > first ? (a.nitems - first + gridDim.x - 1) / gridDim.x : 0;
    const uint64_t total = my_items * nb;
    if (total == 0) return;

    auto issue = [&](uint64_t L) {
        const uint64_t k = L / nb;
        const uint32_t j = (uint32_t)(L - k * nb);
        const uint64_t item = first + k * gridDim.x;
        const uint64_t st = item / a.ntiles;
        const uint64_t q = item - st * a.ntiles;
        const C *src = psi + st * a.N + ((q ^ a.blk_hi[j]) << a.b);
        const int s = (int)(L % (uint64_t)stages);
        if (blockIdx.x == 0 && (int64_t)L == a.withhold) return;  // test hook: never issued
        ++s_iss[s];
        mbar_expect_tx(&full[s], tile_bytes);
        bulk_g2s(bufs + (size_t)s * tile, src, tile_bytes, &full[s]);
    };
    if (t == 0) {
        for (int s = 0; s < stages; ++s) {
            mbar_init(&full[s], 1);
            cnt[s] = 0;
            s_iss[s] = 0;
        }
        *s_abort = 0;
        mbar_fence_init();
        const uint64_t pro = total < (uint64_t)stages ? total : (uint64_t)stages;
        for (uint64_t L = 0; L < pro; ++L) issue(L);
    }
    __syncthreads();

    C acc[AMPS];
    const uint32_t amask = AMPS - 1;
    uint32_t j = 0, s = 0, par = 0;
    uint64_t st = first / a.ntiles;
    uint64_t q = first - st * a.ntiles;

    for (uint64_t L = 0; L < total; ++L) {
        const uint64_t rbase = (q << a.b) | t;
        if (j == 0) {
#pragma unroll
            for (int m = 0; m < AMPS; ++m) acc[m].re = acc[m].im = 0.0;
        }
        // an expired wait sets the abort flag; from then on every warp skips
        // waits and work
        bool skip = *s_abort != 0;
        if (!skip && !mbar_wait_bounded(&full[s], par, a.wait_ns)) {
            if (lane == 0) {
                atomicExch(a.err, kErrMbarTimeout);
                *s_abort = 1;
            }
            skip = true;
        }
        skip = __any_sync(0xffffffffu, skip);
        const C *buf = bufs + (size_t)s * tile;

        if (!skip && (int)j == a.diag_block && diag != nullptr) {
            const C *dg = diag + (q << a.b);
#pragma unroll
            for (int m = 0; m < AMPS; ++m) {
                const uint32_t rl = t + threads * (uint32_t)m;
                cmac(acc[m], dg[rl], buf[rl]);
            }
        }

        const uint32_t g1 = skip ? 0u : a.blk_g0[j + 1];
        for (uint32_t g = a.blk_g0[j]; g < g1; ++g) {
            const GroupDesc gd = a.groups[g];
            const uint32_t lo_t = gd.lo & (threads - 1);
            const uint32_t lo_m = gd.lo >> a.tb;
            const C *src = buf + (t ^ lo_t);
            if (gd.d != kFat) {
                const uint32_t s0 = (uint32_t)__popcll(rbase & gd.z0) & 1u;
                const uint32_t W0 = c_walsh[(gd.z0 >> a.tb) & amask];
                uint32_t u = 0, anyW = 0;
                uint32_t W[kDMax];
#pragma unroll
                for (int i = 0; i < kDMax; ++i) {
                    W[i] = 0;
                    if (i < (int)gd.d) {
                        u |= ((uint32_t)__popcll(rbase & gd.beta[i]) & 1u) << i;
                        W[i] = c_walsh[(gd.beta[i] >> a.tb) & amask];
                        anyW |= W[i];
                    }
                }
                if (anyW == 0) {
                    const C D = tables[gd.off + u];
                    C Dn;
                    Dn.re = -D.re;
                    Dn.im = -D.im;
#pragma unroll
                    for (int m = 0; m < AMPS; ++m) {
                        const C p = src[((uint32_t)m ^ lo_m) << a.tb];
                        const uint32_t sg = ((W0 >> m) ^ s0) & 1u;
                        C Dm;
                        Dm.re = sg ? Dn.re : D.re;
                        Dm.im = sg ? Dn.im : D.im;
                        cmac(acc[m], Dm, p);
                    }
                } else {
#pragma unroll
                    for (int m = 0; m < AMPS; ++m) {
                        uint32_t um = u;
#pragma unroll
                        for (int i = 0; i < kDMax; ++i) um ^= ((W[i] >> m) & 1u) << i;
                        const C D = tables[gd.off + um];
                        const C p = src[((uint32_t)m ^ lo_m) << a.tb];
                        const uint32_t sg = ((W0 >> m) ^ s0) & 1u;
                        cmac(acc[m], cneg_if(D, sg), p);
                    }
                }
            } else {
#pragma unroll
                for (int m = 0; m < AMPS; ++m) {
                    const uint64_t r = rbase | ((uint64_t)m << a.tb);
                    C D;
                    D.re = D.im = 0.0;
                    for (uint32_t kk = 0; kk < gd.cnt; ++kk) {
                        const uint64_t zk = a.fat_z[gd.off + kk];
                        const C ck = fat_c[gd.off + kk];
                        const uint32_t sg = (uint32_t)__popcll(r & zk) & 1u;
                        D.re += sg ? -ck.re : ck.re;
                        D.im += sg ? -ck.im : ck.im;
                    }
                    const C p = src[((uint32_t)m ^ lo_m) << a.tb];
                    cmac(acc[m], D, p);
                }
            }
        }

        if (j == nb - 1) {
            C *yo = y + st * a.N + (q << a.b);
#pragma unroll
            for (int m = 0; m < AMPS; ++m) {
                C o = acc[m];
                const uint32_t rl = t + threads * (uint32_t)m;
                if (a.v != nullptr) {  // fused y = alpha (H psi) + beta v
                    const double2 vv = static_cast<const double2 *>(a.v)[st * a.N + (q << a.b) + rl];
                    const double2 r = cx_axpby(a.ar, a.ai, make_double2(o.re, o.im), a.br, a.bi, vv);
                    o.re = r.x;
                    o.im = r.y;
                }
                yo[rl] = o;
            }
        }

        __syncwarp();
        if (lane == 0) {
            __threadfence_block();
            const uint32_t old = atomicAdd(&cnt[s], 1u);
            if (old == nwarps - 1) {
                cnt[s] = 0;
                if (L + (uint64_t)stages < total && *s_abort == 0) {
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    issue(L + (uint64_t)stages);
                }
            }
        }
        if (++s == (uint32_t)stages) {
            s = 0;
            par ^= 1u;
        }
        if (++j == nb) {
            j = 0;
            q += gridDim.x;
            while (q >= a.ntiles) {
                q -= a.ntiles;
                ++st;
            }
        }
    }
    // After an expired wait: every warp has left the loop (no copy is issued
    // after the abort flag is set), then a bounded wait -- with the full 2 s,
    // whatever a test set for the waits -- for the last copy issued into
    // each stage, whose phase parity is (issues - 1) & 1.
    __syncthreads();
    if (t == 0 && *s_abort) {
        for (int k = 0; k < stages; ++k)
            if (s_iss[k] != 0) mbar_wait_bounded(&full[k], (s_iss[k] - 1u) & 1u, kWaitLimitNs);
    }
}

// ---------------------------------------------------------------- c64c kernels
// Compensated complex64 path.  A 4096-amplitude tile is held by T = 512
// threads x AMPS = 8 amplitudes (single-operator and batched kernels);
// thread t owns r_lo = t + T m.  The host splits every x-group into
// sub-groups whose z masks agree on the register bits [kTb, kTb + log2 AMPS)
// and whose z differences span rank <= 2, so for a thread the sub-group's
// factor is
//     D_m = (-1)^popc(m & zm) * Dt,   Dt = (-1)^popc(r0 & z0) * tab[u],
// r0 = (tile << b) | t, u_i = popc(r0 & beta_i) & 1.  The sign pattern over
// m selects a compile-time instantiation, so the inner step per amplitude is
// one shared-memory load and two packed FMAs:
//     A_m += (+-Dt.re) * p,  B_m += (+-Dt.im) * p      (fma.rn.f32x2)
// and y = A + iB is folded into the running (hi, lo) two-sum pair every
// kFlush partner tiles; hi stays in registers, the error term lo (touched
// only at a fold) lives in shared memory.
//
// Pipeline: a ring of partner tiles filled by 1-D TMA bulk copies.  Warps run
// decoupled: each waits on the stage's full mbarrier, consumes it, and counts
// itself out on a shared counter; the last warp out refills the stage with
// the tile a ring length ahead.  No CTA-wide barrier sits on the
// steady-state path.  The kernels run 16 warps per SM (512 x 8 hides more
// latency than 256 x 16, and fewer register bits leave fewer sign patterns
// to split on).
constexpr int kTb = kC64ThreadBits;       // log2(threads) whenever AMPS >= 2
constexpr int kMsh = kTb + 3;             // byte shift of the register index m
constexpr int kFlush = 8;                 // partner tiles per compensated fold
constexpr int kC64Threads = 1 << kTb;

template <bool WIDE>
__device__ __forceinline__ uint32_t parity(uint64_t r, uint64_t m) {
    if constexpr (WIDE) return (uint32_t)__popcll(r & m) & 1u;
    else return (uint32_t)__popc((uint32_t)r & (uint32_t)m) & 1u;
}

// ---------------------------------------------------------------- c64c, tile table
// The single-operator compensated-c64 kernel.  The per-sub-group work is
// split by who can do it once:
//   * per output tile (cooperatively, into shared memory): for every
//     sub-group the tile-index parity of z0 / beta0,1 applied to its table,
//     stored pre-duplicated as (re, re, im, im) for the packed FMAs;
//   * per thread: the parities of its thread index against 8-bit masks
//     (skipped when the sub-group's masks miss the thread bits), one 16-byte
//     table read, the partner offset;
//   * per run of sub-groups with equal register-bit sign pattern: one
//     dispatch to a compile-time instantiation.
constexpr int kTabStages = 4;  // partner-tile ring depth (timed best of 3, 4, 5)
constexpr size_t kMaxSmemPerBlock = 227u * 1024u;  // sm_100-family opt-in limit
constexpr int kTabEnt = 4;  // per-tile table entries (float4) per sub-group
constexpr uint32_t kTabBhiCap = 1024;  // partner blocks whose XORs are staged in shared memory
// full barriers, stage counters, the abort flag and per-stage issue counts,
// rounded to 16 bytes so that the 16-byte thread descriptors after them stay
// aligned
constexpr size_t kTabBarBytes = ((size_t)kTabStages * 16u + 4u + 15u) & ~(size_t)15u;
static_assert(kTabBarBytes % 16 == 0, "thread descriptors need 16-byte alignment");
// paired kernel: up to three ring slots of two partner tiles; barriers,
// counters, the abort flag and issue counts in 64 bytes
constexpr uint32_t kMaxPairSlots = 3;
constexpr size_t kPairBarBytes = 64;
static_assert(kMaxPairSlots * 8 + kMaxPairSlots * 4 + 4 + kMaxPairSlots * 4 <= kPairBarBytes,
              "pair barrier block");

template <int AMPS, int ZM, bool XM, bool TV>
__device__ __forceinline__ void sub_tab_one(float2 (&A)[AMPS], float2 (&B)[AMPS],
                                            const unsigned char *sm, uint32_t soff,
                                            const float4 *s_tab, const uint4 *tdesc, uint32_t g,
                                            uint32_t t, uint32_t t8) {
    {
        const uint4 d = tdesc[g];
        // thread parities against the three masks, only in runs whose factor
        // depends on the thread (compile-time: no branch per sub-group)
        uint32_t u = 0, sg = 0;
        if constexpr (TV) {
            sg = (uint32_t)__popc(t & d.y) & 1u;
            u = ((uint32_t)__popc(t & d.z) & 1u) | (((uint32_t)__popc(t & d.w) & 1u) << 1);
        }
        const float4 T = s_tab[g * 4 + u];
        // thread sign (-1)^sg on both factor pairs: one packed multiply each
        // (runs whose factor does not depend on the thread have none)
        float2 ap = make_float2(T.x, T.y), bp = make_float2(T.z, T.w);
        if constexpr (TV) {
            const float sv = __uint_as_float(0x3f800000u | (sg << 31));
            ap = __fmul2_rn(ap, make_float2(sv, sv));
            bp = __fmul2_rn(bp, make_float2(sv, sv));
        }
        // partner byte offset: the XOR part (thread and register bits of lo) is
        // precomputed per sub-group; the stage offset occupies higher bits
        const uint32_t off = soff | (t8 ^ (d.x & 0xffffu));  // bit 15: pair half
        float2 p[AMPS];
#pragma unroll
        for (int m = 0; m < AMPS; ++m) {
            const uint32_t o = XM ? (off ^ ((uint32_t)m << kMsh)) : (off + ((uint32_t)m << kMsh));
            p[m] = *reinterpret_cast<const float2 *>(sm + o);
        }
        float2 an = ap, bn = bp;
        if constexpr (ZM != 0) {
            an = __fmul2_rn(ap, make_float2(-1.f, -1.f));
            bn = __fmul2_rn(bp, make_float2(-1.f, -1.f));
        }
#pragma unroll
        for (int m = 0; m < AMPS; ++m) {
            const bool neg = (__builtin_popcount((unsigned)(m & ZM)) & 1) != 0;
            A[m] = __ffma2_rn(neg ? an : ap, p[m], A[m]);
            B[m] = __ffma2_rn(neg ? bn : bp, p[m], B[m]);
        }
    }
}

// two sub-groups per iteration: the second one's loads can issue ahead of
// the first one's packed FMAs
template <int AMPS, int ZM, bool XM, bool TV>
__device__ __forceinline__ void run_tab(float2 (&A)[AMPS], float2 (&B)[AMPS],
                                        const unsigned char *sm, uint32_t soff,
                                        const float4 *s_tab, const uint4 *tdesc, uint32_t g0,
                                        uint32_t g1, uint32_t t, uint32_t t8) {
    uint32_t g = g0;
    for (; g + 1 < g1; g += 2) {
        sub_tab_one<AMPS, ZM, XM, TV>(A, B, sm, soff, s_tab, tdesc, g, t, t8);
        sub_tab_one<AMPS, ZM, XM, TV>(A, B, sm, soff, s_tab, tdesc, g + 1, t, t8);
    }
    if (g < g1) sub_tab_one<AMPS, ZM, XM, TV>(A, B, sm, soff, s_tab, tdesc, g, t, t8);
}

// A pair of key-0 sub-groups g, g+1 in halves 0 and 1 of the slot whose x
// masks leave the partner tiles unpermuted: each has one factor for every
// thread and amplitude (table entry u = 0), and amplitude m of thread t sits
// at a fixed offset from t * 8 in its half -- no descriptor, no address
// arithmetic.  Same products in the same order as two sub_tab_one calls.
template <int AMPS>
__device__ __forceinline__ void cheap_pair_lo0(float2 (&A)[AMPS], float2 (&B)[AMPS],
                                               const unsigned char *sm, uint32_t base,
                                               const float4 *s_tab, uint32_t g) {
    const float4 Ta = s_tab[g * 4], Tb = s_tab[(g + 1) * 4];
    const unsigned char *h0 = sm + base;
    const unsigned char *h1 = h0 + 32768u;
    float2 p[AMPS];
#pragma unroll
    for (int m = 0; m < AMPS; ++m) p[m] = *reinterpret_cast<const float2 *>(h0 + ((uint32_t)m << kMsh));
#pragma unroll
    for (int m = 0; m < AMPS; ++m) {
        A[m] = __ffma2_rn(make_float2(Ta.x, Ta.y), p[m], A[m]);
        B[m] = __ffma2_rn(make_float2(Ta.z, Ta.w), p[m], B[m]);
    }
#pragma unroll
    for (int m = 0; m < AMPS; ++m) p[m] = *reinterpret_cast<const float2 *>(h1 + ((uint32_t)m << kMsh));
#pragma unroll
    for (int m = 0; m < AMPS; ++m) {
        A[m] = __ffma2_rn(make_float2(Tb.x, Tb.y), p[m], A[m]);
        B[m] = __ffma2_rn(make_float2(Tb.z, Tb.w), p[m], B[m]);
    }
}

// Two sub-groups g, g+1 of one x group (same partner amplitudes) whose
// register-bit sign patterns are ZM and ZM ^ (1 << BB): an x group split
// because its terms' z differ on one register bit.  One set of partner loads
// serves both; the factor at register index m is
//   (-1)^popc(m & ZM) * (F_g + (-1)^(m_BB) F_{g+1}),
// with F the thread-signed table entries, so the pair costs the packed FMAs
// of a single sub-group plus four packed adds.
template <int AMPS, int ZM, int BB, bool XM, bool TV>
__device__ __forceinline__ void sub_tab_fused(float2 (&A)[AMPS], float2 (&B)[AMPS],
                                              const unsigned char *sm, uint32_t soff,
                                              const float4 *s_tab, const uint4 *tdesc, uint32_t g,
                                              uint32_t t, uint32_t t8) {
    const uint4 da = tdesc[g], db = tdesc[g + 1];
    uint32_t ua = 0, sa = 0, ub = 0, sb = 0;
    if constexpr (TV) {
        sa = (uint32_t)__popc(t & da.y) & 1u;
        ua = ((uint32_t)__popc(t & da.z) & 1u) | (((uint32_t)__popc(t & da.w) & 1u) << 1);
        sb = (uint32_t)__popc(t & db.y) & 1u;
        ub = ((uint32_t)__popc(t & db.z) & 1u) | (((uint32_t)__popc(t & db.w) & 1u) << 1);
    }
    const float4 Ta = s_tab[g * 4 + ua];
    const float4 Tb = s_tab[(g + 1) * 4 + ub];
    const float sva = __uint_as_float(0x3f800000u | (sa << 31));
    const float svb = __uint_as_float(0x3f800000u | (sb << 31));
    float2 apa = make_float2(Ta.x, Ta.y), bpa = make_float2(Ta.z, Ta.w);
    if constexpr (TV) {
        apa = __fmul2_rn(apa, make_float2(sva, sva));
        bpa = __fmul2_rn(bpa, make_float2(sva, sva));
    }
    // F_a + F_b and F_a - F_b: one rounding each (the sign products are exact)
    const float2 a0 = __ffma2_rn(make_float2(Tb.x, Tb.y), make_float2(svb, svb), apa);
    const float2 b0 = __ffma2_rn(make_float2(Tb.z, Tb.w), make_float2(svb, svb), bpa);
    const float2 a1 = __ffma2_rn(make_float2(Tb.x, Tb.y), make_float2(-svb, -svb), apa);
    const float2 b1 = __ffma2_rn(make_float2(Tb.z, Tb.w), make_float2(-svb, -svb), bpa);
    const uint32_t off = soff | (t8 ^ (da.x & 0xffffu));
    float2 p[AMPS];
#pragma unroll
    for (int m = 0; m < AMPS; ++m) {
        const uint32_t o = XM ? (off ^ ((uint32_t)m << kMsh)) : (off + ((uint32_t)m << kMsh));
        p[m] = *reinterpret_cast<const float2 *>(sm + o);
    }
    float2 na0 = a0, nb0 = b0, na1 = a1, nb1 = b1;
    if constexpr (ZM != 0) {
        na0 = __fmul2_rn(a0, make_float2(-1.f, -1.f));
        nb0 = __fmul2_rn(b0, make_float2(-1.f, -1.f));
        na1 = __fmul2_rn(a1, make_float2(-1.f, -1.f));
        nb1 = __fmul2_rn(b1, make_float2(-1.f, -1.f));
    }
#pragma unroll
    for (int m = 0; m < AMPS; ++m) {
        const bool neg = (__builtin_popcount((unsigned)(m & ZM)) & 1) != 0;
        const bool sel = ((m >> BB) & 1) != 0;
        const float2 fa = neg ? (sel ? na1 : na0) : (sel ? a1 : a0);
        const float2 fb = neg ? (sel ? nb1 : nb0) : (sel ? b1 : b0);
        A[m] = __ffma2_rn(fa, p[m], A[m]);
        B[m] = __ffma2_rn(fb, p[m], B[m]);
    }
}

template <int AMPS, int ZM, int BB, bool XM, bool TV>
__device__ __forceinline__ void run_fused(float2 (&A)[AMPS], float2 (&B)[AMPS],
                                          const unsigned char *sm, uint32_t soff,
                                          const float4 *s_tab, const uint4 *tdesc, uint32_t g0,
                                          uint32_t g1, uint32_t t, uint32_t t8) {
    for (uint32_t g = g0; g + 1 < g1; g += 2)
        sub_tab_fused<AMPS, ZM, BB, XM, TV>(A, B, sm, soff, s_tab, tdesc, g, t, t8);
}

template <int AMPS>
__device__ __forceinline__ void run_tab_dispatch(uint32_t key, float2 (&A)[AMPS],
                                                 float2 (&B)[AMPS], const unsigned char *sm,
                                                 uint32_t soff, const float4 *s_tab,
                                                 const uint4 *tdesc, uint32_t g0, uint32_t g1,
                                                 uint32_t t, uint32_t t8) {
#define QR_RUN_CASE(k)                                                                    \
    case k:                                                                               \
        if constexpr ((k & 15) < AMPS)                                                    \
            run_tab<AMPS, (k & 15), ((k >> 4) & 1) != 0, (k >> 5) != 0>(A, B, sm, soff, s_tab, \
                                                                       tdesc, g0, g1, t, t8); \
        break;
#define QR_RUN_CASE8(k) QR_RUN_CASE(k) QR_RUN_CASE(k + 1) QR_RUN_CASE(k + 2) QR_RUN_CASE(k + 3) \
    QR_RUN_CASE(k + 4) QR_RUN_CASE(k + 5) QR_RUN_CASE(k + 6) QR_RUN_CASE(k + 7)
    switch (key) {
        QR_RUN_CASE8(0) QR_RUN_CASE8(8) QR_RUN_CASE8(16) QR_RUN_CASE8(24)
        QR_RUN_CASE8(32) QR_RUN_CASE8(40) QR_RUN_CASE8(48) QR_RUN_CASE8(56)
        default: break;
    }
#undef QR_RUN_CASE8
#undef QR_RUN_CASE
}

// Pair-plan runs: keys below 64 as run_tab_dispatch; 64 + (ZM | BB << 3 |
// XM << 5 | TV << 6) is a run of fused sub-group pairs (sub_tab_fused).
template <int AMPS>
__device__ __forceinline__ void run_pair_dispatch(uint32_t key, float2 (&A)[AMPS],
                                                  float2 (&B)[AMPS], const unsigned char *sm,
                                                  uint32_t soff, const float4 *s_tab,
                                                  const uint4 *tdesc, uint32_t g0, uint32_t g1,
                                                  uint32_t t, uint32_t t8) {
    if (key < 64u) {
        run_tab_dispatch<AMPS>(key, A, B, sm, soff, s_tab, tdesc, g0, g1, t, t8);
        return;
    }
#define QR_FUSED_CASE(k)                                                                  \
    case k:                                                                               \
        if constexpr ((k & 7) < AMPS && (1 << ((k >> 3) & 3)) < AMPS)                     \
            run_fused<AMPS, (k & 7), ((k >> 3) & 3), ((k >> 5) & 1) != 0, ((k >> 6) & 1) != 0>( \
                A, B, sm, soff, s_tab, tdesc, g0, g1, t, t8);                             \
        break;
#define QR_FUSED_CASE8(k) QR_FUSED_CASE(k) QR_FUSED_CASE(k + 1) QR_FUSED_CASE(k + 2) \
    QR_FUSED_CASE(k + 3) QR_FUSED_CASE(k + 4) QR_FUSED_CASE(k + 5) QR_FUSED_CASE(k + 6) \
    QR_FUSED_CASE(k + 7)
    switch (key - 64u) {
        QR_FUSED_CASE8(0) QR_FUSED_CASE8(8) QR_FUSED_CASE8(16)
        QR_FUSED_CASE8(32) QR_FUSED_CASE8(40) QR_FUSED_CASE8(48)
        QR_FUSED_CASE8(64) QR_FUSED_CASE8(72) QR_FUSED_CASE8(80)
        QR_FUSED_CASE8(96) QR_FUSED_CASE8(104) QR_FUSED_CASE8(112)
        default: break;
    }
#undef QR_FUSED_CASE8
#undef QR_FUSED_CASE
}

template <int AMPS, bool WIDE, bool MULTI>
__global__ void __launch_bounds__(kC64Threads, 1) apply_c64c_tab(const ApplyArgs a) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const uint32_t threads = blockDim.x;
    const uint32_t nwarps = threads >> 5;
    const uint32_t t = threadIdx.x;
    const uint32_t lane = t & 31;
    const uint32_t tile_bytes = (1u << a.b) * 8u;
    const uint32_t tabn = a.nsub < kTabCap ? a.nsub : kTabCap;
    float4 *s_tab = reinterpret_cast<float4 *>(smem_raw + (size_t)kTabStages * tile_bytes);
    float2 *s_lo = reinterpret_cast<float2 *>(s_tab + kTabEnt * (size_t)tabn);
    uint64_t *full = reinterpret_cast<uint64_t *>(s_lo + (size_t)AMPS * threads);
    uint32_t *cnt = reinterpret_cast<uint32_t *>(full + kTabStages);
    volatile uint32_t *s_abort = cnt + kTabStages;
    // copies issued into each stage: the drain after an expired wait waits
    // for the last one's phase, so no copy is in flight when the CTA exits
    uint32_t *s_iss = cnt + kTabStages + 1;
    // sub-group descriptors, runs (g0 | key << 16) and per-block run ranges of
    // the current chunk, indices relative to the chunk; with one chunk they
    // are staged once per CTA
    uint4 *s_td = reinterpret_cast<uint4 *>(reinterpret_cast<unsigned char *>(s_lo) +
                                            (size_t)AMPS * threads * 8u + kTabBarBytes);
    uint32_t *s_run = reinterpret_cast<uint32_t *>(s_td + kTabCap);
    uint32_t *s_blk = s_run + kTabCap + 1;
    // partner-tile XORs in shared memory (up to kTabBhiCap blocks): a refill
    // needs no global load first
    uint64_t *s_bhi = reinterpret_cast<uint64_t *>(
        (reinterpret_cast<uintptr_t>(s_blk + kTabCap + 2) + 7u) & ~(uintptr_t)7u);
    const bool bhi_smem = a.nblocks <= kTabBhiCap;
    if (bhi_smem)
        for (uint32_t i = t; i < a.nblocks; i += threads) s_bhi[i] = a.blk_hi[i];
    const uint64_t *bhi = bhi_smem ? s_bhi : a.blk_hi;
    if constexpr (!MULTI) {
        for (uint32_t i = t; i < a.nsub; i += threads) s_td[i] = a.tdesc[i];
        for (uint32_t i = t; i <= a.nruns; i += threads)
            s_run[i] = a.run_g0[i] | (i < a.nruns ? a.run_key[i] << 16 : 0u);
        for (uint32_t i = t; i <= a.nblocks; i += threads) s_blk[i] = a.blk_r0[i];
    }
    const uint4 *tdesc = s_td;

    const float2 *psi = static_cast<const float2 *>(a.psi);
    float2 *y = static_cast<float2 *>(a.y);
    const float2 *diag = static_cast<const float2 *>(a.diag);
    const uint32_t nb = a.nblocks;
    const uint32_t t8 = t << 3;

    const uint64_t first = blockIdx.x;
    const uint64_t my_items =
        a.nitems > first ? (a.nitems - first + gridDim.x - 1) / gridDim.x : 0;
    const uint64_t total = my_items * nb;
    if (total == 0) return;

    auto issue = [&](uint64_t L) {
        const uint64_t k = L / nb;
        const uint32_t j = (uint32_t)(L - k * nb);
        const uint64_t item = first + k * gridDim.x;
        const uint64_t st = item / a.ntiles;
        const uint64_t q = item - st * a.ntiles;
        const float2 *src = psi + st * a.N + ((q ^ bhi[j]) << a.b);
        const int s = (int)(L % (uint64_t)kTabStages);
        if (blockIdx.x == 0 && (int64_t)L == a.withhold) return;  // test hook: never issued
        ++s_iss[s];
        mbar_expect_tx(&full[s], tile_bytes);
        bulk_g2s(smem_raw + (size_t)s * tile_bytes, src, tile_bytes, &full[s]);
    };
    __syncthreads();  // the prologue reads s_bhi
    if (t == 0) {
        for (int s = 0; s < kTabStages; ++s) {
            mbar_init(&full[s], 1);
            cnt[s] = 0;
            s_iss[s] = 0;
        }
        *s_abort = 0;
        mbar_fence_init();
        const uint64_t pro = total < (uint64_t)kTabStages ? total : (uint64_t)kTabStages;
        for (uint64_t L = 0; L < pro; ++L) issue(L);
    }
    __syncthreads();

    float2 A[AMPS], B[AMPS], hi[AMPS];
    float2 *mylo = s_lo + t;
    uint32_t j = 0, s = 0, par = 0;
    uint32_t cidx = 0, cj0 = 0, next_j = 0;  // current chunk, its first block, the next's
    uint64_t st = first / a.ntiles;
    uint64_t q = first - st * a.ntiles;

    for (uint64_t L = 0; L < total; ++L) {
        if (j == 0) {
#pragma unroll
            for (int m = 0; m < AMPS; ++m) {
                A[m] = B[m] = hi[m] = make_float2(0.f, 0.f);
                mylo[m * threads] = make_float2(0.f, 0.f);
            }
            cidx = 0;
        }
        if (j == 0 || (MULTI && j == next_j)) {
            // table (and, with several chunks, run lists) of the chunk that
            // starts at block j: every warp has finished the previous one
            if (j != 0) ++cidx;
            __syncthreads();
            uint4 c0 = make_uint4(0u, 0u, 0u, 0u), c1 = make_uint4(a.nsub, a.nruns, a.nblocks, 0u);
            if constexpr (MULTI) {
                c0 = a.chunks[cidx];
                c1 = a.chunks[cidx + 1];
                cj0 = c0.z;
                next_j = c1.z;
                for (uint32_t i = t; i < c1.x - c0.x; i += threads) s_td[i] = a.tdesc[c0.x + i];
                for (uint32_t i = t; i <= c1.y - c0.y; i += threads) {
                    const uint32_t r = c0.y + i;
                    s_run[i] = (a.run_g0[r] - c0.x) | (r < a.nruns ? a.run_key[r] << 16 : 0u);
                }
                for (uint32_t i = t; i <= c1.z - c0.z; i += threads)
                    s_blk[i] = a.blk_r0[c0.z + i] - c0.y;
            }
            for (uint32_t gi = t; gi < c1.x - c0.x; gi += threads) {
                const TileDataC64 &d = a.tdata[c0.x + gi];
                const uint32_t uq = parity<WIDE>(q, d.b0h) | (parity<WIDE>(q, d.b1h) << 1);
                const float sq = parity<WIDE>(q, d.z0h) ? -1.f : 1.f;
#pragma unroll
                for (uint32_t u = 0; u < 4; ++u) {
                    const float2 v = d.T[u ^ uq];
                    s_tab[gi * 4 + u] = make_float4(sq * v.x, sq * v.x, sq * v.y, sq * v.y);
                }
            }
            __syncthreads();
        }
        // A wait that expires sets the abort flag; from then on every warp
        // skips waits and work but still reaches each tile barrier.
        bool skip = *s_abort != 0;
        if (!skip && !mbar_wait_bounded(&full[s], par, a.wait_ns)) {
            if (lane == 0) {
                atomicExch(a.err, kErrMbarTimeout);
                *s_abort = 1;
            }
            skip = true;
        }
        skip = __any_sync(0xffffffffu, skip);
        const uint32_t soff = s * tile_bytes;

        if (!skip && (int)j == a.diag_block && diag != nullptr) {
            const float2 *dg = diag + (q << a.b);
#pragma unroll
            for (int m = 0; m < AMPS; ++m) {
                const uint32_t rl = t + threads * (uint32_t)m;
                const float2 d = dg[rl];
                const float2 p = *reinterpret_cast<const float2 *>(smem_raw + soff + rl * 8u);
                A[m] = __ffma2_rn(make_float2(d.x, d.x), p, A[m]);
                B[m] = __ffma2_rn(make_float2(d.y, d.y), p, B[m]);
            }
        }

        const uint32_t jl = MULTI ? j - cj0 : j;
        const uint32_t r1 = skip ? 0u : s_blk[jl + 1];
        uint32_t rw = s_run[s_blk[jl]];
        for (uint32_t r = s_blk[jl]; r < r1; ++r) {
            const uint32_t rn = s_run[r + 1];
            run_tab_dispatch<AMPS>(rw >> 16, A, B, smem_raw, soff, s_tab, tdesc, rw & 0xffffu,
                                   rn & 0xffffu, t, t8);
            rw = rn;
        }

        const bool last = (j == nb - 1);
        if (last || (j % kFlush) == kFlush - 1) {
#pragma unroll
            for (int m = 0; m < AMPS; ++m) {
                const float yr = __fsub_rn(A[m].x, B[m].y);
                const float yi = __fadd_rn(A[m].y, B[m].x);
                float2 lm = mylo[m * threads];
                two_sum_into(hi[m].x, lm.x, yr);
                two_sum_into(hi[m].y, lm.y, yi);
                mylo[m * threads] = lm;
                A[m] = B[m] = make_float2(0.f, 0.f);
            }
        }
        if (last) {
            float2 *yo = y + st * a.N + (q << a.b);
            const float2 *vo = a.v ? static_cast<const float2 *>(a.v) + st * a.N + (q << a.b)
                                   : nullptr;
#pragma unroll
            for (int m = 0; m < AMPS; ++m) {
                const float2 lm = mylo[m * threads];
                const uint32_t rl = t + threads * (uint32_t)m;
                float2 o = make_float2(__fadd_rn(hi[m].x, lm.x), __fadd_rn(hi[m].y, lm.y));
                if (vo)  // fused y = alpha (H psi) + beta v, in FP32
                    o = cx_axpby((float)a.ar, (float)a.ai, o, (float)a.br, (float)a.bi, vo[rl]);
                yo[rl] = o;
            }
        }

        __syncwarp();
        if (lane == 0) {
            __threadfence_block();
            const uint32_t old = atomicAdd(&cnt[s], 1u);
            if (old == nwarps - 1) {
                cnt[s] = 0;
                if (L + (uint64_t)kTabStages < total && *s_abort == 0) {
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    // step kTabStages partner blocks ahead of (st, q, j) with
                    // adds only (no 64-bit division on the steady-state path)
                    uint32_t j2 = j + (uint32_t)kTabStages;
                    uint64_t q2 = q, st2 = st;
                    while (j2 >= nb) {
                        j2 -= nb;
                        q2 += gridDim.x;
                        while (q2 >= a.ntiles) {
                            q2 -= a.ntiles;
                            ++st2;
                        }
                    }
                    const float2 *src = psi + st2 * a.N + ((q2 ^ bhi[j2]) << a.b);
                    if (blockIdx.x != 0 || (int64_t)(L + kTabStages) != a.withhold) {
                        ++s_iss[s];
                        mbar_expect_tx(&full[s], tile_bytes);
                        bulk_g2s(smem_raw + (size_t)s * tile_bytes, src, tile_bytes, &full[s]);
                    }
                }
            }
        }
        if (++s == kTabStages) {
            s = 0;
            par ^= 1u;
        }
        if (++j == nb) {
            j = 0;
            q += gridDim.x;
            while (q >= a.ntiles) {
                q -= a.ntiles;
                ++st;
            }
        }
    }
    // After an expired wait: every warp has left the loop (no copy is issued
    // after the abort flag is set), then a bounded wait for the last copy
    // issued into each stage -- its phase parity is (issues - 1) & 1 -- so
    // that no copy still targets this CTA's shared memory when it exits.
    // The drain keeps the full 2 s bound whatever a test set for the waits:
    // an issued copy always completes.
    __syncthreads();
    if (t == 0 && *s_abort) {
        for (int k = 0; k < kTabStages; ++k)
            if (s_iss[k] != 0) mbar_wait_bounded(&full[k], (s_iss[k] - 1u) & 1u, kWaitLimitNs);
    }
}

// Single-chunk kernel with partner blocks visited in pairs: blocks 2p and
// 2p+1 are loaded into the two stages of one ring slot behind one barrier,
// and the pair's sub-groups (merged, sorted by run key, bit 15 of the
// descriptor's offset selecting the stage) run as one list.  Most partner
// blocks of pair-structured operators hold a single sub-group, for which the
// per-block ring wait, run lookup, dispatch and stage release cost more than
// the sub-group itself.
template <int AMPS, bool WIDE>
__global__ void __launch_bounds__(kC64Threads, 1) apply_c64c_pair(const ApplyArgs a) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const uint32_t threads = blockDim.x;
    const uint32_t nwarps = threads >> 5;
    const uint32_t t = threadIdx.x;
    const uint32_t lane = t & 31;
    const uint32_t tile_bytes = (1u << a.b) * 8u;
    // layout (pair_smem_bytes): ring of nsl slots of two tiles, factor table,
    // barriers / counters (64 bytes), thread descriptors, run list, pair list
    const uint32_t nsl = a.pair_slots;
    const uint32_t tabn = a.nsub;  // a pair plan has at most kTabCap sub-groups
    float4 *s_tab = reinterpret_cast<float4 *>(smem_raw + (size_t)nsl * 2u * tile_bytes);
    uint64_t *full = reinterpret_cast<uint64_t *>(s_tab + kTabEnt * (size_t)tabn);
    uint32_t *cnt = reinterpret_cast<uint32_t *>(full + kMaxPairSlots);
    volatile uint32_t *s_abort = cnt + kMaxPairSlots;
    // copies issued into each slot: the drain after an expired wait waits
    // for the last one's phase, so no copy is in flight when the CTA exits
    uint32_t *s_iss = cnt + kMaxPairSlots + 1;
    uint4 *s_td = reinterpret_cast<uint4 *>(reinterpret_cast<unsigned char *>(full) + kPairBarBytes);
    uint32_t *s_run = reinterpret_cast<uint32_t *>(s_td + tabn);
    uint32_t *s_blk = s_run + a.nruns + 1;
    const uint32_t np = a.npairs, nb = a.nblocks;
    uint64_t *s_bhi = reinterpret_cast<uint64_t *>(
        (reinterpret_cast<uintptr_t>(s_blk + np + 1) + 7u) & ~(uintptr_t)7u);
    for (uint32_t i = t; i < a.nsub; i += threads) s_td[i] = a.tdesc[i];
    for (uint32_t i = t; i <= a.nruns; i += threads)
        s_run[i] = a.run_g0[i] | (i < a.nruns ? a.run_key[i] << 16 : 0u);
    for (uint32_t i = t; i <= np; i += threads) s_blk[i] = a.blk_r0[i];
    for (uint32_t i = t; i < nb; i += threads) s_bhi[i] = a.blk_hi[i];
    __syncthreads();  // the prologue reads s_bhi
    const uint4 *tdesc = s_td;

    const float2 *psi = static_cast<const float2 *>(a.psi);
    float2 *y = static_cast<float2 *>(a.y);
    const float2 *diag = static_cast<const float2 *>(a.diag);
    const uint32_t t8 = t << 3;
    const uint32_t slot_bytes = 2u * tile_bytes;
    const int diag_pair = a.diag_block >= 0 ? (a.diag_block >> 1) : -1;
    const uint32_t diag_half = a.diag_block >= 0 ? ((uint32_t)a.diag_block & 1u) : 0u;

    const uint64_t first = blockIdx.x;
    const uint64_t my_items =
        a.nitems > first ? (a.nitems - first + gridDim.x - 1) / gridDim.x : 0;
    const uint64_t total = my_items * np;
    if (total == 0) return;

    // load pair p of tile (st, q) into slot s: one or two partner tiles
    auto issue_pair = [&](uint64_t L, uint32_t s, uint32_t p, uint64_t st, uint64_t q) {
        if (blockIdx.x == 0 && (int64_t)L == a.withhold) return;  // test hook: never issued
        const uint32_t j0 = 2u * p;
        const uint32_t ntl = j0 + 1 < nb ? 2u : 1u;
        ++s_iss[s];
        mbar_expect_tx(&full[s], ntl * tile_bytes);
        for (uint32_t h = 0; h < ntl; ++h) {
            const float2 *src = psi + st * a.N + ((q ^ s_bhi[j0 + h]) << a.b);
            bulk_g2s(smem_raw + (size_t)s * slot_bytes + (size_t)h * tile_bytes, src, tile_bytes,
                     &full[s]);
        }
    };
    uint64_t st = first / a.ntiles;
    uint64_t q = first - st * a.ntiles;
    if (t == 0) {
        for (uint32_t s = 0; s < nsl; ++s) {
            mbar_init(&full[s], 1);
            cnt[s] = 0;
            s_iss[s] = 0;
        }
        *s_abort = 0;
        mbar_fence_init();
        // prologue: steps 0 .. nsl - 1
        uint32_t p1 = 0;
        uint64_t q1 = q, st1 = st;
        for (uint64_t L = 0; L < total && L < nsl; ++L) {
            issue_pair(L, (uint32_t)L, p1, st1, q1);
            if (++p1 == np) {
                p1 = 0;
                q1 += gridDim.x;
                while (q1 >= a.ntiles) {
                    q1 -= a.ntiles;
                    ++st1;
                }
            }
        }
    }
    __syncthreads();

    // y = A + iB is the FP32 sum of the current window of pairs; every 16
    // pairs it is folded into hi with an error-free two-sum, and the error of
    // that addition is carried into the next window (A starts from it: the
    // compensated summation of Kahan, with no separate low word to keep);
    // the last fold's error is added at the store
    float2 A[AMPS], B[AMPS], hi[AMPS];
    uint32_t p = 0, s = 0, par = 0;
    constexpr uint32_t kFlushPairs = 16;

    for (uint64_t L = 0; L < total; ++L) {
        if (p == 0) {
#pragma unroll
            for (int m = 0; m < AMPS; ++m) A[m] = B[m] = hi[m] = make_float2(0.f, 0.f);
            // table of the new output tile: every warp has finished the last one
            __syncthreads();
            for (uint32_t gi = t; gi < a.nsub; gi += threads) {
                const TileDataC64 &d = a.tdata[gi];
                const uint32_t uq = parity<WIDE>(q, d.b0h) | (parity<WIDE>(q, d.b1h) << 1);
                const float sq = parity<WIDE>(q, d.z0h) ? -1.f : 1.f;
#pragma unroll
                for (uint32_t u = 0; u < 4; ++u) {
                    const float2 v = d.T[u ^ uq];
                    s_tab[gi * 4 + u] = make_float4(sq * v.x, sq * v.x, sq * v.y, sq * v.y);
                }
            }
            __syncthreads();
        }
        // fast path: the stage is complete for the whole warp; otherwise the
        // bounded wait, which also honours another warp's abort
        bool skip = false;
        if (!__all_sync(0xffffffffu, mbar_try_wait(&full[s], par))) {
            skip = *s_abort != 0;
            if (!skip && !mbar_wait_bounded(&full[s], par, a.wait_ns)) {
                if (lane == 0) {
                    atomicExch(a.err, kErrMbarTimeout);
                    *s_abort = 1;
                }
                skip = true;
            }
            skip = __any_sync(0xffffffffu, skip);
        }
        const uint32_t soff = s * slot_bytes;

        if (!skip && (int)p == diag_pair && diag != nullptr) {
            const float2 *dg = diag + (q << a.b);
            const uint32_t doff = soff + diag_half * tile_bytes;
#pragma unroll
            for (int m = 0; m < AMPS; ++m) {
                const uint32_t rl = t + threads * (uint32_t)m;
                const float2 d = dg[rl];
                const float2 pv = *reinterpret_cast<const float2 *>(smem_raw + doff + rl * 8u);
                A[m] = __ffma2_rn(make_float2(d.x, d.x), pv, A[m]);
                B[m] = __ffma2_rn(make_float2(d.y, d.y), pv, B[m]);
            }
        }

        // bit 31 of a pair's first run: exactly two sub-groups of key 0; bit
        // 30: in halves 0 and 1, partner tiles unpermuted
        const uint32_t bw = s_blk[p];
        const uint32_t rb = bw & 0x3fffffffu;
        if (!skip && (bw >> 31) != 0) {
            const uint32_t g0 = s_run[rb] & 0xffffu;
            if ((bw >> 30) & 1u) {
                cheap_pair_lo0<AMPS>(A, B, smem_raw, soff | t8, s_tab, g0);
            } else {
                sub_tab_one<AMPS, 0, false, false>(A, B, smem_raw, soff, s_tab, tdesc, g0, t, t8);
                sub_tab_one<AMPS, 0, false, false>(A, B, smem_raw, soff, s_tab, tdesc, g0 + 1, t,
                                                   t8);
            }
        } else {
            const uint32_t r1 = skip ? 0u : (s_blk[p + 1] & 0x3fffffffu);
            uint32_t rw = s_run[rb];
            for (uint32_t r = rb; r < r1; ++r) {
                const uint32_t rn = s_run[r + 1];
                run_pair_dispatch<AMPS>(rw >> 16, A, B, smem_raw, soff, s_tab, tdesc,
                                        rw & 0xffffu, rn & 0xffffu, t, t8);
                rw = rn;
            }
        }

        const bool last = (p == np - 1);
        if (last || (p % kFlushPairs) == kFlushPairs - 1) {
#pragma unroll
            for (int m = 0; m < AMPS; ++m) {
                const float2 yv =
                    make_float2(__fsub_rn(A[m].x, B[m].y), __fadd_rn(A[m].y, B[m].x));
                A[m] = two_sum_carry2(hi[m], yv);  // the error opens the next window
                B[m] = make_float2(0.f, 0.f);
            }
        }
        if (last) {
            float2 *yo = y + st * a.N + (q << a.b);
            const float2 *vo = a.v ? static_cast<const float2 *>(a.v) + st * a.N + (q << a.b)
                                   : nullptr;
#pragma unroll
            for (int m = 0; m < AMPS; ++m) {
                const uint32_t rl = t + threads * (uint32_t)m;
                float2 o = make_float2(__fadd_rn(hi[m].x, A[m].x), __fadd_rn(hi[m].y, A[m].y));
                if (vo)  // fused y = alpha (H psi) + beta v, in FP32
                    o = cx_axpby((float)a.ar, (float)a.ai, o, (float)a.br, (float)a.bi, vo[rl]);
                yo[rl] = o;
            }
        }

        __syncwarp();
        if (lane == 0) {
            __threadfence_block();
            const uint32_t old = atomicAdd(&cnt[s], 1u);
            if (old == nwarps - 1) {
                cnt[s] = 0;
                if (L + nsl < total && *s_abort == 0) {
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    // nsl pairs ahead of (st, q, p), stepped with adds
                    uint32_t p2 = p + nsl;
                    uint64_t q2 = q, st2 = st;
                    while (p2 >= np) {
                        p2 -= np;
                        q2 += gridDim.x;
                        while (q2 >= a.ntiles) {
                            q2 -= a.ntiles;
                            ++st2;
                        }
                    }
                    issue_pair(L + nsl, s, p2, st2, q2);
                }
            }
        }
        if (++s == nsl) {
            s = 0;
            par ^= 1u;
        }
        if (++p == np) {
            p = 0;
            q += gridDim.x;
            while (q >= a.ntiles) {
                q -= a.ntiles;
                ++st;
            }
        }
    }
    // drain after an expired wait, as in apply_c64c_tab
    __syncthreads();
    if (t == 0 && *s_abort) {
        for (uint32_t k = 0; k < nsl; ++k)
            if (s_iss[k] != 0) mbar_wait_bounded(&full[k], (s_iss[k] - 1u) & 1u, kWaitLimitNs);
    }
}

template <int AMPS>
static size_t tab_smem_bytes(const ApplyArgs &a, int threads) {
    const uint32_t tile_bytes = (1u << a.b) * 8u;
    const uint32_t tabn = a.nsub < kTabCap ? a.nsub : kTabCap;
    return (size_t)kTabStages * tile_bytes + (size_t)tabn * 16u * kTabEnt +
           (size_t)AMPS * threads * 8u + kTabBarBytes +
           (size_t)kTabCap * sizeof(uint4) + (2u * (size_t)kTabCap + 3u) * 4u + 8u +
           (a.nblocks <= kTabBhiCap ? (size_t)a.nblocks * 8u : 0u);
}

// shared memory of the paired kernel with nsl ring slots (exact sizes of the
// table, descriptors and lists of this plan)
static size_t pair_smem_bytes(const ApplyArgs &a, uint32_t nsl) {
    const size_t tile_bytes = ((size_t)1 << a.b) * 8u;
    return (size_t)nsl * 2u * tile_bytes + (size_t)a.nsub * 16u * kTabEnt + kPairBarBytes +
           (size_t)a.nsub * sizeof(uint4) + ((size_t)a.nruns + 1 + a.npairs + 1) * 4u + 8u +
           (size_t)a.nblocks * 8u;
}

template <int AMPS, bool WIDE>
static cudaError_t launch_c64c_tab(const ApplyArgs &a_in, int threads, int nsm, cudaStream_t st) {
    ApplyArgs a = a_in;
    size_t smem = tab_smem_bytes<AMPS>(a, threads);
    // one chunk (operators of up to 512 sub-groups): no chunk bookkeeping;
    // with a pair plan, partner blocks two at a time, in a ring of three
    // slots when the plan's tables leave room for it, else two
    auto kern = a.nchunks > 1 ? apply_c64c_tab<AMPS, WIDE, true> : apply_c64c_tab<AMPS, WIDE, false>;
    if constexpr (AMPS == 8)
        if (a.npairs > 0 && a.nchunks <= 1) {
            kern = apply_c64c_pair<AMPS, WIDE>;
            a.pair_slots = pair_smem_bytes(a, kMaxPairSlots) <= kMaxSmemPerBlock ? kMaxPairSlots : 2u;
            smem = pair_smem_bytes(a, a.pair_slots);
        }
    cudaError_t e = ensure_dyn_smem(reinterpret_cast<const void *>(kern), smem);
    if (e != cudaSuccess) return e;
    uint64_t grid = a.nitems < (uint64_t)nsm ? a.nitems : (uint64_t)nsm;
    if (grid == 0) return cudaSuccess;
    kern<<<(unsigned)grid, threads, smem, st>>>(a);
    count_launch();
    return cudaGetLastError();
}

template <int AMPS>
static cudaError_t launch_c64c(const ApplyArgs &a, int threads, int nsm, cudaStream_t st) {
    // shared memory: partner ring, one table chunk, low parts, run lists
    if (tab_smem_bytes<AMPS>(a, threads) > kMaxSmemPerBlock) return cudaErrorInvalidValue;
    if (a.n > 32 || a.wide) return launch_c64c_tab<AMPS, true>(a, threads, nsm, st);
    return launch_c64c_tab<AMPS, false>(a, threads, nsm, st);
}

// ---------------------------------------------------------------- batched c64c
// Many operators (different n, term counts and state counts) in ONE
// persistent launch over a host-built work list of (operator, state, tile)
// items, with the inner loop of apply_c64c_tab: per output tile the
// operator's per-tile factor table is built in shared memory -- one chunk of
// at most kTabCap sub-groups at a time, its thread descriptors and run lists
// staged beside it -- partner tiles stream through the TMA ring, and each
// run of sub-groups with equal key is one dispatch.  512 threads x 8
// amplitudes; an operator with n < 12 has tiles of 2^n amplitudes, held by
// threads t < tact and register indices m < mcount (the other lanes compute
// on in-bounds shared memory and store nothing).  Every warp passes the
// barrier at an item's start, so the item and its operator -- and the CTA's
// next item -- are copied into shared memory there: the steady state reads
// them with shared loads, and the lane that releases a stage finds the tile
// it loads next, kTabStages steps ahead, by arithmetic on those copies (a
// walk of the work list in global memory only when the lookahead crosses
// more than one item).
__global__ void __launch_bounds__(kC64Threads, 1) apply_c64c_batch(const BatchArgs a) {
    constexpr int AMPS = 8;
    constexpr uint32_t kStageBytes = 4096u * 8u;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const uint32_t threads = blockDim.x;
    const uint32_t nwarps = threads >> 5;
    const uint32_t t = threadIdx.x;
    const uint32_t lane = t & 31;
    const uint32_t t8 = t << 3;
    float4 *s_tab = reinterpret_cast<float4 *>(smem_raw + (size_t)kTabStages * kStageBytes);
    float2 *s_lo = reinterpret_cast<float2 *>(s_tab + kTabEnt * (size_t)kTabCap);
    uint64_t *full = reinterpret_cast<uint64_t *>(s_lo + (size_t)AMPS * threads);
    uint32_t *cnt = reinterpret_cast<uint32_t *>(full + kTabStages);
    volatile uint32_t *s_abort = cnt + kTabStages;
    uint32_t *s_iss = cnt + kTabStages + 1;  // copies issued per stage (drain)
    uint4 *s_td = reinterpret_cast<uint4 *>(reinterpret_cast<unsigned char *>(s_lo) +
                                            (size_t)AMPS * threads * 8u + kTabBarBytes);
    uint32_t *s_run = reinterpret_cast<uint32_t *>(s_td + kTabCap);
    uint32_t *s_blk = s_run + kTabCap + 1;
    const uint32_t stride = gridDim.x;
    if (blockIdx.x >= a.nitems) return;
    // [0]: the current item and its operator, [1]: the CTA's next item
    __shared__ BatchOp s_op[2];
    __shared__ BatchItem s_it[2];
    __shared__ const float2 *s_src[2];

    // step cursor (work-list index, block of that item's operator) -> next step
    auto advance = [&](uint32_t &ik, uint32_t &j) {
        if (++j == a.ops[a.items[ik].op].nblocks) {
            j = 0;
            ik += stride;
        }
    };
    auto issue = [&](uint32_t ik, uint32_t j, uint32_t s) {
        const BatchItem it = a.items[ik];
        const BatchOp &o = a.ops[it.op];
        const uint32_t bytes = (1u << o.b) * 8u;
        const float2 *src =
            a.psi[it.op] + (uint64_t)it.state * o.N + (((uint64_t)it.tile ^ o.blk_hi[j]) << o.b);
        ++s_iss[s];
        mbar_expect_tx(&full[s], bytes);
        bulk_g2s(smem_raw + (size_t)s * kStageBytes, src, bytes, &full[s]);
    };
    if (t == 0) {
        for (int s = 0; s < kTabStages; ++s) {
            mbar_init(&full[s], 1);
            cnt[s] = 0;
            s_iss[s] = 0;
        }
        *s_abort = 0;
        mbar_fence_init();
        uint32_t ik = blockIdx.x, j = 0;
        for (uint32_t s = 0; s < (uint32_t)kTabStages && ik < a.nitems; ++s) {
            issue(ik, j, s);
            advance(ik, j);
        }
    }
    __syncthreads();

    float2 A[AMPS], B[AMPS], hi[AMPS];
    float2 *mylo = s_lo + t;
    uint32_t ik = blockIdx.x, j = 0, s = 0, par = 0;
    uint32_t cidx = 0, cj0 = 0, next_j = 0;  // table chunk, its first block, the next's
    const BatchOp &o = s_op[0];
    const BatchItem &it = s_it[0];
    // the current item's scalars, kept in registers from its first chunk on:
    // tile, block count, x = 0 block, tile bits | threads used << 8 |
    // amplitudes used << 20
    uint64_t q = 0;
    uint32_t nb = 1, geo = 0;
    int dblk = -1;
    while (ik < a.nitems) {
        if (j == 0) {
#pragma unroll
            for (int m = 0; m < AMPS; ++m) {
                A[m] = B[m] = hi[m] = make_float2(0.f, 0.f);
                mylo[m * threads] = make_float2(0.f, 0.f);
            }
            cidx = 0;
            // every warp is done with the last item (its releases included)
            __syncthreads();
            if (t < 2) {
                const uint32_t ikx = ik + t * stride;
                if (ikx < a.nitems) {
                    const BatchItem itx = a.items[ikx];
                    s_it[t] = itx;
                    s_op[t] = a.ops[itx.op];
                    s_src[t] = a.psi[itx.op] + (uint64_t)itx.state * a.ops[itx.op].N;
                }
            }
        }
        if (j == 0 || j == next_j) {
            // table, descriptors and run lists of the chunk starting at block
            // j of this item's operator: every warp is done with the last one
            if (j != 0) ++cidx;
            __syncthreads();
            const uint4 c0 = o.chunks[cidx], c1 = o.chunks[cidx + 1];
            cj0 = c0.z;
            next_j = c1.z;
            for (uint32_t i = t; i < c1.x - c0.x; i += threads) s_td[i] = o.tdesc[c0.x + i];
            for (uint32_t i = t; i <= c1.y - c0.y; i += threads) {
                const uint32_t r = c0.y + i;
                s_run[i] = (o.run_g0[r] - c0.x) | (r < o.nruns ? o.run_key[r] << 16 : 0u);
            }
            for (uint32_t i = t; i <= c1.z - c0.z; i += threads) s_blk[i] = o.blk_r0[c0.z + i] - c0.y;
            const uint64_t qt = it.tile;
            for (uint32_t gi = t; gi < c1.x - c0.x; gi += threads) {
                const TileDataC64 &d = o.tdata[c0.x + gi];
                const uint32_t uq = parity<false>(qt, d.b0h) | (parity<false>(qt, d.b1h) << 1);
                const float sq = parity<false>(qt, d.z0h) ? -1.f : 1.f;
#pragma unroll
                for (uint32_t u = 0; u < 4; ++u) {
                    const float2 v = d.T[u ^ uq];
                    s_tab[gi * 4 + u] = make_float4(sq * v.x, sq * v.x, sq * v.y, sq * v.y);
                }
            }
            q = qt;
            nb = o.nblocks;
            dblk = o.diag_block;
            geo = (uint32_t)o.b | ((uint32_t)o.tact << 8) | ((uint32_t)o.mcount << 20);
            __syncthreads();
        }
        const uint32_t ob = geo & 0xffu, tact = (geo >> 8) & 0xfffu, mcount = geo >> 20;
        // an expired wait sets the abort flag; from then on every warp skips
        // waits and work but still reaches each chunk barrier
        bool skip = *s_abort != 0;
        if (!skip && !mbar_wait_bounded(&full[s], par, a.wait_ns)) {
            if (lane == 0) {
                atomicExch(a.err, kErrMbarTimeout);
                *s_abort = 1;
            }
            skip = true;
        }
        skip = __any_sync(0xffffffffu, skip);
        const uint32_t soff = s * kStageBytes;

        if (!skip && (int)j == dblk && o.diag != nullptr) {
            const float2 *dg = o.diag + (q << ob);
#pragma unroll
            for (int m = 0; m < AMPS; ++m) {
                if (t < tact && (uint32_t)m < mcount) {
                    const uint32_t rl = t + tact * (uint32_t)m;
                    const float2 d = dg[rl];
                    const float2 p = *reinterpret_cast<const float2 *>(smem_raw + soff + rl * 8u);
                    A[m] = __ffma2_rn(make_float2(d.x, d.x), p, A[m]);
                    B[m] = __ffma2_rn(make_float2(d.y, d.y), p, B[m]);
                }
            }
        }

        const uint32_t jl = j - cj0;
        const uint32_t r1 = skip ? 0u : s_blk[jl + 1];
        uint32_t rw = s_run[s_blk[jl]];
        for (uint32_t r = s_blk[jl]; r < r1; ++r) {
            const uint32_t rn = s_run[r + 1];
            run_tab_dispatch<AMPS>(rw >> 16, A, B, smem_raw, soff, s_tab, s_td, rw & 0xffffu,
                                   rn & 0xffffu, t, t8);
            rw = rn;
        }

        const bool last = (j == nb - 1);
        if (last || (j % kFlush) == kFlush - 1) {
#pragma unroll
            for (int m = 0; m < AMPS; ++m) {
                const float2 yv =
                    make_float2(__fsub_rn(A[m].x, B[m].y), __fadd_rn(A[m].y, B[m].x));
                float2 lm = mylo[m * threads];
                two_sum_into2(hi[m], lm, yv);
                mylo[m * threads] = lm;
                A[m] = B[m] = make_float2(0.f, 0.f);
            }
        }
        if (last && t < tact) {
            float2 *yo = a.y[it.op] + (uint64_t)it.state * o.N + (q << ob);
#pragma unroll
            for (int m = 0; m < AMPS; ++m) {
                if ((uint32_t)m < mcount) {
                    const float2 lm = mylo[m * threads];
                    yo[t + tact * (uint32_t)m] =
                        make_float2(__fadd_rn(hi[m].x, lm.x), __fadd_rn(hi[m].y, lm.y));
                }
            }
        }

        __syncwarp();
        if (lane == 0) {
            __threadfence_block();
            const uint32_t old = atomicAdd(&cnt[s], 1u);
            if (old == nwarps - 1) {
                cnt[s] = 0;
                if (*s_abort == 0) {
                    // the step kTabStages ahead: in this item, in the next
                    // one (shared copies), or further (walk the list)
                    uint32_t jf = j + (uint32_t)kTabStages;
                    int which = 0;
                    if (jf >= nb) {
                        jf -= nb;
                        which = (ik + stride < a.nitems && jf < s_op[1].nblocks) ? 1 : -1;
                    }
                    if (which >= 0) {
                        const BatchOp &fo = s_op[which];
                        const uint32_t bytes = (1u << fo.b) * 8u;
                        const float2 *src =
                            s_src[which] + (((uint64_t)s_it[which].tile ^ fo.blk_hi[jf]) << fo.b);
                        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                        ++s_iss[s];
                        mbar_expect_tx(&full[s], bytes);
                        bulk_g2s(smem_raw + (size_t)s * kStageBytes, src, bytes, &full[s]);
                    } else {
                        uint32_t ik2 = ik, j2 = j;
                        for (int k = 0; k < kTabStages && ik2 < a.nitems; ++k) advance(ik2, j2);
                        if (ik2 < a.nitems) {
                            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                            issue(ik2, j2, s);
                        }
                    }
                }
            }
        }
        if (++s == (uint32_t)kTabStages) {
            s = 0;
            par ^= 1u;
        }
        if (++j == nb) {  // the item's block count (register): no load per step
            j = 0;
            ik += stride;
        }
    }
    // drain after an expired wait, as in apply_c64c_tab
    __syncthreads();
    if (t == 0 && *s_abort) {
        for (int k = 0; k < kTabStages; ++k)
            if (s_iss[k] != 0) mbar_wait_bounded(&full[k], (s_iss[k] - 1u) & 1u, kWaitLimitNs);
    }
}

cudaError_t launch_batch_c64c(const BatchArgs &a, int nsm, cudaStream_t st) {
    constexpr int AMPS = 8;
    const size_t smem = (size_t)kTabStages * 4096u * 8u + (size_t)kTabCap * 16u * kTabEnt +
                        (size_t)AMPS * kC64Threads * 8u + kTabBarBytes +
                        (size_t)kTabCap * sizeof(uint4) + (2u * (size_t)kTabCap + 3u) * 4u;
    if (smem > kMaxSmemPerBlock) return cudaErrorInvalidValue;
    cudaError_t e = ensure_dyn_smem(reinterpret_cast<const void *>(apply_c64c_batch), smem);
    if (e != cudaSuccess) return e;
    const uint32_t grid = a.nitems < (uint32_t)nsm ? a.nitems : (uint32_t)nsm;
    if (grid == 0) return cudaSuccess;
    apply_c64c_batch<<<grid, kC64Threads, smem, st>>>(a);
    count_launch();
    return cudaGetLastError();
}

template <int AMPS>
static cudaError_t launch_one(const ApplyArgs &a, int threads, int nsm, cudaStream_t st) {
    const uint32_t tile_bytes = (1u << a.b) * (uint32_t)sizeof(Cplx<double>);
    int stages = (int)((200u * 1024u) / tile_bytes);
    if (stages > kMaxStages) stages = kMaxStages;
    if (stages < 2) stages = 2;
    // stages, then full barriers, stage counters, the abort flag and issue counts
    const size_t smem = (size_t)stages * tile_bytes + kMaxStages * (sizeof(uint64_t) + 8u) + 8u;
    auto kern = apply_c128<AMPS>;
    cudaError_t e = ensure_dyn_smem(reinterpret_cast<const void *>(kern), smem);
    if (e != cudaSuccess) return e;
    uint64_t grid = a.nitems < (uint64_t)nsm ? a.nitems : (uint64_t)nsm;
    if (grid == 0) return cudaSuccess;
    kern<<<(unsigned)grid, threads, smem, st>>>(a, stages);
    count_launch();
    return cudaGetLastError();
}

static cudaError_t dispatch_amps(const ApplyArgs &a, int amps, int threads, int nsm,
                                 cudaStream_t st) {
    switch (amps) {
        case 1: return launch_one<1>(a, threads, nsm, st);
        case 2: return launch_one<2>(a, threads, nsm, st);
        case 4: return launch_one<4>(a, threads, nsm, st);
        case 8: return launch_one<8>(a, threads, nsm, st);
        case 16: return launch_one<16>(a, threads, nsm, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_apply(int dtype, const ApplyArgs &a, int amps, int threads, int nsm,
                         cudaStream_t st) {
    if (dtype == 0) return dispatch_amps(a, amps, threads, nsm, st);
    if (amps >= 2 && a.tb != kTb) return cudaErrorInvalidValue;
    switch (amps) {
        case 1: return launch_c64c<1>(a, threads, nsm, st);
        case 2: return launch_c64c<2>(a, threads, nsm, st);
        case 4: return launch_c64c<4>(a, threads, nsm, st);
        case 8: return launch_c64c<8>(a, threads, nsm, st);
        default: return cudaErrorInvalidValue;
    }
}

// ---------------------------------------------------------------- diagonal
// D0[r] = sum_k c'_k (-1)^popc(r & z_k) over the x = 0 group, in FP64: per
// tile of 2^db amplitudes, fold the tile-index bits of z_k into a sign, sum
// each distinct low-bit pattern z_k & (2^db - 1) into a bin (terms of a bin
// in input order), then an in-place Walsh-Hadamard transform over db bits.
__global__ void __launch_bounds__(256) diag_wht(int db, uint64_t ntiles, const uint64_t *bin_zlo,
                                                const uint32_t *bin_off, uint32_t nbins,
                                                const uint64_t *tz, const double *tc, void *out,
                                                int out_f32) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    double2 *W = reinterpret_cast<double2 *>(smem_raw);
    const uint32_t sz = 1u << db;
    for (uint64_t q = blockIdx.x; q < ntiles; q += gridDim.x) {
        for (uint32_t i = threadIdx.x; i < sz; i += blockDim.x) W[i] = make_double2(0.0, 0.0);
        __syncthreads();
        const uint64_t qhi = q << db;
        for (uint32_t bi = threadIdx.x; bi < nbins; bi += blockDim.x) {
            double wr = 0.0, wi = 0.0;
            for (uint32_t k = bin_off[bi]; k < bin_off[bi + 1]; ++k) {
                const bool neg = (__popcll(qhi & tz[k]) & 1) != 0;
                const double cr = tc[2 * k], ci = tc[2 * k + 1];
                if (k == bin_off[bi]) {
                    wr = neg ? -cr : cr;
                    wi = neg ? -ci : ci;
                } else {
                    wr = neg ? wr - cr : wr + cr;
                    wi = neg ? wi - ci : wi + ci;
                }
            }
            W[bin_zlo[bi]] = make_double2(wr, wi);
        }
        __syncthreads();
        for (int l = 0; l < db; ++l) {
            const uint32_t h = 1u << l;
            for (uint32_t i = threadIdx.x; i < sz / 2; i += blockDim.x) {
                const uint32_t ia = ((i >> l) << (l + 1)) | (i & (h - 1));
                const uint32_t ib = ia | h;
                const double2 u = W[ia], v = W[ib];
                W[ia] = make_double2(u.x + v.x, u.y + v.y);
                W[ib] = make_double2(u.x - v.x, u.y - v.y);
            }
            __syncthreads();
        }
        if (out_f32) {
            float2 *o = static_cast<float2 *>(out) + qhi;
            for (uint32_t i = threadIdx.x; i < sz; i += blockDim.x)
                o[i] = make_float2((float)W[i].x, (float)W[i].y);
        } else {
            double2 *o = static_cast<double2 *>(out) + qhi;
            for (uint32_t i = threadIdx.x; i < sz; i += blockDim.x) o[i] = W[i];
        }
        __syncthreads();
    }
}

cudaError_t launch_diag(int dtype, int n, int db, uint64_t ntiles, const uint64_t *bin_zlo,
                        const uint32_t *bin_off, uint32_t nbins, const uint64_t *tz,
                        const double *tc, void *out, cudaStream_t st) {
    (void)n;
    const size_t smem = ((size_t)1 << db) * sizeof(double2);
    cudaError_t e = ensure_dyn_smem(reinterpret_cast<const void *>(diag_wht), smem);
    if (e != cudaSuccess) return e;
    const unsigned grid = (unsigned)(ntiles < 4096 ? ntiles : 4096);
    diag_wht<<<grid, 256, smem, st>>>(db, ntiles, bin_zlo, bin_off, nbins, tz, tc, out,
                                      dtype == 1);
    count_launch();
    return cudaGetLastError();
}

}  // namespace qr
