// qr_csr.cu -- CSR assembly of a Pauli sum and CSR * vector on sm_103a.
//
// csr_fill replaces qrusty's rowwise builder (qrusty/src/accel.rs:171-210
// make_row, :267-336 make_unsafe_vectors_chunked).  Row r of the matrix has
// exactly G entries, one per distinct x mask: column r ^ x_g, value the sum
// of +-c'_k over the terms of group g in input order (a left fold starting
// from the first term, as make_row's fold does), explicit zeros kept.
//
// Column order without sorting: with the groups' x masks sorted ascending,
// the rank of r ^ x_g among {r ^ x_h} is
//     pos_r(g) = g + sum_{b : bit b of r set} sigma_{g,b},
// where sigma_{g,b} = +S (x_g has 0 at b) or -S (x_g has 1 at b) and S is
// the size of g's sibling subtree at bit b of the binary trie of the x
// masks (nonzero only at the trie's branching bits).  The host precomputes
// the (b, sigma) lists; each thread places one (row, group) entry directly.
//
// Values without a per-row fold: a group's value in row r depends on r only
// through the parities of r against the group's z masks, i.e. against z0 and
// a GF(2) basis beta_1..beta_d of the differences z_k ^ z0.  For d <= 4 the
// host folds the group's +-c'_k in input order once per class (2^(d+1)
// classes) -- the same additions in the same order as make_row, hence the
// same bits -- and the kernel reads the row's class from that table.
#include "qr_common.cuh"

namespace qr {

__global__ void __launch_bounds__(256) csr_indptr_kernel(uint64_t N, uint64_t G,
                                                         uint64_t *indptr) {
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r <= N;
         r += (uint64_t)gridDim.x * blockDim.x)
        indptr[r] = r * G;
}

// Row bits as a 32-bit word when n <= 32 (half the integer work), else 64.
template <bool WIDE> struct RowT { using T = uint32_t; };
template <> struct RowT<true> { using T = uint64_t; };

template <typename W>
__device__ __forceinline__ uint32_t parity(W v) {
    if constexpr (sizeof(W) == 8) return (uint32_t)__popcll(v) & 1u;
    else return (uint32_t)__popc(v) & 1u;
}
template <typename W>
__device__ __forceinline__ int lowbit(W v) {
    if constexpr (sizeof(W) == 8) return __ffsll((long long)v) - 1;
    else return __ffs((int)v) - 1;
}

// sum of sigma_b over the set bits b of m (sig: the group's row of the table)
template <typename W>
__device__ __forceinline__ int32_t sigma_sum(W m, const int32_t *sig) {
    int32_t s = 0;
    for (; m; m &= m - 1) s += sig[lowbit(m)];
    return s;
}

__device__ __forceinline__ void csr_store(const CsrArgs &a, uint64_t rr, int32_t pos, uint64_t col,
                                          double2 v) {
    if (pos < 0 || (uint64_t)pos >= a.G) {  // cannot happen for a valid trie table
        atomicExch(a.err, kErrCsrPos);
        return;
    }
    const uint64_t o = rr * a.G + (uint64_t)pos;
    a.indices[o] = col;
    reinterpret_cast<double2 *>(a.data)[o] = v;
}

// Class of row r for group d: bit 0 = parity(r & z0), bit j+1 = parity(r & beta_j).
template <typename W>
__device__ __forceinline__ uint32_t csr_class(const CsrGroup &d, W r) {
    uint32_t c = parity<W>(r & (W)d.z0);
#pragma unroll
    for (int j = 0; j < kCsrMaxRank; ++j)
        if ((uint32_t)j < d.d) c |= parity<W>(r & (W)d.beta[j]) << (j + 1);
    return c;
}

constexpr int kCsrThreads = 256;
constexpr uint32_t kCsrSmemSig = 12288;  // sigma entries staged in shared memory (48 KB)
constexpr size_t kCsrLutBytes = 16u * 1024u;
constexpr uint32_t kCsrSmemCtab = 2048;  // class-table entries staged in shared memory (32 KB)

// Low-bit width of the per-group position lookup table: G x (2^L + 1)
// 32-bit entries (rows padded by one word so lanes on consecutive groups hit
// distinct banks) within 16 KB, so that with the staging buffers four
// 256-thread blocks fit an SM's 228 KB.  L <= 8, so 256-row launches stay aligned.
__host__ __device__ inline int csr_lut_bits(uint32_t G) {
    int L = 8;
    while (L > 1 && (size_t)G * ((1u << L) + 1) * 4u > kCsrLutBytes) --L;
    return L;
}

// Class-table groups.  G <= 256: blocks take chunks of 2^L rows; in a chunk,
// thread t owns group g = t % G of rows t / G, t / G + 256 / G, ..., so its
// descriptor and position mask stay in registers; the position terms of the
// row bits above the chunk are summed once per chunk and the low L bits come
// from a shared-memory table built per block.  G > 256: one row per pass,
// threads stride the groups.  Fold-mode groups are left to csr_fold_kernel,
// so no lane of a warp waits on another's long fold.
template <bool WIDE>
__global__ void __launch_bounds__(kCsrThreads) csr_fill_kernel(const CsrArgs a) {
    using W = typename RowT<WIDE>::T;
    extern __shared__ int32_t s_dyn[];
    const uint32_t G = (uint32_t)a.G;
    if (G <= (uint32_t)kCsrThreads) {
        const int L = csr_lut_bits(G);
        const uint32_t lsz = (1u << L) + 1;  // padded row
        for (uint32_t i = threadIdx.x; i < G * lsz; i += kCsrThreads) {
            const uint32_t g = i / lsz, v = i - g * lsz;
            const W pm = (W)a.pmask[g] & (((W)1 << L) - 1) & (W)v;
            s_dyn[i] = v < (1u << L) ? sigma_sum<W>(pm, a.sig + (size_t)g * (uint32_t)a.n) : 0;
        }
        // class tables next to the position table when they fit
        double2 *s_ctab = reinterpret_cast<double2 *>(s_dyn + ((G * lsz + 3u) & ~3u));
        const bool ctab_smem = a.nctab <= kCsrSmemCtab;
        if (ctab_smem)
            for (uint32_t i = threadIdx.x; i < a.nctab; i += kCsrThreads) s_ctab[i] = a.ctab[i];
        __syncthreads();
        const uint32_t rpp = kCsrThreads / G;
        const uint32_t t = threadIdx.x;
        if (t >= rpp * G) return;  // no barrier follows
        const uint32_t rs = t / G, g = t - rs * G;
        const CsrGroup d = a.grp[g];
        if (d.d == kCsrFold) return;
        const W xg = (W)a.gx[g], pm = (W)a.pmask[g];
        const W lomask = ((W)1 << L) - 1;
        const int32_t *sg = a.sig + (size_t)g * (uint32_t)a.n;
        const int32_t *lut = s_dyn + g * lsz;
        const uint64_t nchunk = (a.nrows + lomask) >> L;
        // the class table is read through a pointer of known state space
        // (shared or global), so the loads are LDS / LDG, not generic
        auto rows = [&](const double2 *tab) {
            for (uint64_t ch = blockIdx.x; ch < nchunk; ch += gridDim.x) {
                const uint64_t rr0 = ch << L;
                const W base = (W)(a.row0 + rr0);
                const int32_t phi = (int32_t)g + sigma_sum<W>(base & pm & ~lomask, sg);
                const uint64_t rend = min(rr0 + ((uint64_t)1 << L), a.nrows);
                // two rows per step: their table reads are in flight together
                for (uint64_t rr = rr0 + rs; rr < rend; rr += 2 * (uint64_t)rpp) {
                    const uint64_t rr2 = rr + rpp;
                    const W r = (W)(a.row0 + rr), r2 = (W)(a.row0 + rr2);
                    const bool two = rr2 < rend;
                    const double2 v1 = tab[csr_class<W>(d, r)];
                    const double2 v2 = two ? tab[csr_class<W>(d, r2)] : v1;
                    csr_store(a, rr, phi + lut[(uint32_t)(r & lomask)], (uint64_t)(r ^ xg), v1);
                    if (two)
                        csr_store(a, rr2, phi + lut[(uint32_t)(r2 & lomask)], (uint64_t)(r2 ^ xg),
                                  v2);
                }
            }
        };
        if (ctab_smem) rows(s_ctab + d.tab);
        else rows(a.ctab + d.tab);
    } else {
        const uint64_t nsig = (uint64_t)G * (uint32_t)a.n;
        const bool staged = nsig <= kCsrSmemSig;
        if (staged)
            for (uint32_t i = threadIdx.x; i < nsig; i += kCsrThreads) s_dyn[i] = a.sig[i];
        __syncthreads();
        const int32_t *sig = staged ? s_dyn : a.sig;
        for (uint64_t rr = blockIdx.x; rr < a.nrows; rr += gridDim.x) {
            const W r = (W)(a.row0 + rr);
            for (uint32_t g = threadIdx.x; g < G; g += kCsrThreads) {
                const CsrGroup d = a.grp[g];
                if (d.d == kCsrFold) continue;
                const int32_t pos = (int32_t)g + sigma_sum<W>(r & (W)a.pmask[g],
                                                              sig + (size_t)g * (uint32_t)a.n);
                csr_store(a, rr, pos, (uint64_t)(r ^ (W)a.gx[g]),
                          a.ctab[d.tab + csr_class<W>(d, r)]);
            }
        }
    }
}

// Fold-mode groups (z span wider than kCsrMaxRank): one thread per row, all
// lanes of a warp on the same group, the group's +-c'_k folded in input-term
// order from the first term (make_row's fold), terms read warp-uniformly.
// The leading terms up to z-span rank kCsrPrefixRank come from the host's
// per-class fold of them (same additions, same order); the rest are added
// per row.  A part (re or im) whose every coefficient is +-0 takes no FP64
// additions: under round-to-nearest a sum of signed zeros is -0 exactly when
// every addend is -0, so the fold's result is -0 iff each +-c'_k part is -0.
template <bool RZ, bool IZ>
__device__ __forceinline__ double2 csr_fold_row(const CsrArgs &a, uint64_t r, const CsrGroup &d,
                                                uint32_t f) {
    const uint64_t *tz = a.tz;
    const double *tc = a.tc;
    double vr = 0.0, vi = 0.0;
    uint32_t nr = 1u, ni = 1u;  // every addend so far -0 (zero parts)
    uint32_t k = d.k0;
    const uint32_t m = d.pre & 0xffffffu;
    if (m != 0) {
        // the fold of the leading m terms, looked up by the row's sign class
        const uint32_t dp = d.pre >> 24;
        const uint64_t *pb = a.pbeta + (size_t)f * kCsrPrefixRank;
        uint32_t c = (uint32_t)__popcll(r & d.z0) & 1u;
        for (uint32_t j = 0; j < dp; ++j) c |= ((uint32_t)__popcll(r & pb[j]) & 1u) << (j + 1);
        const double2 v = a.ptab[d.tab + c];
        vr = v.x;
        vi = v.y;
        nr = (uint32_t)signbit(v.x);
        ni = (uint32_t)signbit(v.y);
        k += m;
    }
    for (; k < d.k1; ++k) {
        // sign applied to the bit pattern: no floating-point negation
        const uint64_t sb = (uint64_t)(__popcll(r & tz[k]) & 1) << 63;
        if constexpr (RZ) {
            nr &= (uint32_t)(sb >> 63) ^ (uint32_t)signbit(tc[2 * k]);
        } else {
            const double cr = __longlong_as_double(__double_as_longlong(tc[2 * k]) ^ (long long)sb);
            vr = k == d.k0 ? cr : __dadd_rn(vr, cr);
        }
        if constexpr (IZ) {
            ni &= (uint32_t)(sb >> 63) ^ (uint32_t)signbit(tc[2 * k + 1]);
        } else {
            const double ci =
                __longlong_as_double(__double_as_longlong(tc[2 * k + 1]) ^ (long long)sb);
            vi = k == d.k0 ? ci : __dadd_rn(vi, ci);
        }
    }
    if constexpr (RZ) vr = nr ? -0.0 : 0.0;
    if constexpr (IZ) vi = ni ? -0.0 : 0.0;
    return make_double2(vr, vi);
}

// ------------------------------------------------------------ staged fill
// Rows are assembled in shared memory and leave the SM as contiguous TMA
// bulk stores (cp.async.bulk shared -> global): a warp's entries of one row
// land at permuted positions, which as direct global stores become many
// partial-line L2 writes.  Two staging buffers of R rows (R a power of two
// dividing the 2^L-row chunk) alternate, so the bulk store of one overlaps
// the assembly of the next.  Fold-mode groups (per-row FP64 folds) are
// computed first by csr_fold_kernel<true> into a row-major value buffer and
// copied into the stage here: folded inside the staged pass, their serial
// chains would hold every warp of the block at the sub-chunk barrier, and
// stored in place after it, each entry becomes a DRAM read-modify-write of
// a line the bulk store has already evicted.  Without a value buffer the
// fold entries are left unset and stored afterwards by csr_fold_kernel<false>.
constexpr size_t kCsrStageBytes = 24u * 1024u;  // one buffer: R rows x G x (8 + 16) bytes
constexpr uint32_t kCsrFvSlots = 4;              // fold-value ring depth (sub-chunks)

__host__ __device__ inline int csr_stage_rows(uint32_t G, int L) {
    int R = 1 << L;
    while (R > 2 && (size_t)R * G * 24u > kCsrStageBytes) R >>= 1;
    return R;
}

__device__ __forceinline__ uint32_t csr_saddr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void csr_bulk_s2g(void *dst, const void *src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst),
                 "r"(csr_saddr(src)), "r"(bytes)
                 : "memory");
}

template <bool WIDE>
__global__ void __launch_bounds__(kCsrThreads) csr_fill_staged_kernel(const CsrArgs a) {
    using W = typename RowT<WIDE>::T;
    extern __shared__ __align__(128) int32_t s_dyn[];
    const uint32_t G = (uint32_t)a.G;
    const int L = csr_lut_bits(G);
    const uint32_t lsz = (1u << L) + 1;
    const uint32_t t = threadIdx.x;
    for (uint32_t i = t; i < G * lsz; i += kCsrThreads) {
        const uint32_t g = i / lsz, v = i - g * lsz;
        const W pm = (W)a.pmask[g] & (((W)1 << L) - 1) & (W)v;
        s_dyn[i] = v < (1u << L) ? sigma_sum<W>(pm, a.sig + (size_t)g * (uint32_t)a.n) : 0;
    }
    double2 *s_ctab = reinterpret_cast<double2 *>(s_dyn + ((G * lsz + 3u) & ~3u));
    const bool ctab_smem = a.nctab <= kCsrSmemCtab;
    if (ctab_smem)
        for (uint32_t i = t; i < a.nctab; i += kCsrThreads) s_ctab[i] = a.ctab[i];
    // staging buffers, 128-byte aligned: per buffer R*G indices then R*G values
    const uint32_t R = (uint32_t)csr_stage_rows(G, L);
    const uint32_t ent = R * G;
    const size_t head = ((size_t)((G * lsz + 3u) & ~3u) * 4u +
                         (ctab_smem ? (size_t)a.nctab * sizeof(double2) : 0u) + 127u) &
                        ~(size_t)127u;
    unsigned char *stage = reinterpret_cast<unsigned char *>(s_dyn) + head;
    const size_t buf_bytes = ((size_t)ent * 24u + 127u) & ~(size_t)127u;
    // with precomputed fold values: high-bit position term of each fold-mode
    // group for the current chunk
    int32_t *s_phi = reinterpret_cast<int32_t *>(stage + 2 * buf_bytes);
    const uint32_t nfv = a.fvals ? a.nfold : 0u;
    __syncthreads();

    const uint32_t rpp = kCsrThreads / G;
    const uint32_t rs = t / G, g = t - rs * G;
    const bool lane_on = t < rpp * G;  // idle threads still take every barrier
    CsrGroup d{};
    W xg = 0, pm = 0;
    const int32_t *sg = a.sig;
    bool active = false;
    if (lane_on) {
        d = a.grp[g];
        active = d.d != kCsrFold;
        xg = (W)a.gx[g];
        pm = (W)a.pmask[g];
        sg = a.sig + (size_t)g * (uint32_t)a.n;
    }
    const W lomask = ((W)1 << L) - 1;
    const int32_t *lut = s_dyn + (lane_on ? g : 0u) * lsz;
    const double2 *tab = (ctab_smem ? s_ctab : a.ctab) + d.tab;
    const uint64_t nchunk = (a.nrows + lomask) >> L;
    // fold-mode entries: with nfold * R <= threads, the highest nfold * R
    // threads (idle in the class-table pass whenever rpp * G < threads) own
    // one item (f, rl) of every sub-chunk each and copy its value into a
    // kCsrFvSlots-deep shared ring, kCsrFvSlots - 1 sub-chunks ahead
    // (cp.async: no register waits on the load; the values come from DRAM,
    // the fill's write stream having evicted them from L2)
    const bool ring = nfv > 0 && nfv * R <= (uint32_t)kCsrThreads;
    const uint32_t base_it = ring ? (uint32_t)kCsrThreads - nfv * R : (uint32_t)kCsrThreads;
    const bool own = ring && t >= base_it;
    const uint32_t i_it = own ? t - base_it : 0u;
    const uint32_t f_it = i_it / R, rl_it = i_it - (i_it / R) * R;
    const uint32_t g_it = own ? a.fold[f_it] : 0u;
    const uint64_t x_it = own ? a.gx[g_it] : 0ull;
    double2 *s_fv = reinterpret_cast<double2 *>(s_phi + ((nfv + 3u) & ~3u));  // slots x nfold*R
    auto next_sub = [&](uint64_t &c, uint64_t &s0) {
        const uint64_t e = min((c << L) + ((uint64_t)1 << L), a.nrows);
        s0 += R;
        if (s0 >= e) {
            c += gridDim.x;
            s0 = c << L;
        }
    };
    auto prefetch = [&](uint64_t c, uint64_t s0, uint32_t slot) {
        if (own && c < nchunk) {
            const uint32_t rows = (uint32_t)min((uint64_t)R, min((c << L) + ((uint64_t)1 << L),
                                                                   a.nrows) - s0);
            if (rl_it < rows) {
                const double2 *src = a.fvals + (size_t)f_it * a.nrows + s0 + rl_it;
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                                 csr_saddr(s_fv + (size_t)slot * nfv * R + i_it)),
                             "l"(src)
                             : "memory");
            }
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    uint32_t k = 0;  // sub-chunks issued by this block: buffer k & 1, ring slot k % kCsrFvSlots
    uint64_t ch = blockIdx.x, sc = ch << L;
    uint64_t chP = ch, scP = sc;  // prefetch cursor: sub-chunk k + kCsrFvSlots - 1
    if (ring)
        for (uint32_t q = 0; q + 1 < kCsrFvSlots; ++q) {
            prefetch(chP, scP, q);
            next_sub(chP, scP);
        }
    int32_t phi = 0;
    while (ch < nchunk) {
        const uint64_t rr0 = ch << L;
        const uint64_t rend = min(rr0 + ((uint64_t)1 << L), a.nrows);
        const uint32_t rows = (uint32_t)min((uint64_t)R, rend - sc);
        unsigned char *buf = stage + (size_t)(k & 1u) * buf_bytes;
        uint64_t *s_idx = reinterpret_cast<uint64_t *>(buf);
        double2 *s_val = reinterpret_cast<double2 *>(buf + (size_t)ent * 8u);
        // the bulk store that last read this buffer (two sub-chunks ago) has
        // finished reading it
        if (t == 0) asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
        if (sc == rr0) {  // chunk start: high-bit position terms
            phi = active ? (int32_t)g + sigma_sum<W>((W)(a.row0 + rr0) & pm & ~lomask, sg) : 0;
            // (the previous sub-chunk's barrier has retired every reader of s_phi)
            for (uint32_t f = t; f < nfv; f += kCsrThreads) {
                const uint32_t gf = a.fold[f];
                s_phi[f] = (int32_t)gf + sigma_sum<W>((W)(a.row0 + rr0) & (W)a.pmask[gf] & ~lomask,
                                                      a.sig + (size_t)gf * (uint32_t)a.n);
            }
        }
        __syncthreads();
        if (ring) {
            prefetch(chP, scP, (k + kCsrFvSlots - 1) % kCsrFvSlots);
            next_sub(chP, scP);
        }
        if (active) {
#pragma unroll 2
            for (uint32_t rl = rs; rl < rows; rl += rpp) {
                const W r = (W)(a.row0 + sc + rl);
                const double2 v =
                    ctab_smem ? s_ctab[d.tab + csr_class<W>(d, r)] : tab[csr_class<W>(d, r)];
                const int32_t pos = phi + lut[(uint32_t)(r & lomask)];
                if (pos < 0 || (uint32_t)pos >= G) {  // cannot happen for a valid trie table
                    atomicExch(a.err, kErrCsrPos);
                    continue;
                }
                s_idx[rl * G + (uint32_t)pos] = (uint64_t)(r ^ xg);
                s_val[rl * G + (uint32_t)pos] = v;
            }
        }
        // fold-mode entries from the values the fold pass wrote
        auto place = [&](uint32_t f, uint32_t rl, uint32_t gf, uint64_t xf, double2 v) {
            const W r = (W)(a.row0 + sc + rl);
            const int32_t pos = s_phi[f] + s_dyn[gf * lsz + (uint32_t)(r & lomask)];
            if (pos < 0 || (uint32_t)pos >= G) {
                atomicExch(a.err, kErrCsrPos);
                return;
            }
            s_idx[rl * G + (uint32_t)pos] = (uint64_t)r ^ xf;
            s_val[rl * G + (uint32_t)pos] = v;
        };
        const uint32_t nitem = nfv * rows;
        if (ring) {
            // this thread's copy for sub-chunk k has landed (newer ones pending)
            asm volatile("cp.async.wait_group %0;" ::"n"(kCsrFvSlots - 1) : "memory");
            if (own && rl_it < rows)
                place(f_it, rl_it, g_it, x_it,
                      s_fv[(size_t)(k % kCsrFvSlots) * nfv * R + i_it]);
        } else {
            for (uint32_t i = t; i < nitem; i += kCsrThreads) {
                const uint32_t f = i / rows, rl = i - f * rows;
                const uint32_t gf = a.fold[f];
                place(f, rl, gf, a.gx[gf], a.fvals[(size_t)f * a.nrows + sc + rl]);
            }
        }
        // shared writes visible to the bulk-copy (async) proxy
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (t == 0) {
            csr_bulk_s2g(a.indices + sc * G, s_idx, rows * G * 8u);
            csr_bulk_s2g(a.data + 2 * sc * G, s_val, rows * G * 16u);
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        }
        next_sub(ch, sc);
        ++k;
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    if (t == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

// VALS: write the values row-major per fold group into a.fvals (coalesced),
// for the staged fill to place; otherwise store the entries in place.
template <bool VALS>
__global__ void __launch_bounds__(kCsrThreads) csr_fold_kernel(const CsrArgs a) {
    for (uint32_t f = blockIdx.y; f < a.nfold; f += gridDim.y) {
        const uint32_t g = a.fold[f];
        const CsrGroup d = a.grp[g];
        const uint64_t xg = a.gx[g], pm = a.pmask[g];
        const int32_t *sg = a.sig + (size_t)g * (uint32_t)a.n;
        for (uint64_t rr = blockIdx.x * (uint64_t)kCsrThreads + threadIdx.x; rr < a.nrows;
             rr += (uint64_t)gridDim.x * kCsrThreads) {
            const uint64_t r = a.row0 + rr;
            double2 v;
            switch (d.zparts & 3u) {  // warp-uniform
                case 1: v = csr_fold_row<true, false>(a, r, d, f); break;
                case 2: v = csr_fold_row<false, true>(a, r, d, f); break;
                case 3: v = csr_fold_row<true, true>(a, r, d, f); break;
                default: v = csr_fold_row<false, false>(a, r, d, f); break;
            }
            if constexpr (VALS)
                a.fvals[(size_t)f * a.nrows + rr] = v;
            else
                csr_store(a, rr, (int32_t)g + sigma_sum<uint64_t>(r & pm, sg), r ^ xg, v);
        }
    }
}

// fold-mode groups, after the fill kernel on the same stream
static cudaError_t launch_csr_fold(const CsrArgs &a, int nsm, cudaStream_t st) {
    if (a.nfold == 0) return cudaSuccess;
    uint64_t gx = (a.nrows + kCsrThreads - 1) / kCsrThreads;
    const uint32_t gy = a.nfold < 65535u ? a.nfold : 65535u;
    uint64_t cap = ((uint64_t)nsm * 8 + gy - 1) / gy;
    if (cap < 1) cap = 1;
    if (gx > cap) gx = cap;
    if (a.fvals)
        csr_fold_kernel<true><<<dim3((unsigned)gx, gy), kCsrThreads, 0, st>>>(a);
    else
        csr_fold_kernel<false><<<dim3((unsigned)gx, gy), kCsrThreads, 0, st>>>(a);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_csr_fill(const CsrArgs &a, int nsm, cudaStream_t st) {
    if (a.row0 == 0 && a.indptr != nullptr) {
        uint64_t g = (a.N + 1 + 255) / 256;
        if (g > (uint64_t)nsm * 8) g = (uint64_t)nsm * 8;
        csr_indptr_kernel<<<(unsigned)g, 256, 0, st>>>(a.N, a.G, a.indptr);
        count_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (a.nrows == 0 || a.G == 0) return cudaSuccess;
    size_t smem;
    uint64_t g;
    const bool aligned = ((uintptr_t)a.indices % 16u) == 0 && ((uintptr_t)a.data % 16u) == 0;
    if (a.G <= (uint64_t)kCsrThreads) {
        const int L = csr_lut_bits((uint32_t)a.G);
        g = (a.nrows + (1u << L) - 1) >> L;
        smem = (((size_t)a.G * ((1u << L) + 1) + 3u) & ~(size_t)3u) * sizeof(int32_t);
        if (a.nctab <= kCsrSmemCtab) smem += (size_t)a.nctab * sizeof(double2);
        // staged path: every bulk store a whole number of 16-byte units
        // (even row counts) from 16-byte aligned outputs
        if (aligned && L >= 1 && a.nrows % 2 == 0) {
            const uint32_t R = (uint32_t)csr_stage_rows((uint32_t)a.G, L);
            const size_t buf = ((size_t)R * a.G * 24u + 127u) & ~(size_t)127u;
            size_t sm = ((smem + 127u) & ~(size_t)127u) + 2 * buf;
            if (a.fvals && a.nfold > 0) {  // chunk positions, then the value ring
                sm += (((size_t)a.nfold + 3u) & ~(size_t)3u) * 4u;
                if ((size_t)a.nfold * R <= (size_t)kCsrThreads)
                    sm += (size_t)kCsrFvSlots * a.nfold * R * 16u;
            }
            auto kern = (a.n > 32 || a.wide) ? csr_fill_staged_kernel<true> : csr_fill_staged_kernel<false>;
            cudaError_t e0 =
                cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            if (e0 != cudaSuccess) return e0;
            int per_sm = 0;
            e0 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kCsrThreads, sm);
            if (e0 != cudaSuccess) return e0;
            if (per_sm < 1) per_sm = 1;
            if (g > (uint64_t)nsm * per_sm) g = (uint64_t)nsm * per_sm;
            if (a.fvals) {  // fold values first; the staged pass places them
                cudaError_t e = launch_csr_fold(a, nsm, st);
                if (e != cudaSuccess) return e;
            }
            kern<<<(unsigned)g, kCsrThreads, sm, st>>>(a);
            count_launch();
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess || a.fvals) return e;
            return launch_csr_fold(a, nsm, st);
        }
    } else {
        g = a.nrows;
        const uint64_t nsig = a.G * (uint64_t)a.n;
        smem = nsig <= kCsrSmemSig ? (size_t)nsig * sizeof(int32_t) : 0;
    }
    auto kern = (a.n > 32 || a.wide) ? csr_fill_kernel<true> : csr_fill_kernel<false>;
    cudaError_t e0 = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)(kCsrLutBytes + kCsrSmemCtab * sizeof(double2)) + 64);
    if (e0 != cudaSuccess) return e0;
    // one wave of resident blocks striding the row chunks (no partial second wave)
    int per_sm = 0;
    e0 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kCsrThreads, smem);
    if (e0 != cudaSuccess) return e0;
    if (per_sm < 1) per_sm = 1;
    if (g > (uint64_t)nsm * per_sm) g = (uint64_t)nsm * per_sm;
    kern<<<(unsigned)g, kCsrThreads, smem, st>>>(a);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    CsrArgs b = a;
    b.fvals = nullptr;  // direct path: fold entries stored in place
    return launch_csr_fold(b, nsm, st);
}

// y = A v, complex128.  S lanes per row, U entries per lane per step with
// the step's tail predicated, so that a row of up to S * U entries costs one
// round of dependent loads (index, then the gathered v); the lanes' partial
// sums meet in a butterfly over the S lanes.  The GB300's FP64 rate is the
// bound: a step whose S * U slots match the row length wastes no DFMA slot.
// Replaces spmat_dot_densevec (qrusty/src/accel.rs:338-370).
template <int S, int U>
__device__ __forceinline__ void spmv_rows(uint64_t nrows, uint64_t ncols,
                                          const uint64_t *__restrict__ indptr,
                                          const uint64_t *__restrict__ indices,
                                          const double2 *__restrict__ data,
                                          const double2 *__restrict__ v, double2 *__restrict__ y) {
    const uint32_t sl = threadIdx.x & (S - 1);
    const uint64_t groups = (uint64_t)gridDim.x * (blockDim.x / S);
    for (uint64_t r = blockIdx.x * (uint64_t)(blockDim.x / S) + (threadIdx.x / S); r < nrows;
         r += groups) {
        const uint64_t j0 = indptr[r], j1 = indptr[r + 1];
        double sr = 0.0, si = 0.0, tr = 0.0, ti = 0.0;
        for (uint64_t j = j0 + sl; j < j1; j += (uint64_t)U * S) {
            uint64_t c[U];
            double2 d[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {  // the matrix streams once: evict-first loads
                const bool ok = j + (uint64_t)u * S < j1;
                c[u] = ok ? __ldcs(indices + j + u * S) : ncols;
                d[u] = ok ? __ldcs(data + j + u * S) : make_double2(0.0, 0.0);
            }
            double2 x[U];
#pragma unroll
            for (int u = 0; u < U; ++u)
                x[u] = c[u] < ncols ? __ldg(v + c[u]) : make_double2(0.0, 0.0);
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (c[u] >= ncols) continue;  // out-of-range columns (and the tail) are skipped
                double &ar = (u & 1) ? tr : sr, &ai = (u & 1) ? ti : si;
                ar = fma(d[u].x, x[u].x, fma(-d[u].y, x[u].y, ar));
                ai = fma(d[u].x, x[u].y, fma(d[u].y, x[u].x, ai));
            }
        }
        sr += tr;
        si += ti;
#pragma unroll
        for (int o = S / 2; o > 0; o >>= 1) {
            sr += __shfl_xor_sync(0xffffffffu, sr, o, S);
            si += __shfl_xor_sync(0xffffffffu, si, o, S);
        }
        if (sl == 0) y[r] = make_double2(sr, si);
    }
}

constexpr int kSpmvLanes = 4;   // lanes per row
constexpr int kSpmvMaxStep = 16;  // entries per lane per step, at most

// The step depth U is chosen from the first row's length (every row of a
// Pauli-sum CSR holds G entries; any CSR is handled at any depth).
__global__ void __launch_bounds__(256) csr_spmv_kernel(uint64_t nrows, uint64_t ncols,
                                                       const uint64_t *__restrict__ indptr,
                                                       const uint64_t *__restrict__ indices,
                                                       const double2 *__restrict__ data,
                                                       const double2 *__restrict__ v,
                                                       double2 *__restrict__ y) {
    constexpr int S = kSpmvLanes;
    const uint64_t len0 = indptr[1] - indptr[0];
    const uint64_t want = (len0 + S - 1) / S;
    const int u = want < 1 ? 1 : (want > (uint64_t)kSpmvMaxStep ? kSpmvMaxStep : (int)want);
#define QR_SPMV_CASE(k) \
    case k: spmv_rows<S, k>(nrows, ncols, indptr, indices, data, v, y); break;
    switch (u) {
        QR_SPMV_CASE(1) QR_SPMV_CASE(2) QR_SPMV_CASE(3) QR_SPMV_CASE(4)
        QR_SPMV_CASE(5) QR_SPMV_CASE(6) QR_SPMV_CASE(7) QR_SPMV_CASE(8)
        QR_SPMV_CASE(9) QR_SPMV_CASE(10) QR_SPMV_CASE(11) QR_SPMV_CASE(12)
        QR_SPMV_CASE(13) QR_SPMV_CASE(14) QR_SPMV_CASE(15)
        default: spmv_rows<S, kSpmvMaxStep>(nrows, ncols, indptr, indices, data, v, y); break;
    }
#undef QR_SPMV_CASE
}

cudaError_t launch_csr_spmv(uint64_t nrows, uint64_t ncols, const uint64_t *indptr,
                            const uint64_t *indices, const double *data, const double *v,
                            double *y, int nsm, cudaStream_t st) {
    if (nrows == 0) return cudaSuccess;
    // no host read of nnz or row lengths: the call stays asynchronous
    const uint64_t rows_per_block = 256 / kSpmvLanes;
    uint64_t g = (nrows + rows_per_block - 1) / rows_per_block;
    if (g > (uint64_t)nsm * 16) g = (uint64_t)nsm * 16;
    csr_spmv_kernel<<<(unsigned)g, 256, 0, st>>>(nrows, ncols, indptr, indices,
                                                 reinterpret_cast<const double2 *>(data),
                                                 reinterpret_cast<const double2 *>(v),
                                                 reinterpret_cast<double2 *>(y));
    count_launch();
    return cudaGetLastError();
}

}  // namespace qr
