// qr_host.cu -- C ABI of libqrusty_gpu (declared in include/qrusty_gpu.h).
//
// Host half of the GB300 Pauli-operator hot path: validates the terms,
// computes c'_k in FP64, groups the terms by x mask, prepares the CSR and
// apply tables, owns the operator's device memory and launches the kernels
// of qr_csr.cu / qr_apply.cu.  No CPU fallback exists: every numeric result
// is computed on the GPU.
//
// Compiled with -ffp-contract=off: c'_k = m(phase) * c_k must round exactly
// as num-complex's (ar*br - ai*bi, ar*bi + ai*br) does in qrusty's
// make_params (qrusty/src/accel.rs:141-157).
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "../../include/qrusty_gpu.h"
#include "qr_common.cuh"

namespace qr {

static std::atomic<uint64_t> g_launches{0};
void count_launch(uint64_t k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

cudaError_t ensure_dyn_smem(const void *fn, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, size_t> set;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    auto key = std::make_pair(dev, fn);
    auto it = set.find(key);
    if (it != set.end() && it->second >= bytes) return cudaSuccess;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) set[key] = bytes;
    return e;
}

static thread_local std::string g_err;

static int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}
static int cuda_fail(cudaError_t e, const char *what) {
    return fail(QR_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}
int set_error(int code, const char *msg) { return fail(code, "%s", msg); }

#define QR_CUDA(call, what)                          \
    do {                                             \
        cudaError_t e_ = (call);                     \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

struct cd {
    double re, im;
};

// Device buffer with RAII release.
// Device buffer that keeps its allocation when refilled with no more bytes
// than it holds (plan rebuilds after a coefficient update reuse it instead of
// a cudaFree / cudaMalloc pair, which would synchronise the device).
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0, cap = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = cap = 0;
    }
    cudaError_t alloc(size_t b) {
        if (b == 0) b = 16;
        if (p && b <= cap) {
            bytes = b;
            return cudaSuccess;
        }
        release();
        cudaError_t e = cudaMalloc(&p, b);
        if (e == cudaSuccess) bytes = cap = b;
        else p = nullptr;
        return e;
    }
    template <typename T>
    cudaError_t upload(const std::vector<T> &v) {
        cudaError_t e = alloc(v.size() * sizeof(T));
        if (e != cudaSuccess) return e;
        if (!v.empty()) e = cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
        return e;
    }
    template <typename T>
    T *as() const { return static_cast<T *>(p); }
};

struct Plan {
    bool built = false;
    int b = 0, tb = 0, threads = 0, amps = 0;
    uint32_t nblocks = 0;
    uint64_t ngroups = 0, nfat = 0;
    int diag_block = -1;
    bool has_diag = false;
    DevBuf groups, tables, fat_z, fat_c, blk_hi, blk_g0, diag;
    // compensated-c64 kernel tables
    uint32_t nsub = 0, nruns = 0, nchunks = 0, npairs = 0;
    DevBuf tdesc, tdata, blk_r0, run_g0, run_key, chunks;
    // what the plan was built for, and its coefficient program: the slots
    // that qr_op_set_coeffs_device recomputes on the device, with the
    // diagonal's term list kept so that diag_wht can run again
    int dtype = 0, adjoint = 0;
    uint32_t nslots = 0;
    DevBuf cslots, cmem, ccoord;
    DevBuf dg_tz, dg_tc, dg_bz, dg_boff;
    uint32_t dg_nbins = 0;
    int dg_db = 0;
};

}  // namespace qr

using namespace qr;

struct qr_op {
    int n = 0;
    uint64_t N = 0, T = 0;
    int device = 0;
    int nsm = 0;
    // input terms on the device: masks, phases and the last coefficients
    // (input order); every table below is derived from them on the device
    DevBuf d_x, d_z, d_ph, d_coef;
    // grouping on the device (qr_group.cu): CSR order and the ascending x
    // groups, the merged strings (FP64 simplification, first-occurrence
    // order) with each one's input terms, the apply plan's x-groups
    uint64_t G = 0, M = 0, Ga = 0;
    DevBuf d_order, d_tz, d_gx, d_goff, d_mmap, d_mm_off, d_mm_terms, d_mx, d_mz, d_madj;
    DevBuf d_ag_off, d_ag_mem, d_mc;
    // host copies of the grouping, read by the apply plan builder and the
    // operator diagonal; mc is refetched from d_mc while host_coef_stale
    std::vector<uint64_t> gx, mx, mz;
    std::vector<uint32_t> goff, ag_off, ag_mem;
    std::vector<cd> mc;
    bool host_coef_stale = false;
    // CSR tables, built on the device on first use; their coefficient parts
    // follow every coefficient update on the device
    bool csr_ready = false;
    uint32_t nfold = 0, nctab = 0;
    DevBuf d_tc, d_pmask, d_sig, d_grp, d_coord, d_ctab, d_fold, d_pbeta, d_ptab, d_fv;
    // term-gradient batches (complex64, n >= 12): merged strings sorted by
    // partner tile x >> 12, batches of <= 8 strings of one partner tile
    bool tg_ready = false;
    uint32_t tg_nbatch = 0;
    DevBuf d_tg_x, d_tg_z, d_tg_perm, d_tg_bat;
    DevBuf expect_y;                    // H psi buffer of qr_expect
    Plan plans[2][2];  // [dtype][adjoint]
    Plan bplans[13];   // compensated-c64 plans with an explicit tile width (batched launches)
    DevBuf d_err;
    // host-call staging
    cudaStream_t hstream = nullptr;
    cudaStream_t cstream = nullptr;  // host-call copies of states 1.. (overlap)
    cudaEvent_t cev = nullptr;
    DevBuf stage_in, stage_out;
    // bumped by every host coefficient update: a qr_batch built on this
    // operator compares it with the value it recorded and rebuilds when they
    // differ (device updates rewrite the built tables in place instead)
    uint64_t coef_gen = 0;
    // test hooks (qr_op_set_test_hooks): mbarrier wait bound (0 = default),
    // withheld ring step (-1 = none), 64-bit row words forced
    uint64_t test_wait_ns = 0;
    int64_t test_withhold = -1;
    int test_wide = 0;
};

namespace {

struct Span {
    std::vector<uint64_t> basis;
    std::vector<uint64_t> coord;  // per term
    bool overflow = false;
    size_t used = 0;  // leading terms whose coordinates are set (all, without overflow)
};
Span gf2_span(const std::vector<uint64_t> &zs, size_t dmax);

// ---------------------------------------------------------------- coefficients
// After a device coefficient update the host copy of the merged coefficients
// is older than d_mc: fetch it (synchronous) before a plan is built.
int sync_host_coeffs(qr_op *op) {
    if (!op->host_coef_stale) return QR_OK;
    // the update ran on the caller's stream, which may not be ordered with
    // the legacy stream: wait for the device
    QR_CUDA(cudaDeviceSynchronize(), "fetch merged coefficients: sync");
    op->mc.resize(op->M);
    QR_CUDA(cudaMemcpy(op->mc.data(), op->d_mc.p, op->M * sizeof(cd), cudaMemcpyDeviceToHost),
            "fetch merged coefficients");
    op->host_coef_stale = false;
    return QR_OK;
}

// Coefficient-dependent CSR tables from d_coef, on stream st.
int refresh_csr_values(qr_op *op, cudaStream_t st) {
    QR_CUDA(csr_values(op->G, op->T, op->d_order.as<uint32_t>(), op->d_coef.as<double2>(),
                       op->d_ph.as<uint8_t>(), op->d_tc.as<double2>(), op->d_grp.as<CsrGroup>(),
                       op->d_coord.as<uint16_t>(), op->d_ctab.as<double2>(),
                       op->d_ptab.as<double2>(), st),
            "CSR coefficient tables");
    return QR_OK;
}

// CSR tables on the device, once per operator (qr_group.cu): the position
// trie, group spans and descriptors, then the coefficient parts.
int upload_csr_tables(qr_op *op) {
    if (op->csr_ready) return QR_OK;
    // d_coef may have been written on another stream
    QR_CUDA(cudaDeviceSynchronize(), "CSR tables: sync");
    const uint64_t G = op->G, T = op->T;
    QR_CUDA(op->d_pmask.alloc(G * sizeof(uint64_t)), "alloc position masks");
    QR_CUDA(op->d_sig.alloc(G * op->n * sizeof(int32_t)), "alloc position table");
    QR_CUDA(op->d_grp.alloc(G * sizeof(CsrGroup)), "alloc group descriptors");
    QR_CUDA(op->d_coord.alloc(T * sizeof(uint16_t)), "alloc span coordinates");
    QR_CUDA(op->d_fold.alloc(G * sizeof(uint32_t)), "alloc fold groups");
    QR_CUDA(op->d_pbeta.alloc(G * kCsrPrefixRank * sizeof(uint64_t)), "alloc prefix bases");
    QR_CUDA(op->d_tc.alloc(T * sizeof(cd)), "alloc CSR coefficients");
    CsrStructOut o{op->d_pmask.as<uint64_t>(), op->d_sig.as<int32_t>(), op->d_grp.as<CsrGroup>(),
                   op->d_coord.as<uint16_t>(), op->d_fold.as<uint32_t>(),
                   op->d_pbeta.as<uint64_t>()};
    CsrStructCounts cnt;
    QR_CUDA(csr_structure(op->n, G, op->d_gx.as<uint64_t>(), op->d_goff.as<uint32_t>(),
                          op->d_tz.as<uint64_t>(), o, &cnt, nullptr),
            "CSR tables");
    if (cnt.nctab > 0xffffffffull || cnt.nptab > 0xffffffffull)
        return fail(QR_EINVAL, "qr_csr_build: class tables too large");
    QR_CUDA(op->d_ctab.alloc(cnt.nctab * sizeof(cd)), "alloc class tables");
    QR_CUDA(op->d_ptab.alloc(cnt.nptab * sizeof(cd)), "alloc prefix tables");
    op->nctab = (uint32_t)cnt.nctab;
    op->nfold = cnt.nfold;
    int rc = refresh_csr_values(op, nullptr);
    if (rc) return rc;
    QR_CUDA(cudaStreamSynchronize(nullptr), "CSR tables: sync");
    op->csr_ready = true;
    return QR_OK;
}

// GF(2) span of the z differences of one group: basis (pivot = msb, unique)
// and the coordinates of every term's difference in that basis.
Span gf2_span(const std::vector<uint64_t> &zs, size_t dmax) {
    Span sp;
    const uint64_t z0 = zs[0];
    sp.coord.resize(zs.size());
    for (size_t k = 0; k < zs.size(); ++k) {
        uint64_t v = zs[k] ^ z0;
        uint64_t c = 0;
        // basis kept in order of insertion; reduce by descending pivot
        std::vector<size_t> ord(sp.basis.size());
        for (size_t i = 0; i < ord.size(); ++i) ord[i] = i;
        std::sort(ord.begin(), ord.end(),
                  [&](size_t a, size_t b) { return sp.basis[a] > sp.basis[b]; });
        for (size_t i : ord) {
            const uint64_t bv = sp.basis[i];
            const int piv = 63 - __builtin_clzll(bv);
            if ((v >> piv) & 1ull) {
                v ^= bv;
                c |= 1ull << i;
            }
        }
        if (v != 0) {
            if (sp.basis.size() >= dmax) {
                sp.overflow = true;
                sp.used = k;
                return sp;
            }
            c |= 1ull << sp.basis.size();
            sp.basis.push_back(v);
        }
        sp.coord[k] = c;
    }
    sp.used = zs.size();
    return sp;
}

template <typename Real>
void push_cplx(std::vector<unsigned char> &buf, cd v) {
    Cplx<Real> c;
    c.re = (Real)v.re;
    c.im = (Real)v.im;
    const unsigned char *p = reinterpret_cast<const unsigned char *>(&c);
    buf.insert(buf.end(), p, p + sizeof(c));
}

// One sub-group of the apply plan: terms sharing x (and, for the c64c
// kernel, z on the register bits), with their FP64 table or term list.
struct SubGroup {
    uint64_t hi = 0;       // partner-tile XOR (x >> b)
    uint32_t lo = 0;       // x & (tile - 1)
    uint32_t zm = 0;       // z bits on the register bits (c64c), or kFat
    uint64_t z0 = 0;
    uint64_t beta[kDMax] = {0, 0, 0, 0};
    uint32_t d = 0;        // rank, or kFat
    std::vector<cd> table; // 2^d entries
    std::vector<uint64_t> fz;
    std::vector<cd> fc;
    // merged strings of the sub-group in fold order, each with its coordinate
    // in the span basis (table entry u adds it with sign (-1)^popc(u & coord))
    std::vector<uint32_t> mem;
    std::vector<uint8_t> coord;
};

int build_plan(qr_op *op, int dtype, int adjoint, int tile_bits = -1) {
    Plan &pl = tile_bits < 0 ? op->plans[dtype][adjoint] : op->bplans[tile_bits];
    if (pl.built) return QR_OK;
    {
        const int rc = sync_host_coeffs(op);
        if (rc) return rc;
    }
    pl.dtype = dtype;
    pl.adjoint = adjoint;
    // coefficient program (see CoefSlot): members packed per slot
    std::vector<CoefSlot> slots;
    std::vector<uint32_t> cmem;
    std::vector<uint8_t> ccoord;
    auto add_slot = [&](uint64_t dst, const uint32_t *mem, const uint8_t *coord, size_t cnt,
                        uint32_t d, uint8_t kind) {
        CoefSlot sl;
        sl.dst = dst;
        sl.m0 = (uint32_t)cmem.size();
        sl.cnt = (uint16_t)cnt;
        sl.d = (uint8_t)d;
        sl.kind = kind;
        for (size_t k = 0; k < cnt; ++k) {
            cmem.push_back(mem[k]);
            ccoord.push_back(coord ? coord[k] : 0);
        }
        slots.push_back(sl);
    };
    const int n = op->n;
    const bool f32 = dtype == QR_C64C;
    pl.b = tile_bits < 0 ? std::min(n, 12) : std::min(n, tile_bits);
    const int tmax = !f32 ? 512 : (1 << kC64ThreadBits);
    pl.threads = std::min(1 << pl.b, tmax);
    pl.amps = (1 << pl.b) / pl.threads;
    pl.tb = 0;
    while ((1 << pl.tb) < pl.threads) ++pl.tb;
    const uint64_t tmask = (1ull << pl.b) - 1;

    // coefficients of this plan (adjoint: conj(c) * (-1)^popc(x & z))
    const size_t M = op->mx.size();
    std::vector<cd> c(M);
    for (size_t k = 0; k < M; ++k) {
        c[k] = op->mc[k];
        if (adjoint) {
            c[k].im = -c[k].im;
            if (__builtin_popcountll(op->mx[k] & op->mz[k]) & 1) {
                c[k].re = -c[k].re;
                c[k].im = -c[k].im;
            }
        }
    }
    // x-groups of the merged strings in first-occurrence order (grouped on
    // the device at creation)
    std::vector<uint64_t> gxs(op->Ga);
    std::vector<std::vector<size_t>> members(op->Ga);
    for (size_t g = 0; g < op->Ga; ++g) {
        members[g].assign(op->ag_mem.begin() + op->ag_off[g], op->ag_mem.begin() + op->ag_off[g + 1]);
        gxs[g] = op->mx[members[g][0]];
    }
    // The compensated-c64 kernel keeps a sub-group's factor thread-constant
    // up to a Walsh sign over the register bits [tb, tb + log2 amps): split
    // each x-group by its terms' z bits there.  The c128 kernel does not split.
    int abits = 0;
    while ((1 << abits) < pl.amps) ++abits;
    const uint64_t mmask = f32 ? (((1ull << abits) - 1) << pl.tb) : 0;
    std::vector<size_t> diag_terms;
    std::vector<SubGroup> subs;
    for (size_t g = 0; g < gxs.size(); ++g) {
        if (gxs[g] == 0) {
            std::vector<uint64_t> zs;
            for (size_t k : members[g]) zs.push_back(op->mz[k]);
            if (gf2_span(zs, kDMax).overflow) {
                diag_terms = members[g];
                continue;
            }
        }
        std::vector<uint64_t> pkeys;
        std::vector<std::vector<size_t>> parts;
        for (size_t k : members[g]) {
            const uint64_t key = op->mz[k] & mmask;
            size_t pi = 0;
            while (pi < pkeys.size() && pkeys[pi] != key) ++pi;
            if (pi == pkeys.size()) {
                pkeys.push_back(key);
                parts.emplace_back();
            }
            parts[pi].push_back(k);
        }
        // c64c: split further until every sub-group has rank <= 2 (terms whose
        // z differences agree beyond the first two basis vectors)
        std::vector<std::vector<size_t>> pieces;
        for (const auto &part : parts) {
            if (!f32) {
                pieces.push_back(part);
                continue;
            }
            std::vector<uint64_t> zs;
            for (size_t k : part) zs.push_back(op->mz[k]);
            Span full = gf2_span(zs, 64);
            if (full.basis.size() <= 2) {
                pieces.push_back(part);
                continue;
            }
            std::vector<uint64_t> hk;
            std::vector<std::vector<size_t>> hp;
            for (size_t kk = 0; kk < part.size(); ++kk) {
                const uint64_t key = full.coord[kk] >> 2;
                size_t pi = 0;
                while (pi < hk.size() && hk[pi] != key) ++pi;
                if (pi == hk.size()) {
                    hk.push_back(key);
                    hp.emplace_back();
                }
                hp[pi].push_back(part[kk]);
            }
            for (auto &h : hp) pieces.push_back(std::move(h));
        }
        for (const auto &part : pieces) {
            std::vector<uint64_t> zs;
            for (size_t k : part) zs.push_back(op->mz[k]);
            Span sp = gf2_span(zs, kDMax);
            SubGroup sg;
            sg.hi = gxs[g] >> pl.b;
            sg.lo = (uint32_t)(gxs[g] & tmask);
            sg.z0 = zs[0];
            if (!sp.overflow) {
                sg.d = (uint32_t)sp.basis.size();
                sg.zm = (uint32_t)((sg.z0 & mmask) >> pl.tb);
                for (size_t i = 0; i < sp.basis.size(); ++i) sg.beta[i] = sp.basis[i];
                const uint32_t ent = 1u << sg.d;
                for (size_t kk = 0; kk < part.size(); ++kk) {
                    sg.mem.push_back((uint32_t)part[kk]);
                    sg.coord.push_back((uint8_t)sp.coord[kk]);
                }
                for (uint32_t u = 0; u < ent; ++u) {
                    cd acc{0.0, 0.0};
                    for (size_t kk = 0; kk < part.size(); ++kk) {
                        const cd v = c[part[kk]];
                        if (__builtin_popcountll(u & sp.coord[kk]) & 1) {
                            acc.re -= v.re;
                            acc.im -= v.im;
                        } else {
                            acc.re += v.re;
                            acc.im += v.im;
                        }
                    }
                    sg.table.push_back(acc);
                }
            } else {
                sg.d = kFat;
                sg.zm = kFat;
                for (size_t k : part) {
                    sg.fz.push_back(op->mz[k]);
                    sg.fc.push_back(c[k]);
                    sg.mem.push_back((uint32_t)k);
                    sg.coord.push_back(0);
                }
            }
            subs.push_back(std::move(sg));
        }
    }
    pl.has_diag = !diag_terms.empty();
    // order: partner tile ascending, then (c64c) run key zm with fat last
    std::vector<size_t> ord(subs.size());
    for (size_t i = 0; i < ord.size(); ++i) ord[i] = i;
    // run key: register-bit sign pattern zm, register bits in the partner
    // XOR (xm), and whether the factor depends on the thread index (tv)
    auto runkey = [&](const SubGroup &g) -> uint32_t {
        if (g.d == kFat || g.d > 2) return 0xffffffffu;
        const uint64_t tm = (uint64_t)pl.threads - 1;
        const uint64_t b0 = g.d > 0 ? g.beta[0] : 0, b1 = g.d > 1 ? g.beta[1] : 0;
        const uint32_t tv = ((g.z0 | b0 | b1) & tm) != 0 ? 1u : 0u;
        return (g.zm & 15u) | (((g.lo >> pl.tb) != 0 ? 1u : 0u) << 4) | (tv << 5);
    };
    std::stable_sort(ord.begin(), ord.end(), [&](size_t a, size_t b) {
        if (subs[a].hi != subs[b].hi) return subs[a].hi < subs[b].hi;
        return f32 && runkey(subs[a]) < runkey(subs[b]);
    });
    std::vector<uint64_t> bhi;
    std::vector<uint32_t> bg0;
    if (pl.has_diag && (ord.empty() || subs[ord[0]].hi != 0)) {
        bhi.push_back(0);
        bg0.push_back(0);
    }
    for (size_t i = 0; i < ord.size(); ++i) {
        const uint64_t h = subs[ord[i]].hi;
        if (bhi.empty() || bhi.back() != h) {
            bhi.push_back(h);
            bg0.push_back((uint32_t)i);
        }
    }
    bg0.push_back((uint32_t)ord.size());
    if (f32) {
        // the per-tile table holds at most kTabCap sub-groups: a partner tile
        // with more is visited as several consecutive blocks (same partner)
        std::vector<uint64_t> vh;
        std::vector<uint32_t> vg;
        for (size_t j = 0; j + 1 < bg0.size(); ++j) {
            uint32_t g = bg0[j];
            do {
                vh.push_back(bhi[j]);
                vg.push_back(g);
                g += std::min<uint32_t>(kTabCap, bg0[j + 1] - g);
            } while (g < bg0[j + 1]);
        }
        vg.push_back((uint32_t)ord.size());
        bhi.swap(vh);
        bg0.swap(vg);
    }
    // pair plans: partner blocks with one sub-group are cheap to consume and
    // a ring of three pairs cannot hide the refill behind a run of them, so
    // the blocks are paired heavy with heavy and light with light and the
    // heavy pairs are spread evenly among the light ones, each closing a run
    // of light pairs (the tile's last pair is heavy, so the ring refills
    // across the table rebuild and the next tile starts on light pairs); the
    // same order for every output tile
    if (f32 && tile_bits < 0 && ord.size() <= (size_t)kTabCap && bhi.size() >= 4 &&
        pl.amps == 8) {
        const size_t nbk = bhi.size();
        std::vector<uint32_t> heavy, light;
        for (uint32_t j = 0; j < nbk; ++j)
            ((bg0[j + 1] - bg0[j] > 1 || bhi[j] == 0) ? heavy : light).push_back(j);
        std::vector<std::vector<uint32_t>> hp, lp;
        for (size_t i = 0; i < heavy.size(); i += 2)
            hp.push_back(i + 1 < heavy.size() ? std::vector<uint32_t>{heavy[i], heavy[i + 1]}
                                              : std::vector<uint32_t>{heavy[i]});
        // an odd heavy block takes a light partner
        size_t l0 = 0;
        if (!hp.empty() && hp.back().size() == 1 && !light.empty()) hp.back().push_back(light[l0++]);
        for (size_t i = l0; i < light.size(); i += 2)
            lp.push_back(i + 1 < light.size() ? std::vector<uint32_t>{light[i], light[i + 1]}
                                              : std::vector<uint32_t>{light[i]});
        // a single-block pair can only be the last one
        std::vector<uint32_t> tail;
        if (!lp.empty() && lp.back().size() == 1) {
            tail = lp.back();
            lp.pop_back();
        } else if (!hp.empty() && hp.back().size() == 1) {
            tail = hp.back();
            hp.pop_back();
        }
        std::vector<std::vector<uint32_t>> seq;
        const size_t nh = hp.size(), tot = hp.size() + lp.size();
        size_t ih = 0, il = 0;
        for (size_t k = 0; k < tot; ++k) {
            // heavy pair ih goes at position floor((ih + 1) * tot / nh) - 1
            if (ih < nh && (il >= lp.size() || k >= (ih + 1) * tot / nh - 1))
                seq.push_back(hp[ih++]);
            else seq.push_back(lp[il++]);
        }
        if (!tail.empty()) seq.push_back(tail);
        std::vector<size_t> nord;
        std::vector<uint64_t> nbhi;
        std::vector<uint32_t> nbg0;
        for (const auto &pr : seq)
            for (uint32_t j : pr) {
                nbhi.push_back(bhi[j]);
                nbg0.push_back((uint32_t)nord.size());
                for (uint32_t g = bg0[j]; g < bg0[j + 1]; ++g) nord.push_back(ord[g]);
            }
        nbg0.push_back((uint32_t)nord.size());
        ord.swap(nord);
        bhi.swap(nbhi);
        bg0.swap(nbg0);
    }
    pl.nblocks = (uint32_t)bhi.size();
    pl.ngroups = ord.size();
    pl.diag_block = -1;
    for (size_t j = 0; j < bhi.size(); ++j)
        if (bhi[j] == 0 && pl.diag_block < 0) pl.diag_block = (int)j;

    // single-chunk c64c plans: partner blocks are visited in pairs (two
    // stages behind one barrier, one ring slot); each pair's sub-groups are
    // merged and sorted by run key, their block recorded as the half
    std::vector<uint32_t> half(ord.size(), 0u), pg0, pkey;
    pl.npairs = 0;
    if (f32 && tile_bits < 0 && ord.size() <= (size_t)kTabCap && pl.nblocks >= 2 &&
        pl.amps == 8) {
        const uint32_t np = (pl.nblocks + 1) / 2;
        std::vector<size_t> ord2;
        std::vector<uint32_t> half2;
        ord2.reserve(ord.size());
        const uint64_t tm = (uint64_t)pl.threads - 1;
        auto small = [&](const SubGroup &g) { return g.d != kFat && g.d <= 2; };
        auto thread_var = [&](const SubGroup &g) -> uint32_t {
            const uint64_t b0 = g.d > 0 ? g.beta[0] : 0, b1 = g.d > 1 ? g.beta[1] : 0;
            return ((g.z0 | b0 | b1) & tm) != 0 ? 1u : 0u;
        };
        for (uint32_t p = 0; p < np; ++p) {
            pg0.push_back((uint32_t)ord2.size());
            const uint32_t ga = bg0[2 * p], gm = bg0[std::min(2 * p + 1, pl.nblocks)],
                           gb = bg0[std::min(2 * p + 2, pl.nblocks)];
            // fused pairs: two sub-groups of one x group (same partner
            // amplitudes) whose register-bit sign patterns differ in one bit
            std::vector<uint32_t> items;
            std::vector<char> used(gb - ga, 0);
            struct Fused { uint32_t key, a, b; };
            std::vector<Fused> fused;
            for (uint32_t i = ga; i < gb; ++i) {
                const SubGroup &si = subs[ord[i]];
                if (used[i - ga]) continue;
                for (uint32_t j = i + 1; j < gb && small(si); ++j) {
                    const SubGroup &sj = subs[ord[j]];
                    if (used[j - ga] || !small(sj) || si.hi != sj.hi || si.lo != sj.lo ||
                        (i >= gm) != (j >= gm))
                        continue;
                    const uint32_t diff = si.zm ^ sj.zm;
                    if (__builtin_popcount(diff) != 1) continue;
                    const uint32_t a = si.zm < sj.zm ? i : j, b = si.zm < sj.zm ? j : i;
                    const uint32_t bb = (uint32_t)__builtin_ctz(diff);
                    const uint32_t xm = (si.lo >> pl.tb) != 0 ? 1u : 0u;
                    const uint32_t tv = thread_var(si) | thread_var(sj);
                    // key 64 + (ZM | BB << 3 | XM << 5 | TV << 6): 64..191
                    fused.push_back({64u + ((subs[ord[a]].zm & 7u) | (bb << 3) | (xm << 5) |
                                            (tv << 6)),
                                     a, b});
                    used[i - ga] = used[j - ga] = 1;
                    break;
                }
                if (!used[i - ga]) items.push_back(i);
            }
            std::stable_sort(items.begin(), items.end(), [&](uint32_t x, uint32_t y) {
                return runkey(subs[ord[x]]) < runkey(subs[ord[y]]);
            });
            std::stable_sort(fused.begin(), fused.end(),
                             [](const Fused &x, const Fused &y) { return x.key < y.key; });
            for (uint32_t i : items) {
                ord2.push_back(ord[i]);
                half2.push_back(i >= gm ? 1u : 0u);
                pkey.push_back(runkey(subs[ord[i]]) & 63u);
            }
            for (const Fused &f : fused) {
                for (uint32_t i : {f.a, f.b}) {
                    ord2.push_back(ord[i]);
                    half2.push_back(i >= gm ? 1u : 0u);
                    pkey.push_back(f.key);
                }
            }
        }
        pg0.push_back((uint32_t)ord2.size());
        ord.swap(ord2);
        half.swap(half2);
        pl.npairs = np;
    }

    std::vector<unsigned char> tab, fc;
    std::vector<uint64_t> fz;
    uint32_t ntab = 0, nfat_terms = 0;
    std::vector<GroupDesc> descs;           // c128 kernel
    pl.nfat = 0;
    for (size_t i = 0; i < ord.size(); ++i) {
        const SubGroup &sg = subs[ord[i]];
        GroupDesc d;
        memset(&d, 0, sizeof(d));
        d.z0 = sg.z0;
        d.lo = sg.lo;
        d.d = sg.d;
        for (int q = 0; q < kDMax; ++q) d.beta[q] = sg.beta[q];
        if (sg.d != kFat) {
            d.off = ntab;
            for (const cd &v : sg.table) {
                if (f32) push_cplx<float>(tab, v);
                else push_cplx<double>(tab, v);
            }
            ntab += (uint32_t)sg.table.size();
        } else {
            d.off = nfat_terms;
            d.cnt = (uint32_t)sg.fz.size();
            for (size_t k = 0; k < sg.fz.size(); ++k) {
                fz.push_back(sg.fz[k]);
                if (f32) push_cplx<float>(fc, sg.fc[k]);
                else push_cplx<double>(fc, sg.fc[k]);
            }
            nfat_terms += d.cnt;
            pl.nfat++;
        }
        descs.push_back(d);
    }
    if (f32) {
        // per-tile-table kernel arrays
        std::vector<uint4> td;
        std::vector<TileDataC64> tdd;
        std::vector<uint32_t> r0v, rg0, rkey;
        const uint64_t tmask_t = (uint64_t)pl.threads - 1;
        for (size_t i = 0; i < ord.size(); ++i) {
            const SubGroup &sg = subs[ord[i]];
            const uint64_t b0 = sg.d > 0 && sg.d != kFat ? sg.beta[0] : 0;
            const uint64_t b1 = sg.d > 1 && sg.d != kFat ? sg.beta[1] : 0;
            const uint32_t zt = (uint32_t)(sg.z0 & tmask_t), bt0 = (uint32_t)(b0 & tmask_t),
                           bt1 = (uint32_t)(b1 & tmask_t);
            const uint32_t tvar = (zt | bt0 | bt1) != 0 ? 1u : 0u;
            // byte-offset XOR of the partner within the tile: thread bits of lo
            // (x 8 bytes) and register bits of lo (x 8 x threads); needs
            // threads == 1 << kC64ThreadBits whenever lo has register bits
            const uint32_t lt = (uint32_t)(sg.lo & tmask_t), lm = sg.lo >> pl.tb;
            const uint32_t dx = (lt << 3) | (lm << (pl.tb + 3));
            td.push_back(make_uint4(dx | (half[i] << 15) | (tvar << 31), zt, bt0, bt1));
            TileDataC64 d;
            memset(&d, 0, sizeof(d));
            d.z0h = sg.z0 >> pl.b;
            d.b0h = b0 >> pl.b;
            d.b1h = b1 >> pl.b;
            for (size_t u = 0; u < sg.table.size() && u < 4; ++u)
                d.T[u] = make_float2((float)sg.table[u].re, (float)sg.table[u].im);
            tdd.push_back(d);
        }
        // runs per block, or per pair of blocks
        const std::vector<uint32_t> &rng = pl.npairs ? pg0 : bg0;
        const uint32_t nunits = pl.npairs ? pl.npairs : pl.nblocks;
        for (uint32_t j = 0; j < nunits; ++j) {
            r0v.push_back((uint32_t)rkey.size());
            for (uint32_t g = rng[j]; g < rng[j + 1]; ++g) {
                // pair plans: per-position keys (fused pairs carry keys >= 64)
                const uint32_t k = pl.npairs ? pkey[g] : (runkey(subs[ord[g]]) & 63u);
                if (g == rng[j] || k != rkey.back()) {
                    rkey.push_back(k);
                    rg0.push_back(g);
                }
            }
        }
        r0v.push_back((uint32_t)rkey.size());
        rg0.push_back((uint32_t)ord.size());
        // chunks: consecutive blocks holding at most kTabCap sub-groups; the
        // kernel rebuilds its table (and staged run lists) at each chunk start
        std::vector<uint4> ch;
        for (uint32_t j = 0; j < pl.nblocks; ++j) {
            if (ch.empty() || bg0[j + 1] - ch.back().x > kTabCap)
                ch.push_back(make_uint4(bg0[j], r0v[j], j, 0));
        }
        if (ch.empty()) ch.push_back(make_uint4(0, 0, 0, 0));
        pl.nchunks = (uint32_t)ch.size();
        ch.push_back(make_uint4((uint32_t)ord.size(), (uint32_t)rkey.size(), pl.nblocks, 0));
        QR_CUDA(pl.chunks.upload(ch), "upload chunks");
        if (td.empty()) {
            td.push_back(make_uint4(0, 0, 0, 0));
            TileDataC64 z;
            memset(&z, 0, sizeof(z));
            tdd.push_back(z);
        }
        QR_CUDA(pl.tdesc.upload(td), "upload thread descriptors");
        QR_CUDA(pl.tdata.upload(tdd), "upload tile data");
        for (size_t i = 0; i < ord.size(); ++i) {
            const SubGroup &sg = subs[ord[i]];
            if (sg.d == kFat || sg.d > 2 || sg.mem.size() > 0xffff)
                return fail(QR_EINVAL, "plan: sub-group of rank > 2 in a complex64 plan");
            add_slot((uint64_t)pl.tdata.p + i * sizeof(TileDataC64) + offsetof(TileDataC64, T),
                     sg.mem.data(), sg.coord.data(), sg.mem.size(), sg.d, 0);
        }
        // pair plans: bit 31 of a pair's first run marks a pair of exactly two
        // sub-groups with key 0 (no sign pattern, no register-bit XOR, factor
        // constant over the threads), which the kernel runs without the run
        // list; bit 30 in addition when the two sit in halves 0 and 1 and
        // neither permutes the partner tile (x & (tile - 1) == 0), so that
        // their partner offsets are known at compile time
        if (pl.npairs) {
            for (uint32_t j = 0; j < pl.npairs; ++j) {
                const uint32_t a0 = pg0[j], a1 = pg0[j] + 1;
                if (pg0[j + 1] - pg0[j] == 2 && pkey[a0] == 0 && pkey[a1] == 0) {
                    r0v[j] |= 0x80000000u;
                    if (subs[ord[a0]].lo == 0 && subs[ord[a1]].lo == 0 && half[a0] == 0 &&
                        half[a1] == 1)
                        r0v[j] |= 0x40000000u;
                }
            }
        }
        QR_CUDA(pl.blk_r0.upload(r0v), "upload block runs");
        QR_CUDA(pl.run_g0.upload(rg0), "upload runs");
        QR_CUDA(pl.run_key.upload(rkey), "upload run keys");
        pl.nruns = (uint32_t)rkey.size();
        pl.nsub = (uint32_t)ord.size();
    }
    if (!f32) {  // the complex128 kernel's group descriptors, tables, term lists
        if (descs.empty()) descs.push_back(GroupDesc{});  // keep a valid pointer
        QR_CUDA(pl.groups.upload(descs), "upload groups");
        QR_CUDA(pl.tables.upload(tab), "upload tables");
        QR_CUDA(pl.fat_z.upload(fz), "upload fat z");
        QR_CUDA(pl.fat_c.upload(fc), "upload fat c");
        for (size_t i = 0; i < ord.size(); ++i) {
            const SubGroup &sg = subs[ord[i]];
            const GroupDesc &d = descs[i];
            if (sg.d != kFat) {
                if (sg.mem.size() > 0xffff) return fail(QR_EINVAL, "plan: group too large");
                add_slot((uint64_t)pl.tables.p + (uint64_t)d.off * sizeof(Cplx<double>),
                         sg.mem.data(), sg.coord.data(), sg.mem.size(), sg.d, 1);
            } else {
                for (size_t kk = 0; kk < sg.mem.size(); ++kk)
                    add_slot((uint64_t)pl.fat_c.p + (uint64_t)(d.off + kk) * sizeof(Cplx<double>),
                             &sg.mem[kk], nullptr, 1, 0, 2);
            }
        }
    }
    QR_CUDA(pl.blk_hi.upload(bhi), "upload blocks");
    QR_CUDA(pl.blk_g0.upload(bg0), "upload block groups");

    if (pl.has_diag) {
        const int db = std::min(n, 12);
        const uint64_t dmask = (1ull << db) - 1;
        std::vector<size_t> dt = diag_terms;
        std::stable_sort(dt.begin(), dt.end(), [&](size_t a, size_t b) {
            return (op->mz[a] & dmask) < (op->mz[b] & dmask);
        });
        std::vector<uint64_t> tz, bz;
        std::vector<double> tcv;
        std::vector<uint32_t> boff;
        for (size_t i = 0; i < dt.size(); ++i) {
            const uint64_t zl = op->mz[dt[i]] & dmask;
            if (i == 0 || zl != bz.back()) {
                bz.push_back(zl);
                boff.push_back((uint32_t)i);
            }
            tz.push_back(op->mz[dt[i]]);
            tcv.push_back(c[dt[i]].re);
            tcv.push_back(c[dt[i]].im);
        }
        boff.push_back((uint32_t)dt.size());
        QR_CUDA(pl.dg_tz.upload(tz), "upload diag z");
        QR_CUDA(pl.dg_tc.upload(tcv), "upload diag c");
        QR_CUDA(pl.dg_bz.upload(bz), "upload diag bins");
        QR_CUDA(pl.dg_boff.upload(boff), "upload diag bin offsets");
        pl.dg_nbins = (uint32_t)bz.size();
        pl.dg_db = db;
        for (size_t i = 0; i < dt.size(); ++i) {
            const uint32_t mi = (uint32_t)dt[i];
            add_slot((uint64_t)pl.dg_tc.p + i * 2 * sizeof(double), &mi, nullptr, 1, 0, 2);
        }
        const size_t esz = f32 ? sizeof(Cplx<float>) : sizeof(Cplx<double>);
        QR_CUDA(pl.diag.alloc(op->N * esz), "alloc diagonal");
        QR_CUDA(launch_diag(dtype, n, db, op->N >> db, pl.dg_bz.as<uint64_t>(),
                            pl.dg_boff.as<uint32_t>(), pl.dg_nbins, pl.dg_tz.as<uint64_t>(),
                            pl.dg_tc.as<double>(), pl.diag.p, nullptr),
                "diagonal kernel");
        QR_CUDA(cudaDeviceSynchronize(), "diagonal kernel sync");
    }
    if (slots.empty()) slots.push_back(CoefSlot{});  // keep valid pointers
    QR_CUDA(pl.cslots.upload(slots), "upload coefficient program");
    QR_CUDA(pl.cmem.upload(cmem), "upload coefficient program members");
    QR_CUDA(pl.ccoord.upload(ccoord), "upload coefficient program coordinates");
    pl.nslots = cmem.empty() ? 0u : (uint32_t)slots.size();
    pl.built = true;
    return QR_OK;
}

// bound of every mbarrier wait of the apply kernels
constexpr uint64_t kDefaultWaitNs = 2000000000ull;

// Creation: upload the terms once, then group them on the device
// (qr_group.cu) -- CSR order and groups, merged strings, the apply plan's
// x-groups -- and fold the merged coefficients (merge_coeffs_kernel).  The
// host keeps copies of what the apply plan builder reads.
int create_tables(qr_op *op, const uint64_t *x, const uint64_t *z, const uint8_t *phase,
                  const double *coeff) {
    const uint64_t T = op->T;
    QR_CUDA(op->d_err.alloc(sizeof(int)), "qr_op_create: device allocation");
    QR_CUDA(cudaMemset(op->d_err.p, 0, sizeof(int)), "qr_op_create: clear error word");
    QR_CUDA(op->d_x.alloc(T * 8), "alloc x masks");
    QR_CUDA(op->d_z.alloc(T * 8), "alloc z masks");
    QR_CUDA(op->d_ph.alloc(T), "alloc phases");
    QR_CUDA(op->d_coef.alloc(T * sizeof(cd)), "alloc coefficients");
    QR_CUDA(cudaMemcpy(op->d_x.p, x, T * 8, cudaMemcpyHostToDevice), "upload x masks");
    QR_CUDA(cudaMemcpy(op->d_z.p, z, T * 8, cudaMemcpyHostToDevice), "upload z masks");
    QR_CUDA(cudaMemcpy(op->d_ph.p, phase, T, cudaMemcpyHostToDevice), "upload phases");
    QR_CUDA(cudaMemcpy(op->d_coef.p, coeff, T * sizeof(cd), cudaMemcpyHostToDevice),
            "upload coefficients");
    DevBuf *u32s[] = {&op->d_order, &op->d_mmap, &op->d_mm_terms, &op->d_ag_mem};
    for (DevBuf *b : u32s) QR_CUDA(b->alloc(T * 4), "alloc grouping tables");
    DevBuf *offs[] = {&op->d_goff, &op->d_mm_off, &op->d_ag_off};
    for (DevBuf *b : offs) QR_CUDA(b->alloc((T + 1) * 4), "alloc grouping offsets");
    DevBuf *u64s[] = {&op->d_tz, &op->d_gx, &op->d_mx, &op->d_mz};
    for (DevBuf *b : u64s) QR_CUDA(b->alloc(T * 8), "alloc grouping masks");
    QR_CUDA(op->d_madj.alloc(T), "alloc adjoint signs");
    TermGroupsOut o{op->d_order.as<uint32_t>(), op->d_tz.as<uint64_t>(), op->d_gx.as<uint64_t>(),
                    op->d_goff.as<uint32_t>(), op->d_mmap.as<uint32_t>(),
                    op->d_mm_off.as<uint32_t>(), op->d_mm_terms.as<uint32_t>(),
                    op->d_mx.as<uint64_t>(), op->d_mz.as<uint64_t>(), op->d_madj.as<uint8_t>(),
                    op->d_ag_off.as<uint32_t>(), op->d_ag_mem.as<uint32_t>()};
    TermGroupCounts cnt;
    QR_CUDA(group_terms(op->n, T, op->d_x.as<uint64_t>(), op->d_z.as<uint64_t>(), o, &cnt,
                        nullptr),
            "qr_op_create: grouping terms");
    op->G = cnt.G;
    op->M = cnt.M;
    op->Ga = cnt.Ga;
    QR_CUDA(op->d_mc.alloc(op->M * sizeof(cd)), "alloc merged coefficients");
    QR_CUDA(launch_merge_coeffs((uint32_t)op->M, op->d_mm_off.as<uint32_t>(),
                                op->d_mm_terms.as<uint32_t>(), op->d_coef.as<double2>(),
                                op->d_ph.as<uint8_t>(), op->d_mc.as<double2>(), nullptr),
            "merge coefficients");
    op->gx.resize(op->G);
    op->goff.resize(op->G + 1);
    op->mx.resize(op->M);
    op->mz.resize(op->M);
    op->mc.resize(op->M);
    op->ag_off.resize(op->Ga + 1);
    op->ag_mem.resize(op->M);
    QR_CUDA(cudaMemcpy(op->gx.data(), op->d_gx.p, op->G * 8, cudaMemcpyDeviceToHost), "fetch gx");
    QR_CUDA(cudaMemcpy(op->goff.data(), op->d_goff.p, (op->G + 1) * 4, cudaMemcpyDeviceToHost),
            "fetch group offsets");
    QR_CUDA(cudaMemcpy(op->mx.data(), op->d_mx.p, op->M * 8, cudaMemcpyDeviceToHost), "fetch mx");
    QR_CUDA(cudaMemcpy(op->mz.data(), op->d_mz.p, op->M * 8, cudaMemcpyDeviceToHost), "fetch mz");
    QR_CUDA(cudaMemcpy(op->mc.data(), op->d_mc.p, op->M * sizeof(cd), cudaMemcpyDeviceToHost),
            "fetch merged coefficients");
    QR_CUDA(cudaMemcpy(op->ag_off.data(), op->d_ag_off.p, (op->Ga + 1) * 4,
                       cudaMemcpyDeviceToHost),
            "fetch x-group offsets");
    QR_CUDA(cudaMemcpy(op->ag_mem.data(), op->d_ag_mem.p, op->M * 4, cudaMemcpyDeviceToHost),
            "fetch x-group members");
    return QR_OK;
}

int check_device(const qr_op *op) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (dev != op->device)
        return fail(QR_ESTATE, "operator lives on device %d but device %d is current", op->device,
                    dev);
    return QR_OK;
}

int check_kernel_error(qr_op *op) {
    int h = 0;
    QR_CUDA(cudaMemcpy(&h, op->d_err.p, sizeof(int), cudaMemcpyDeviceToHost), "read error word");
    if (h != kErrNone) {
        int z = 0;
        cudaMemcpy(op->d_err.p, &z, sizeof(int), cudaMemcpyHostToDevice);
        return fail(QR_EKERNEL, "kernel reported error %d (%s)", h,
                    h == kErrMbarTimeout ? "bounded mbarrier wait expired"
                                         : "CSR position out of range");
    }
    return QR_OK;
}

}  // namespace

extern "C" {

int qr_op_create(int32_t n, uint64_t nterms, const uint64_t *x, const uint64_t *z,
                 const uint8_t *phase, const double *coeff, qr_op **out) {
    if (!out) return fail(QR_EINVAL, "qr_op_create: out is null");
    *out = nullptr;
    if (n < 1 || n > 63) return fail(QR_EINVAL, "qr_op_create: n=%d outside [1, 63]", n);
    if (nterms == 0)
        return fail(QR_EINVAL, "SparsePauliOp::new: at least one pauli must be supplied");
    if (nterms > 0xffffffffull) return fail(QR_EINVAL, "qr_op_create: too many terms");
    if (!x || !z || !phase || !coeff) return fail(QR_EINVAL, "qr_op_create: null term array");
    const uint64_t lim = (n == 64) ? ~0ull : ((1ull << n) - 1);
    for (uint64_t k = 0; k < nterms; ++k) {
        if ((x[k] & ~lim) || (z[k] & ~lim))
            return fail(QR_EINVAL, "qr_op_create: term %llu has mask bits beyond n=%d",
                        (unsigned long long)k, n);
        if (phase[k] > 3)
            return fail(QR_EINVAL, "qr_op_create: term %llu phase %u > 3", (unsigned long long)k,
                        (unsigned)phase[k]);
    }
    qr_op *op = new (std::nothrow) qr_op();
    if (!op) return fail(QR_ENOMEM, "qr_op_create: out of host memory");
    op->n = n;
    op->N = 1ull << n;
    op->T = nterms;
    cudaError_t e = cudaGetDevice(&op->device);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&op->nsm, cudaDevAttrMultiProcessorCount, op->device);
    if (e != cudaSuccess) {
        delete op;
        return cuda_fail(e, "qr_op_create: no usable CUDA device");
    }
    const int rc = create_tables(op, x, z, phase, coeff);
    if (rc) {
        delete op;
        return rc;
    }
    *out = op;
    return QR_OK;
}

int qr_op_destroy(qr_op *op) {
    if (!op) return QR_OK;
    int dev = -1;
    cudaGetDevice(&dev);
    const int home = op->device;
    if (dev != home) cudaSetDevice(home);
    if (op->hstream) cudaStreamDestroy(op->hstream);
    if (op->cstream) cudaStreamDestroy(op->cstream);
    if (op->cev) cudaEventDestroy(op->cev);
    delete op;
    if (dev >= 0 && dev != home) cudaSetDevice(dev);
    return QR_OK;
}

int qr_check(qr_op *op, void *stream) {
    if (!op) return fail(QR_EINVAL, "qr_check: null operator");
    int rc = check_device(op);
    if (rc) return rc;
    QR_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)), "qr_check sync");
    return check_kernel_error(op);
}

int qr_op_get_info(const qr_op *op_c, qr_op_info *info) {
    if (!op_c || !info) return fail(QR_EINVAL, "qr_op_get_info: null argument");
    qr_op *op = const_cast<qr_op *>(op_c);
    int rc = check_device(op);
    if (rc) return rc;
    rc = build_plan(op, QR_C64C, 0);
    if (rc) return rc;
    rc = build_plan(op, QR_C128, 0);
    if (rc) return rc;
    const Plan &pl = op->plans[QR_C64C][0];
    info->n = op->n;
    info->tile_bits = pl.b;
    info->nterms = op->T;
    info->ngroups = op->G;
    info->nmerged = op->M;
    info->nblocks = pl.nblocks;
    info->nfat = op->plans[QR_C128][0].nfat;
    info->nsub = pl.nsub;
    info->has_diag = pl.has_diag ? 1 : 0;
    info->device = op->device;
    return QR_OK;
}

int qr_op_get_groups(const qr_op *op, uint64_t *ngroups, uint64_t *gx, uint32_t *goff,
                     uint32_t *order, uint32_t *mmap) {
    if (!op || !ngroups) return fail(QR_EINVAL, "qr_op_get_groups: null argument");
    int rc = check_device(op);
    if (rc) return rc;
    *ngroups = op->G;
    QR_CUDA(cudaDeviceSynchronize(), "qr_op_get_groups sync");
    if (gx) std::memcpy(gx, op->gx.data(), op->G * sizeof(uint64_t));
    if (goff) std::memcpy(goff, op->goff.data(), (op->G + 1) * sizeof(uint32_t));
    if (order)
        QR_CUDA(cudaMemcpy(order, op->d_order.p, op->T * 4, cudaMemcpyDeviceToHost),
                "fetch term order");
    if (mmap)
        QR_CUDA(cudaMemcpy(mmap, op->d_mmap.p, op->T * 4, cudaMemcpyDeviceToHost),
                "fetch merged-string map");
    return QR_OK;
}

int qr_csr_size(const qr_op *op, uint64_t *nrows, uint64_t *nnz) {
    if (!op || !nrows || !nnz) return fail(QR_EINVAL, "qr_csr_size: null argument");
    *nrows = op->N;
    if (op->G != 0 && op->N > ~0ull / op->G) return fail(QR_EINVAL, "qr_csr_size: nnz overflows");
    *nnz = op->N * op->G;
    return QR_OK;
}

int qr_csr_build(qr_op *op, uint64_t *indptr, uint64_t *indices, double *data, int32_t mem,
                 void *stream) {
    if (!op || !indptr || !indices || !data) return fail(QR_EINVAL, "qr_csr_build: null argument");
    if (mem != QR_MEM_DEVICE && mem != QR_MEM_HOST)
        return fail(QR_EINVAL, "qr_csr_build: mem must be QR_MEM_DEVICE or QR_MEM_HOST");
    int rc = check_device(op);
    if (rc) return rc;
    rc = upload_csr_tables(op);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CsrArgs a;
    a.N = op->N;
    a.G = op->G;
    a.gx = op->d_gx.as<uint64_t>();
    a.n = op->n;
    a.grp = op->d_grp.as<CsrGroup>();
    a.pmask = op->d_pmask.as<uint64_t>();
    a.sig = op->d_sig.as<int32_t>();
    a.fold = op->d_fold.as<uint32_t>();
    a.nfold = op->nfold;
    a.ctab = op->d_ctab.as<double2>();
    a.pbeta = op->d_pbeta.as<uint64_t>();
    a.ptab = op->d_ptab.as<double2>();
    a.nctab = op->nctab;
    a.tz = op->d_tz.as<uint64_t>();
    a.tc = op->d_tc.as<double>();
    a.err = op->d_err.as<int>();
    a.wide = op->test_wide;
    a.fvals = nullptr;
    // fold-mode values buffer (nfold x rows) for the staged fill; without
    // it the fold entries are stored in place after the fill
    auto fold_buffer = [&](uint64_t rows) {
        a.fvals = nullptr;
        if (op->nfold == 0 || op->G > 256) return;
        if (op->d_fv.alloc((size_t)op->nfold * rows * sizeof(double2)) == cudaSuccess)
            a.fvals = op->d_fv.as<double2>();
        else
            (void)cudaGetLastError();  // allocation failure is not sticky: clear it
    };
    if (mem == QR_MEM_DEVICE) {
        fold_buffer(op->N);
        a.indptr = indptr;
        a.indices = indices;
        a.data = data;
        a.row0 = 0;
        a.nrows = op->N;
        QR_CUDA(launch_csr_fill(a, op->nsm, st), "csr fill launch");
        return QR_OK;
    }
    // host destination: build in row chunks of <= ~1 GiB on the device
    const uint64_t per_row = op->G * 24;
    uint64_t rows = (1ull << 30) / (per_row ? per_row : 1);
    // whole 256-row chunks, so that every launch starts on a chunk boundary
    rows = rows < 256 ? 256 : rows & ~255ull;
    if (rows > op->N) rows = op->N;
    DevBuf d_ptr, d_idx, d_dat;
    QR_CUDA(d_ptr.alloc((op->N + 1) * sizeof(uint64_t)), "alloc indptr staging");
    QR_CUDA(d_idx.alloc(rows * op->G * sizeof(uint64_t)), "alloc indices staging");
    QR_CUDA(d_dat.alloc(rows * op->G * 2 * sizeof(double)), "alloc data staging");
    fold_buffer(rows);
    for (uint64_t r0 = 0; r0 < op->N; r0 += rows) {
        const uint64_t nr = std::min(rows, op->N - r0);
        a.indptr = (r0 == 0) ? d_ptr.as<uint64_t>() : nullptr;
        a.indices = d_idx.as<uint64_t>();
        a.data = d_dat.as<double>();
        a.row0 = r0;
        a.nrows = nr;
        QR_CUDA(launch_csr_fill(a, op->nsm, st), "csr fill launch");
        QR_CUDA(cudaMemcpyAsync(indices + r0 * op->G, d_idx.p, nr * op->G * sizeof(uint64_t),
                                cudaMemcpyDeviceToHost, st),
                "copy indices");
        QR_CUDA(cudaMemcpyAsync(data + 2 * r0 * op->G, d_dat.p, nr * op->G * 2 * sizeof(double),
                                cudaMemcpyDeviceToHost, st),
                "copy data");
    }
    QR_CUDA(cudaMemcpyAsync(indptr, d_ptr.p, (op->N + 1) * sizeof(uint64_t),
                            cudaMemcpyDeviceToHost, st),
            "copy indptr");
    QR_CUDA(cudaStreamSynchronize(st), "csr build sync");
    return check_kernel_error(op);
}

static int apply_impl(const char *name, qr_op *op, int32_t dtype, const void *psi, void *y,
                      int32_t nstates, int32_t adjoint, void *stream, const void *v,
                      const double *alpha, const double *beta) {
    if (!op || !psi || !y) return fail(QR_EINVAL, "%s: null argument", name);
    if (dtype != QR_C128 && dtype != QR_C64C)
        return fail(QR_EINVAL, "%s: dtype must be QR_C128 or QR_C64C", name);
    if (nstates < 1) return fail(QR_EINVAL, "%s: nstates=%d < 1", name, nstates);
    if (adjoint != 0 && adjoint != 1) return fail(QR_EINVAL, "%s: adjoint must be 0 or 1", name);
    if (op->n > 40) return fail(QR_EINVAL, "%s: n=%d too large for a state vector", name, op->n);
    const size_t esz = dtype == QR_C128 ? 16 : 8;
    const uint64_t bytes = (uint64_t)nstates * op->N * esz;
    const char *pb = static_cast<const char *>(psi), *yb = static_cast<const char *>(y);
    if (pb < yb + bytes && yb < pb + bytes) return fail(QR_EINVAL, "%s: psi and y overlap", name);
    if ((reinterpret_cast<uintptr_t>(psi) | reinterpret_cast<uintptr_t>(y)) & 15)
        return fail(QR_EINVAL, "%s: psi and y must be 16-byte aligned", name);
    if (v) {
        // v is only read: it may be psi, or y itself (each element of y is
        // read by the thread that then writes it), but not a shifted view of y
        const char *vb = static_cast<const char *>(v);
        if (vb != yb && vb < yb + bytes && yb < vb + bytes)
            return fail(QR_EINVAL, "%s: v overlaps y without being y", name);
        if (reinterpret_cast<uintptr_t>(v) & 15)
            return fail(QR_EINVAL, "%s: v must be 16-byte aligned", name);
    }
    int rc = check_device(op);
    if (rc) return rc;
    rc = build_plan(op, dtype, adjoint);
    if (rc) return rc;
    const Plan &pl = op->plans[dtype][adjoint];
    ApplyArgs a{};
    a.psi = psi;
    a.y = y;
    a.N = op->N;
    a.n = op->n;
    a.b = pl.b;
    a.tb = pl.tb;
    a.nstates = nstates;
    a.ntiles = op->N >> pl.b;
    a.nitems = (uint64_t)nstates * a.ntiles;
    a.groups = pl.groups.as<GroupDesc>();
    a.tables = pl.tables.p;
    a.fat_z = pl.fat_z.as<uint64_t>();
    a.fat_c = pl.fat_c.p;
    a.blk_hi = pl.blk_hi.as<uint64_t>();
    a.blk_g0 = pl.blk_g0.as<uint32_t>();
    a.nblocks = pl.nblocks;
    a.diag = pl.has_diag ? pl.diag.p : nullptr;
    a.diag_block = pl.diag_block;
    a.err = op->d_err.as<int>();
    a.nsub = pl.nsub;
    a.tdesc = pl.tdesc.as<uint4>();
    a.tdata = pl.tdata.as<TileDataC64>();
    a.blk_r0 = pl.blk_r0.as<uint32_t>();
    a.run_g0 = pl.run_g0.as<uint32_t>();
    a.run_key = pl.run_key.as<uint32_t>();
    a.nruns = pl.nruns;
    a.chunks = pl.chunks.as<uint4>();
    a.nchunks = pl.nchunks;
    a.npairs = pl.npairs;
    a.wait_ns = op->test_wait_ns ? op->test_wait_ns : kDefaultWaitNs;
    a.withhold = op->test_withhold;
    a.wide = op->test_wide;
    a.v = v;
    if (v) {
        a.ar = alpha[0];
        a.ai = alpha[1];
        a.br = beta[0];
        a.bi = beta[1];
    }
    if (pl.nblocks == 0 && !v) {
        // operator without terms reachable here cannot happen (T >= 1); keep y defined
        QR_CUDA(cudaMemsetAsync(y, 0, bytes, static_cast<cudaStream_t>(stream)), "zero y");
        return QR_OK;
    }
    QR_CUDA(launch_apply(dtype, a, pl.amps, pl.threads, op->nsm,
                         static_cast<cudaStream_t>(stream)),
            "apply launch");
    return QR_OK;
}

int qr_apply(qr_op *op, int32_t dtype, const void *psi, void *y, int32_t nstates, int32_t adjoint,
             void *stream) {
    return apply_impl("qr_apply", op, dtype, psi, y, nstates, adjoint, stream, nullptr, nullptr,
                      nullptr);
}

int qr_apply_axpby(qr_op *op, int32_t dtype, const double *alpha, const void *psi,
                   const double *beta, const void *v, void *y, int32_t nstates, void *stream) {
    if (!alpha || !beta || !v) return fail(QR_EINVAL, "qr_apply_axpby: null argument");
    return apply_impl("qr_apply_axpby", op, dtype, psi, y, nstates, 0, stream, v, alpha, beta);
}

int qr_apply_host(qr_op *op, int32_t dtype, const void *psi_host, void *y_host, int32_t nstates,
                  int32_t adjoint) {
    if (!op || !psi_host || !y_host) return fail(QR_EINVAL, "qr_apply_host: null argument");
    if (dtype != QR_C128 && dtype != QR_C64C)
        return fail(QR_EINVAL, "qr_apply_host: dtype must be QR_C128 or QR_C64C");
    if (nstates < 1) return fail(QR_EINVAL, "qr_apply_host: nstates=%d < 1", nstates);
    int rc = check_device(op);
    if (rc) return rc;
    const size_t esz = dtype == QR_C128 ? 16 : 8;
    const uint64_t bytes = (uint64_t)nstates * op->N * esz;
    if (!op->hstream) QR_CUDA(cudaStreamCreateWithFlags(&op->hstream, cudaStreamNonBlocking),
                              "create stream");
    if (op->stage_in.bytes < bytes) QR_CUDA(op->stage_in.alloc(bytes), "alloc psi staging");
    // Pinned (page-locked, mapped) y: the kernel stores each finished output
    // tile straight into host memory, so the write-back overlaps the
    // computation instead of following it.  Pageable y: device staging + copy.
    void *y_dev = nullptr;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, y_host) == cudaSuccess && at.type == cudaMemoryTypeHost &&
        at.devicePointer != nullptr)
        y_dev = at.devicePointer;
    cudaGetLastError();  // a pageable pointer may leave a benign error behind
    if (!y_dev && op->stage_out.bytes < bytes)
        QR_CUDA(op->stage_out.alloc(bytes), "alloc y staging");
    const char *pb = static_cast<const char *>(psi_host);
    char *yb = static_cast<char *>(y_host);
    if (nstates > 1 && (pb + bytes <= yb || yb + bytes <= pb)) {
        // Several states, psi and y apart: state s + 1 is copied in on a
        // second stream while the kernel works on state s (an event orders
        // each state's kernel after its copy), so only the first copy is
        // not hidden.
        if (!op->cstream)
            QR_CUDA(cudaStreamCreateWithFlags(&op->cstream, cudaStreamNonBlocking), "create stream");
        if (!op->cev) QR_CUDA(cudaEventCreateWithFlags(&op->cev, cudaEventDisableTiming), "event");
        const uint64_t b1 = op->N * esz;
        char *in = static_cast<char *>(op->stage_in.p);
        char *out = static_cast<char *>(y_dev ? y_dev : op->stage_out.p);
        for (int32_t st = 0; st < nstates; ++st) {
            QR_CUDA(cudaMemcpyAsync(in + st * b1, pb + st * b1, b1, cudaMemcpyHostToDevice,
                                    op->cstream),
                    "copy psi to device");
            QR_CUDA(cudaEventRecord(op->cev, op->cstream), "record copy");
            QR_CUDA(cudaStreamWaitEvent(op->hstream, op->cev, 0), "order apply after copy");
            rc = qr_apply(op, dtype, in + st * b1, out + st * b1, 1, adjoint, op->hstream);
            if (rc) return rc;
            if (!y_dev)
                QR_CUDA(cudaMemcpyAsync(yb + st * b1, out + st * b1, b1, cudaMemcpyDeviceToHost,
                                        op->hstream),
                        "copy y to host");
        }
        QR_CUDA(cudaStreamSynchronize(op->hstream), "apply_host sync");
        return check_kernel_error(op);
    }
    QR_CUDA(cudaMemcpyAsync(op->stage_in.p, psi_host, bytes, cudaMemcpyHostToDevice, op->hstream),
            "copy psi to device");
    rc = qr_apply(op, dtype, op->stage_in.p, y_dev ? y_dev : op->stage_out.p, nstates, adjoint,
                  op->hstream);
    if (rc) return rc;
    if (!y_dev)
        QR_CUDA(cudaMemcpyAsync(y_host, op->stage_out.p, bytes, cudaMemcpyDeviceToHost,
                                op->hstream),
                "copy y to host");
    QR_CUDA(cudaStreamSynchronize(op->hstream), "apply_host sync");
    return check_kernel_error(op);
}

int qr_csr_spmv(uint64_t nrows, uint64_t ncols, const uint64_t *indptr, const uint64_t *indices,
                const double *data, const double *v, double *y, void *stream) {
    if (!indptr || !indices || !data || !v || !y) return fail(QR_EINVAL, "qr_csr_spmv: null argument");
    int dev = 0, nsm = 0;
    QR_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    QR_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev), "device attribute");
    QR_CUDA(launch_csr_spmv(nrows, ncols, indptr, indices, data, v, y, nsm,
                            static_cast<cudaStream_t>(stream)),
            "csr spmv launch");
    return QR_OK;
}

// ---------------------------------------------------------------- vector helpers
static int current_nsm(int *nsm) {
    int dev = 0;
    QR_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    QR_CUDA(cudaDeviceGetAttribute(nsm, cudaDevAttrMultiProcessorCount, dev), "device attribute");
    return QR_OK;
}

static int vec_call(const char *name, int op, int32_t dtype, uint64_t len, const void *x,
                    const void *y, void *z, const double *a, const double *b, double tol,
                    void *stream) {
    if (dtype != QR_C128 && dtype != QR_C64C)
        return fail(QR_EINVAL, "%s: dtype must be QR_C128 or QR_C64C", name);
    if (len == 0) return QR_OK;
    if (!x || !z || (op != 2 && !y) || !a) return fail(QR_EINVAL, "%s: null argument", name);
    int nsm = 0;
    int rc = current_nsm(&nsm);
    if (rc) return rc;
    QR_CUDA(launch_vec_op(op, dtype == QR_C64C, len, x, y, z, a, b, tol, nsm,
                          static_cast<cudaStream_t>(stream)),
            name);
    return QR_OK;
}

int qr_axpby(int32_t dtype, uint64_t len, const double *a, const void *x, const double *b,
             const void *y, void *z, void *stream) {
    if (len && !b) return fail(QR_EINVAL, "qr_axpby: null argument");
    return vec_call("qr_axpby", 0, dtype, len, x, y, z, a, b, 0.0, stream);
}

int qr_axpy(int32_t dtype, uint64_t len, const double *a, const void *x, const void *y, void *z,
            void *stream) {
    return vec_call("qr_axpy", 1, dtype, len, x, y, z, a, nullptr, 0.0, stream);
}

int qr_ax(int32_t dtype, uint64_t len, const double *a, const void *x, void *z, void *stream) {
    return vec_call("qr_ax", 2, dtype, len, x, nullptr, z, a, nullptr, 0.0, stream);
}

int qr_precond2(int32_t dtype, uint64_t len, const void *diag, const void *dx, const double *e,
                double tol, void *out, void *stream) {
    return vec_call("qr_precond2", 3, dtype, len, diag, dx, out, e, nullptr, tol, stream);
}

int qr_csr_diagonal(uint64_t nrows, uint64_t ncols, const uint64_t *indptr,
                    const uint64_t *indices, const double *data, double *out, void *stream) {
    const uint64_t nd = nrows < ncols ? nrows : ncols;
    if (nd == 0) return QR_OK;
    if (!indptr || !indices || !data || !out)
        return fail(QR_EINVAL, "qr_csr_diagonal: null argument");
    int nsm = 0;
    int rc = current_nsm(&nsm);
    if (rc) return rc;
    QR_CUDA(launch_csr_diag(nd, indptr, indices, data, out, nsm,
                            static_cast<cudaStream_t>(stream)),
            "csr diagonal launch");
    return QR_OK;
}

int qr_op_diagonal(qr_op *op, int32_t dtype, void *out, void *stream) {
    if (!op || !out) return fail(QR_EINVAL, "qr_op_diagonal: null argument");
    if (dtype != QR_C128 && dtype != QR_C64C)
        return fail(QR_EINVAL, "qr_op_diagonal: dtype must be QR_C128 or QR_C64C");
    int rc = check_device(op);
    if (rc) return rc;
    rc = upload_csr_tables(op);
    if (rc) return rc;
    // groups are sorted by x ascending, so an x = 0 group is group 0
    const uint32_t nt = (op->G > 0 && op->gx[0] == 0) ? op->goff[1] - op->goff[0] : 0;
    QR_CUDA(launch_op_diag(op->N, nt, op->d_tz.as<uint64_t>(), op->d_tc.as<double>(), out,
                           dtype == QR_C64C, op->nsm, static_cast<cudaStream_t>(stream)),
            "operator diagonal launch");
    return QR_OK;
}

// Merged coefficients and the built CSR tables from d_coef, on stream st.
static int recompute_coeffs(qr_op *op, cudaStream_t st) {
    QR_CUDA(launch_merge_coeffs((uint32_t)op->M, op->d_mm_off.as<uint32_t>(),
                                op->d_mm_terms.as<uint32_t>(), op->d_coef.as<double2>(),
                                op->d_ph.as<uint8_t>(), op->d_mc.as<double2>(), st),
            "merge coefficients");
    if (op->csr_ready) return refresh_csr_values(op, st);
    return QR_OK;
}

int qr_op_set_coeffs(qr_op *op, const double *coeff) {
    if (!op || !coeff) return fail(QR_EINVAL, "qr_op_set_coeffs: null argument");
    int rc = check_device(op);
    if (rc) return rc;
    QR_CUDA(cudaDeviceSynchronize(), "qr_op_set_coeffs sync");
    QR_CUDA(cudaMemcpy(op->d_coef.p, coeff, op->T * sizeof(cd), cudaMemcpyHostToDevice),
            "upload coefficients");
    rc = recompute_coeffs(op, nullptr);
    if (rc) return rc;
    op->host_coef_stale = true;  // plans built below fetch the new merged sums
    for (int d = 0; d < 2; ++d)
        for (int j = 0; j < 2; ++j) op->plans[d][j].built = false;
    // plans are rebuilt on next use into the buffers they already hold
    for (Plan &bp : op->bplans) bp.built = false;
    ++op->coef_gen;
    return QR_OK;
}

int qr_op_set_coeffs_device(qr_op *op, const double *coeff, void *stream) {
    if (!op || !coeff) return fail(QR_EINVAL, "qr_op_set_coeffs_device: null argument");
    int rc = check_device(op);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    QR_CUDA(cudaMemcpyAsync(op->d_coef.p, coeff, op->T * sizeof(cd), cudaMemcpyDeviceToDevice,
                            st),
            "copy device coefficients");
    rc = recompute_coeffs(op, st);
    if (rc) return rc;
    auto refresh = [&](Plan &pl) -> int {
        if (!pl.built) return QR_OK;
        QR_CUDA(launch_coef_program(pl.cslots.as<CoefSlot>(), pl.nslots, pl.cmem.as<uint32_t>(),
                                    pl.ccoord.as<uint8_t>(), op->d_mc.as<double2>(),
                                    op->d_madj.as<uint8_t>(), pl.adjoint, st),
                "coefficient program");
        if (pl.has_diag)
            QR_CUDA(launch_diag(pl.dtype, op->n, pl.dg_db, op->N >> pl.dg_db,
                                pl.dg_bz.as<uint64_t>(), pl.dg_boff.as<uint32_t>(), pl.dg_nbins,
                                pl.dg_tz.as<uint64_t>(), pl.dg_tc.as<double>(), pl.diag.p, st),
                    "diagonal kernel");
        return QR_OK;
    };
    for (int d = 0; d < 2; ++d)
        for (int j = 0; j < 2; ++j) {
            rc = refresh(op->plans[d][j]);
            if (rc) return rc;
        }
    for (Plan &bp : op->bplans) {
        rc = refresh(bp);
        if (rc) return rc;
    }
    op->host_coef_stale = true;
    return QR_OK;
}

int qr_op_set_test_hooks(qr_op *op, uint32_t flags, uint64_t wait_ns, int64_t withhold_step) {
    if (!op) return fail(QR_EINVAL, "qr_op_set_test_hooks: null operator");
    if (flags & ~(uint32_t)QR_TEST_FORCE_WIDE)
        return fail(QR_EINVAL, "qr_op_set_test_hooks: unknown flag bits 0x%x", flags);
    if (wait_ns != 0 && wait_ns < 1000000ull)
        return fail(QR_EINVAL, "qr_op_set_test_hooks: wait_ns below 1 ms");
    if (withhold_step < -1) return fail(QR_EINVAL, "qr_op_set_test_hooks: withhold_step < -1");
    op->test_wide = (flags & QR_TEST_FORCE_WIDE) ? 1 : 0;
    op->test_wait_ns = wait_ns;
    op->test_withhold = withhold_step;
    return QR_OK;
}

int qr_vdot(int32_t n, int32_t dtype, const void *a, const void *b, int32_t nstates, double *out,
            void *stream) {
    if (!a || !b || !out) return fail(QR_EINVAL, "qr_vdot: null argument");
    if (n < 1 || n > 40) return fail(QR_EINVAL, "qr_vdot: n=%d outside [1, 40]", n);
    if (dtype != QR_C128 && dtype != QR_C64C) return fail(QR_EINVAL, "qr_vdot: bad dtype");
    if (nstates < 1) return fail(QR_EINVAL, "qr_vdot: nstates=%d < 1", nstates);
    // one grid row per state (gridDim.y)
    if (nstates > 65535) return fail(QR_EINVAL, "qr_vdot: nstates=%d > 65535", nstates);
    int dev = 0, nsm = 0;
    QR_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    QR_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev), "device attribute");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const uint64_t N = 1ull << n;
    const uint32_t nblk = vdot_blocks(N, nsm);
    void *partial = nullptr;
    QR_CUDA(cudaMallocAsync(&partial, (size_t)nstates * nblk * sizeof(double2), st),
            "vdot scratch");
    cudaError_t e = launch_vdot(dtype, N, a, b, nstates, static_cast<double2 *>(partial), nblk,
                                reinterpret_cast<double2 *>(out), st);
    cudaFreeAsync(partial, st);
    if (e != cudaSuccess) return cuda_fail(e, "vdot launch");
    return QR_OK;
}

int qr_expect(qr_op *op, int32_t dtype, const void *psi, int32_t nstates, double *out,
              void *stream) {
    if (!op || !psi || !out) return fail(QR_EINVAL, "qr_expect: null argument");
    if (dtype != QR_C128 && dtype != QR_C64C) return fail(QR_EINVAL, "qr_expect: bad dtype");
    if (nstates < 1) return fail(QR_EINVAL, "qr_expect: nstates=%d < 1", nstates);
    if (nstates > 65535) return fail(QR_EINVAL, "qr_expect: nstates=%d > 65535", nstates);
    int rc = check_device(op);
    if (rc) return rc;
    const size_t esz = dtype == QR_C128 ? 16 : 8;
    const uint64_t bytes = (uint64_t)nstates * op->N * esz;
    if (op->expect_y.bytes < bytes) QR_CUDA(op->expect_y.alloc(bytes), "alloc expect buffer");
    rc = qr_apply(op, dtype, psi, op->expect_y.p, nstates, 0, stream);
    if (rc) return rc;
    return qr_vdot(op->n, dtype, psi, op->expect_y.p, nstates, out, stream);
}

int qr_term_grad(qr_op *op, int32_t dtype, const void *psi, const void *g, int32_t nstates,
                 double *out, void *stream) {
    if (!op || !psi || !g || !out) return fail(QR_EINVAL, "qr_term_grad: null argument");
    if (dtype != QR_C128 && dtype != QR_C64C) return fail(QR_EINVAL, "qr_term_grad: bad dtype");
    if (nstates < 1) return fail(QR_EINVAL, "qr_term_grad: nstates=%d < 1", nstates);
    if (op->n > 40) return fail(QR_EINVAL, "qr_term_grad: n=%d too large", op->n);
    int rc = check_device(op);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const uint32_t nstr = (uint32_t)op->M;
    if (dtype == QR_C64C && op->n >= 12) {
        if (!op->tg_ready) {
            // strings by partner tile, input order kept within one; batches
            // of <= 8 never span two partner tiles, largest first
            std::vector<uint32_t> ord(nstr);
            for (uint32_t i = 0; i < nstr; ++i) ord[i] = i;
            std::stable_sort(ord.begin(), ord.end(), [&](uint32_t a, uint32_t b) {
                return (op->mx[a] >> 12) < (op->mx[b] >> 12);
            });
            std::vector<uint64_t> sx(nstr), sz(nstr);
            for (uint32_t i = 0; i < nstr; ++i) {
                sx[i] = op->mx[ord[i]];
                sz[i] = op->mz[ord[i]];
            }
            std::vector<uint2> bat;
            for (uint32_t i = 0; i < nstr;) {
                uint32_t j = i + 1;
                while (j < nstr && j - i < 8 && (sx[j] >> 12) == (sx[i] >> 12)) ++j;
                bat.push_back(make_uint2(i, j - i));
                i = j;
            }
            std::stable_sort(bat.begin(), bat.end(),
                             [](const uint2 &a, const uint2 &b) { return a.y > b.y; });
            QR_CUDA(op->d_tg_x.upload(sx), "upload gradient strings");
            QR_CUDA(op->d_tg_z.upload(sz), "upload gradient strings");
            QR_CUDA(op->d_tg_perm.upload(ord), "upload gradient order");
            QR_CUDA(op->d_tg_bat.upload(bat), "upload gradient batches");
            op->tg_nbatch = (uint32_t)bat.size();
            op->tg_ready = true;
        }
        // about 8 work items per SM, chunks of at least 16 tiles
        const uint64_t TT = (op->N >> 12) * (uint64_t)nstates;
        uint64_t nchunk = ((uint64_t)op->nsm * 8 + op->tg_nbatch - 1) / op->tg_nbatch;
        if (nchunk > TT / 16) nchunk = TT / 16;
        if (nchunk < 1) nchunk = 1;
        void *scratch = nullptr;
        const size_t pbytes = (size_t)nstr * nchunk * sizeof(double2);
        QR_CUDA(cudaMallocAsync(&scratch, pbytes + (size_t)nstr * sizeof(double2) + 16, st),
                "term-grad scratch");
        double2 *partial = static_cast<double2 *>(scratch);
        double2 *R = partial + (size_t)nstr * nchunk;
        auto *counter = reinterpret_cast<unsigned long long *>(R + nstr);
        cudaError_t e = launch_term_grad_tiles(
            op->N, nstates, op->d_tg_x.as<uint64_t>(), op->d_tg_z.as<uint64_t>(),
            op->d_tg_perm.as<uint32_t>(), op->d_tg_bat.as<uint2>(), op->tg_nbatch, nstr, psi, g,
            partial, (uint32_t)nchunk, R, op->T, op->d_mmap.as<uint32_t>(), op->d_ph.as<uint8_t>(),
            reinterpret_cast<double2 *>(out), counter, op->nsm, st);
        cudaFreeAsync(scratch, st);
        if (e != cudaSuccess) return cuda_fail(e, "term-grad launch");
        return QR_OK;
    }
    // blocks take 4 strings each: enough chunks for ~8 blocks per SM
    const uint64_t nbatch = (nstr + 3) / 4;
    uint64_t nchunk = ((uint64_t)op->nsm * 8 + nbatch - 1) / nbatch;
    const uint64_t maxc = op->N >= 4096 ? op->N / 4096 : 1;
    if (nchunk > maxc) nchunk = maxc;
    if (nchunk < 1) nchunk = 1;
    const uint64_t chunk = (op->N + nchunk - 1) / nchunk;
    void *scratch = nullptr;
    const size_t pbytes = (size_t)nstr * nchunk * sizeof(double2);
    QR_CUDA(cudaMallocAsync(&scratch, pbytes + (size_t)nstr * sizeof(double2), st),
            "term-grad scratch");
    double2 *partial = static_cast<double2 *>(scratch);
    double2 *R = partial + (size_t)nstr * nchunk;
    cudaError_t e = launch_term_grad(dtype, op->N, nstates, op->d_mx.as<uint64_t>(),
                                     op->d_mz.as<uint64_t>(), nstr, psi, g, partial,
                                     (uint32_t)nchunk, chunk, R, op->T, op->d_mmap.as<uint32_t>(),
                                     op->d_ph.as<uint8_t>(), reinterpret_cast<double2 *>(out), st);
    cudaFreeAsync(scratch, st);
    if (e != cudaSuccess) return cuda_fail(e, "term-grad launch");
    return QR_OK;
}

}  // extern "C"

// tile width of the persistent batched kernel: 512 threads x 8 amplitudes
constexpr int kBatchTileBits = 12;

struct qr_batch {
    static constexpr int kForks = 4;  // parallel branches of the per-operator graph
    int device = 0, nsm = 0;
    std::vector<qr_op *> ops;
    std::vector<int32_t> nstates;
    int tile_bits = 0;
    // 0: one persistent work-list kernel, 1: graph of per-operator kernels,
    // 2: both in one graph -- the persistent kernel for the small operators
    // (fewer work items than half the SMs), one kernel per large operator
    int mode = 0;
    int force_mode = -1;  // -1: the autotuner chooses
    std::vector<char> sel;    // operators in the persistent kernel's work list
    std::vector<char> small;  // operators with fewer items than half the SMs
    DevBuf d_ops, d_items, d_ptrs, d_err;
    uint32_t nitems = 0;
    std::vector<const void *> cur_psi;
    std::vector<void *> cur_y;
    bool ptrs_changed = false;
    std::vector<uint64_t> gens;  // each operator's coef_gen when the graph was made
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cap = nullptr;
    cudaStream_t fork[kForks] = {};
    cudaEvent_t fork_ev[kForks + 1] = {};
};

namespace {

// Operator tables and the work list for tile width tb; items are ordered by
// decreasing per-tile work so the persistent CTAs' round-robin balances.
int batch_build(qr_batch *bt, int tb) {
    std::vector<BatchOp> bo(bt->ops.size());
    std::vector<std::pair<double, size_t>> cost;
    for (size_t i = 0; i < bt->ops.size(); ++i) {
        if (!bt->sel[i]) continue;  // applied by its own kernel (modes 1, 2)
        qr_op *op = bt->ops[i];
        int rc = build_plan(op, QR_C64C, 0, tb);
        if (rc) return rc;
        const Plan &pl = op->bplans[tb];
        BatchOp &o = bo[i];
        memset(&o, 0, sizeof(o));
        o.N = op->N;
        o.ntiles = op->N >> pl.b;
        o.b = pl.b;
        o.mcount = pl.amps;
        o.tact = pl.threads;
        o.diag_block = pl.diag_block;
        o.nblocks = pl.nblocks;
        o.nsub = pl.nsub;
        o.nruns = pl.nruns;
        o.nchunks = pl.nchunks;
        o.tdesc = pl.tdesc.as<uint4>();
        o.tdata = pl.tdata.as<TileDataC64>();
        o.blk_hi = pl.blk_hi.as<uint64_t>();
        o.blk_r0 = pl.blk_r0.as<uint32_t>();
        o.run_g0 = pl.run_g0.as<uint32_t>();
        o.run_key = pl.run_key.as<uint32_t>();
        o.chunks = pl.chunks.as<uint4>();
        o.diag = pl.has_diag ? pl.diag.as<float2>() : nullptr;
        // work per output tile: the sub-groups' inner steps plus per-block
        // bookkeeping, over the tile's amplitudes
        cost.push_back({(double)(pl.nsub + 2 * pl.nblocks + 4 * pl.nchunks) * (double)(1u << pl.b),
                        i});
    }
    std::stable_sort(cost.begin(), cost.end(),
                     [](const std::pair<double, size_t> &a, const std::pair<double, size_t> &b) {
                         return a.first > b.first;
                     });
    std::vector<BatchItem> items;
    for (auto &c : cost) {
        const size_t i = c.second;
        for (int32_t st = 0; st < bt->nstates[i]; ++st)
            for (uint64_t q = 0; q < bo[i].ntiles; ++q)
                items.push_back(BatchItem{(uint32_t)i, (uint32_t)st, (uint32_t)q, 0u});
    }
    if (items.size() > 0xffffffffull) return fail(QR_EINVAL, "qr_batch: work list too long");
    bt->nitems = (uint32_t)items.size();
    QR_CUDA(bt->d_ops.upload(bo), "upload batch operators");
    QR_CUDA(bt->d_items.upload(items), "upload batch work list");
    bt->tile_bits = tb;
    return QR_OK;
}

BatchArgs batch_args(qr_batch *bt) {
    BatchArgs a;
    a.ops = bt->d_ops.as<BatchOp>();
    a.items = bt->d_items.as<BatchItem>();
    a.nitems = bt->nitems;
    float2 **pp = bt->d_ptrs.as<float2 *>();
    a.psi = pp;
    a.y = pp + bt->ops.size();
    a.err = bt->d_err.as<int>();
    a.wait_ns = kDefaultWaitNs;
    return a;
}

int batch_upload_ptrs(qr_batch *bt, const void *const *psi, void *const *y, cudaStream_t st) {
    const size_t n = bt->ops.size();
    bool same = bt->cur_psi.size() == n;
    for (size_t i = 0; same && i < n; ++i) same = bt->cur_psi[i] == psi[i] && bt->cur_y[i] == y[i];
    if (same) return QR_OK;
    for (size_t i = 0; i < n; ++i) {
        if (!psi[i] || !y[i]) return fail(QR_EINVAL, "qr_batch_apply: null state pointer");
        if ((reinterpret_cast<uintptr_t>(psi[i]) | reinterpret_cast<uintptr_t>(y[i])) & 15)
            return fail(QR_EINVAL, "qr_batch_apply: states must be 16-byte aligned");
    }
    QR_CUDA(cudaStreamSynchronize(st), "qr_batch_apply sync before pointer update");
    std::vector<const void *> h(2 * n);
    for (size_t i = 0; i < n; ++i) {
        h[i] = psi[i];
        h[n + i] = y[i];
    }
    QR_CUDA(cudaMemcpy(bt->d_ptrs.p, h.data(), h.size() * sizeof(void *), cudaMemcpyHostToDevice),
            "upload batch pointers");
    bt->cur_psi.assign(psi, psi + n);
    bt->cur_y.assign(y, y + n);
    bt->ptrs_changed = true;
    return QR_OK;
}

// The batch's graph on the current pointers, on kForks parallel branches:
// the persistent work-list kernel over the selected operators (branch 0)
// and one compensated-c64 apply per other operator (round-robin over the
// remaining branches, or all of them when nothing is selected).  The
// selected operators' tables and work list (batch_build) and the other
// operators' plans must already exist.
int capture_graph(qr_batch *bt, cudaGraph_t *graph) {
    cudaStream_t cap = bt->cap;
    bool any_sel = false;
    for (char c : bt->sel) any_sel |= c != 0;
    QR_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeRelaxed), "begin capture");
    cudaError_t e = cudaEventRecord(bt->fork_ev[qr_batch::kForks], cap);
    for (int k = 0; k < qr_batch::kForks && e == cudaSuccess; ++k)
        e = cudaStreamWaitEvent(bt->fork[k], bt->fork_ev[qr_batch::kForks], 0);
    int rc = QR_OK;
    if (any_sel && e == cudaSuccess) e = launch_batch_c64c(batch_args(bt), bt->nsm, bt->fork[0]);
    const int first = any_sel ? 1 : 0, nbr = qr_batch::kForks - first;
    int k = 0;
    for (size_t i = 0; i < bt->ops.size() && e == cudaSuccess && !rc; ++i) {
        if (bt->sel[i]) continue;
        rc = apply_impl("qr_batch_apply", bt->ops[i], QR_C64C, bt->cur_psi[i], bt->cur_y[i],
                        bt->nstates[i], 0, bt->fork[first + (k++ % nbr)], nullptr, nullptr,
                        nullptr);
    }
    for (int f = 0; f < qr_batch::kForks && e == cudaSuccess; ++f) {
        e = cudaEventRecord(bt->fork_ev[f], bt->fork[f]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(cap, bt->fork_ev[f], 0);
    }
    cudaError_t e2 = cudaStreamEndCapture(cap, graph);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "batch graph capture");
    if (e2 != cudaSuccess) return cuda_fail(e2, "end capture");
    return QR_OK;
}

void drop_graph(qr_batch *bt) {
    if (bt->exec) cudaGraphExecDestroy(bt->exec);
    if (bt->graph) cudaGraphDestroy(bt->graph);
    bt->exec = nullptr;
    bt->graph = nullptr;
}

// Select the operators of a mode, build what the graph needs (work list
// and tables of the selected ones, plans of the others, uncaptured) and
// capture and instantiate it.
int instantiate_mode(qr_batch *bt, int mode) {
    drop_graph(bt);
    for (size_t i = 0; i < bt->ops.size(); ++i)
        bt->sel[i] = mode == 0 ? 1 : (mode == 1 ? 0 : bt->small[i]);
    int rc = batch_build(bt, kBatchTileBits);
    for (size_t i = 0; i < bt->ops.size() && !rc; ++i)
        if (!bt->sel[i]) rc = build_plan(bt->ops[i], QR_C64C, 0);
    if (!rc) rc = capture_graph(bt, &bt->graph);
    if (rc) return rc;
    QR_CUDA(cudaGraphInstantiate(&bt->exec, bt->graph, 0), "graph instantiate");
    bt->mode = mode;
    return QR_OK;
}

uint64_t graph_kernels(const qr_batch *bt) {
    uint64_t k = 0;
    bool any_sel = false;
    for (size_t i = 0; i < bt->ops.size(); ++i) {
        if (bt->sel[i]) any_sel = true;
        else ++k;
    }
    return k + (any_sel ? 1 : 0);
}

void record_gens(qr_batch *bt) {
    bt->gens.resize(bt->ops.size());
    for (size_t i = 0; i < bt->ops.size(); ++i) bt->gens[i] = bt->ops[i]->coef_gen;
}

// An operator's coefficients changed since the graph was made: its plan
// tables are rebuilt (outside any capture) and the graph made again.
int refresh_after_coeffs(qr_batch *bt, cudaStream_t st) {
    bool stale = bt->gens.size() != bt->ops.size();
    for (size_t i = 0; !stale && i < bt->ops.size(); ++i)
        stale = bt->gens[i] != bt->ops[i]->coef_gen;
    if (!stale) return QR_OK;
    QR_CUDA(cudaStreamSynchronize(st), "qr_batch_apply sync before plan rebuild");
    int rc = instantiate_mode(bt, bt->mode);
    if (!rc) record_gens(bt);
    return rc;
}

}  // namespace

extern "C" {

int qr_batch_create(int32_t nops, qr_op *const *ops, const int32_t *nstates, qr_batch **out) {
    if (!out || !ops || !nstates || nops < 1) return fail(QR_EINVAL, "qr_batch_create: bad arguments");
    *out = nullptr;
    int dev = -1;
    QR_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    for (int32_t i = 0; i < nops; ++i) {
        if (!ops[i]) return fail(QR_EINVAL, "qr_batch_create: null operator %d", i);
        if (ops[i]->device != dev)
            return fail(QR_ESTATE, "qr_batch_create: operator %d is on another device", i);
        if (ops[i]->n > 32) return fail(QR_EINVAL, "qr_batch_create: operator %d has n > 32", i);
        if (nstates[i] < 1) return fail(QR_EINVAL, "qr_batch_create: nstates[%d] < 1", i);
    }
    qr_batch *bt = new (std::nothrow) qr_batch();
    if (!bt) return fail(QR_ENOMEM, "qr_batch_create: out of host memory");
    bt->device = dev;
    bt->ops.assign(ops, ops + nops);
    bt->nstates.assign(nstates, nstates + nops);
    cudaError_t e = cudaDeviceGetAttribute(&bt->nsm, cudaDevAttrMultiProcessorCount, dev);
    bt->sel.assign(nops, 1);
    bt->small.assign(nops, 0);
    for (int32_t i = 0; i < nops; ++i) {
        const int b = std::min(ops[i]->n, kBatchTileBits);
        const uint64_t items = (ops[i]->N >> b) * (uint64_t)nstates[i];
        bt->small[i] = 2 * items <= (uint64_t)bt->nsm ? 1 : 0;
    }
    if (e == cudaSuccess) e = bt->d_ptrs.alloc(2 * (size_t)nops * sizeof(void *));
    if (e == cudaSuccess) e = bt->d_err.alloc(sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(bt->d_err.p, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&bt->cap, cudaStreamNonBlocking);
    for (int k = 0; k < qr_batch::kForks && e == cudaSuccess; ++k)
        e = cudaStreamCreateWithFlags(&bt->fork[k], cudaStreamNonBlocking);
    for (int k = 0; k <= qr_batch::kForks && e == cudaSuccess; ++k)
        e = cudaEventCreateWithFlags(&bt->fork_ev[k], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        delete bt;
        return cuda_fail(e, "qr_batch_create");
    }
    *out = bt;
    return QR_OK;
}

int qr_batch_destroy(qr_batch *bt) {
    if (!bt) return QR_OK;
    if (bt->cap) cudaStreamSynchronize(bt->cap);
    drop_graph(bt);
    for (auto &f : bt->fork)
        if (f) cudaStreamDestroy(f);
    for (auto &ev : bt->fork_ev)
        if (ev) cudaEventDestroy(ev);
    if (bt->cap) cudaStreamDestroy(bt->cap);
    delete bt;
    return QR_OK;
}

int qr_batch_tile_bits(const qr_batch *bt) { return bt ? bt->tile_bits : 0; }

int qr_batch_mode(const qr_batch *bt) { return bt && bt->exec ? bt->mode : -1; }

int qr_batch_set_mode(qr_batch *bt, int32_t mode) {
    if (!bt || mode < -1 || mode > 2) return fail(QR_EINVAL, "qr_batch_set_mode: bad arguments");
    if (bt->exec) return fail(QR_ESTATE, "qr_batch_set_mode: the first apply has already chosen");
    bt->force_mode = mode;
    return QR_OK;
}

int qr_batch_apply(qr_batch *bt, const void *const *psi, void *const *y, void *stream) {
    if (!bt || !psi || !y) return fail(QR_EINVAL, "qr_batch_apply: null argument");
    int dev = -1;
    QR_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev != bt->device) return fail(QR_ESTATE, "qr_batch_apply: wrong current device");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int rc = batch_upload_ptrs(bt, psi, y, st);
    if (rc) return rc;
    if (bt->exec) {
        rc = refresh_after_coeffs(bt, st);
        if (rc) return rc;
    }
    if (bt->exec && bt->mode != 0 && bt->ptrs_changed) {
        // per-operator graph nodes carry the state pointers: capture again
        rc = instantiate_mode(bt, bt->mode);
        if (rc) return rc;
    }
    bt->ptrs_changed = false;
    if (!bt->exec) {
        // autotuner: time each form on these buffers (one warm-up, three
        // timed launches of its graph) -- the persistent work-list kernel,
        // a graph of one kernel per operator, and, when the batch has both
        // small and large operators, the persistent kernel for the small
        // ones beside per-operator kernels for the large ones
        bool any_small = false, any_large = false;
        for (char c : bt->small) (c ? any_small : any_large) = true;
        std::vector<int> cands;
        if (bt->force_mode >= 0) cands.push_back(bt->force_mode);
        else {
            cands = {0, 1};
            if (any_small && any_large) cands.push_back(2);
        }
        int best = -1;
        float best_ms = 0.f;
        cudaEvent_t e0, e1;
        QR_CUDA(cudaEventCreate(&e0), "event");
        QR_CUDA(cudaEventCreate(&e1), "event");
        for (int m : cands) {
            rc = instantiate_mode(bt, m);
            if (rc) break;
            if (cands.size() == 1) {
                best = m;
                break;
            }
            cudaError_t e = cudaGraphLaunch(bt->exec, bt->cap);
            if (e == cudaSuccess) e = cudaEventRecord(e0, bt->cap);
            for (int k = 0; k < 3 && e == cudaSuccess; ++k) e = cudaGraphLaunch(bt->exec, bt->cap);
            if (e == cudaSuccess) e = cudaEventRecord(e1, bt->cap);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            float ms = 0.f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
            if (e != cudaSuccess) {
                rc = cuda_fail(e, "qr_batch autotune");
                break;
            }
            if (best < 0 || ms < best_ms) {
                best = m;
                best_ms = ms;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (rc) return rc;
        if (bt->mode != best) {
            rc = instantiate_mode(bt, best);
            if (rc) return rc;
        }
        bt->tile_bits = kBatchTileBits;
        record_gens(bt);
        QR_CUDA(cudaStreamSynchronize(bt->cap), "autotune sync");
        int h = 0;
        QR_CUDA(cudaMemcpy(&h, bt->d_err.p, sizeof(int), cudaMemcpyDeviceToHost), "error word");
        if (h) return fail(QR_EKERNEL, "batched kernel reported error %d", h);
        for (qr_op *op : bt->ops) {
            rc = check_kernel_error(op);
            if (rc) return rc;
        }
    }
    QR_CUDA(cudaGraphLaunch(bt->exec, st), "graph launch");
    count_launch(graph_kernels(bt));  // kernels the graph runs
    return QR_OK;
}

int qr_last_error(char *buf, size_t len) {
    const int L = (int)g_err.size();
    if (buf && len > 0) {
        size_t c = std::min(len - 1, g_err.size());
        memcpy(buf, g_err.data(), c);
        buf[c] = '\0';
    }
    return L;
}

uint64_t qr_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

}  // extern "C"
