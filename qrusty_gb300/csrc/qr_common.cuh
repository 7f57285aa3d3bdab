// qr_common.cuh -- internal types shared by the host layer and the kernels
// of libqrusty_gpu (not part of the public C ABI in include/qrusty_gpu.h).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace qr {

// Largest rank of a group's z-difference span that qr_apply evaluates with
// a 2^d-entry table; groups above it are evaluated term by term ("fat").
constexpr int kDMax = 4;
constexpr uint32_t kFat = 0xffffffffu;

// One x-group of the apply plan.  All terms of the group share the x mask;
// their z masks are z0 ^ delta_k with delta_k in span(beta[0..d)).  The
// group's diagonal factor at row r is
//   D(r) = (-1)^popc(r & z0) * table[off + pi(r)],  pi(r)_i = popc(r & beta_i) & 1.
// Fat groups (d == kFat) list their cnt terms at fat_z/fat_c[off ...].
struct alignas(16) GroupDesc {
    uint64_t z0;
    uint64_t beta[kDMax];
    uint32_t lo;    // x & (tile - 1): XOR partner inside the partner tile
    uint32_t d;     // rank, or kFat
    uint32_t off;   // table offset (entries) or fat-term offset
    uint32_t cnt;   // fat-term count
};

template <typename Real> struct Cplx;
template <> struct alignas(8) Cplx<float> { float re, im; };
template <> struct alignas(16) Cplx<double> { double re, im; };

// Per-sub-group data of the per-tile table of the compensated-c64 kernel:
// the masks' tile-index parts (>> b) and the FP32 table T[u] of the factor.
struct alignas(16) TileDataC64 {
    uint64_t z0h, b0h, b1h, pad;
    float2 T[4];
};
static_assert(sizeof(TileDataC64) == 64, "TileDataC64 is read as four 16-byte words");

struct ApplyArgs {
    const void *psi;
    void *y;
    uint64_t N;             // 2^n amplitudes per state
    int n;
    int b;                  // tile bits
    int tb;                 // log2(threads)
    int nstates;
    uint64_t ntiles;        // N >> b
    uint64_t nitems;        // nstates * ntiles
    const GroupDesc *groups;
    const void *tables;     // Cplx<Real>
    const uint64_t *fat_z;
    const void *fat_c;      // Cplx<Real>
    const uint64_t *blk_hi; // partner-tile XOR per block
    const uint32_t *blk_g0; // groups of block j: [blk_g0[j], blk_g0[j+1])
    uint32_t nblocks;
    const void *diag;       // Cplx<Real>[N] or null (only read in block hi == 0)
    int diag_block;         // index of the hi == 0 block, or -1
    int *err;               // device error word
    // compensated-c64 plan: sub-groups (see qr_apply.cu)
    uint32_t nsub;
    // per-tile-table kernel: per sub-group a 16-byte thread descriptor
    // {partner byte-offset XOR | pair half << 15 | tvar << 31, z0_t, beta0_t,
    //  beta1_t} (the thread-bit parts of z0 and of the basis) and its
    // TileDataC64; sub-groups of a block (or pair of blocks) in runs of
    // equal key
    const uint4 *tdesc;
    const TileDataC64 *tdata;
    const uint32_t *blk_r0;   // runs of block (pair) j: [blk_r0[j], blk_r0[j+1])
    const uint32_t *run_g0;   // sub-groups of run r: [run_g0[r], run_g0[r+1])
    const uint32_t *run_key;  // key = zm | xm << 4 | tv << 5 (factor depends on the thread);
                              // pair plans: 64 + (zm | bb << 3 | xm << 5 | tv << 6) for
                              // runs of fused sub-group pairs
    uint32_t nruns;
    // chunks of consecutive blocks with at most kTabCap sub-groups:
    // {first sub-group, first run, first block, 0}, nchunks + 1 entries
    const uint4 *chunks;
    uint32_t nchunks;
    // > 0: partner blocks visited in pairs (blocks 2p, 2p+1 in one ring slot
    // of two stages); blk_r0 then indexes pairs and tdesc bit 15 is the half
    uint32_t npairs;
    // fused epilogue y = alpha * (H psi) + beta * v when v != nullptr
    const void *v;
    double ar, ai, br, bi;
    // bound of every mbarrier wait (ns); 2 s unless a test shortens it
    uint64_t wait_ns;
    // test hook (qr_op_set_test_hooks): the ring step whose partner-tile copy
    // CTA 0 never issues, so that its wait runs out; -1 = none
    int64_t withhold;
    // 64-bit row words (the n > 32 instantiations) forced at any n (test hook)
    int wide;
    // paired kernel: ring slots of two partner tiles (set by the launcher)
    uint32_t pair_slots;
};



// One operator of a batched compensated-c64 launch (device copy): the
// per-tile-table plan of the operator (no partner-tile pairs) and its tile
// geometry.
struct BatchOp {
    uint64_t N, ntiles;
    int32_t b, mcount, tact, diag_block;  // tile bits, amplitudes / threads used, x = 0 block
    uint32_t nblocks, nsub, nruns, nchunks;
    const uint4 *tdesc;
    const TileDataC64 *tdata;
    const uint64_t *blk_hi;
    const uint32_t *blk_r0, *run_g0, *run_key;
    const uint4 *chunks;
    const float2 *diag;
};
struct BatchItem {
    uint32_t op, state, tile, pad;
};
struct BatchArgs {
    const BatchOp *ops;
    const BatchItem *items;  // sorted by decreasing work per tile
    uint32_t nitems;
    const float2 *const *psi;  // per operator: its first state; state s at + s * N
    float2 *const *y;
    int *err;
    uint64_t wait_ns;          // bound of every mbarrier wait
};
cudaError_t launch_batch_c64c(const BatchArgs &a, int nsm, cudaStream_t st);

// One entry of a plan's coefficient program (qr_op_set_coeffs_device): the
// value(s) at dst computed from merged strings [m0, m0 + cnt) of the plan's
// coefficients c_m (the merged coefficients, or for an adjoint plan
// conj(c_m) (-1)^popc(x_m & z_m)).  kind 0: 2^d FP32 table entries (float2),
// entry u = the fold from 0 of +-c_m in member order, sign (-1)^popc(u &
// coord_m); kind 1: the same in FP64 (double2); kind 2: c_m itself (double2,
// cnt = 1).  The additions are those of the host plan builder, in its order.
struct CoefSlot {
    uint64_t dst;
    uint32_t m0;
    uint16_t cnt;
    uint8_t d, kind;
};
static_assert(sizeof(CoefSlot) == 16, "CoefSlot layout");

// qr_coef.cu
cudaError_t launch_merge_coeffs(uint32_t M, const uint32_t *mm_off, const uint32_t *mm_terms,
                                const double2 *coeff, const uint8_t *phase, double2 *mc,
                                cudaStream_t st);
cudaError_t launch_coef_program(const CoefSlot *slots, uint32_t nslots, const uint32_t *mem,
                                const uint8_t *coord, const double2 *mc, const uint8_t *madj,
                                int adjoint, cudaStream_t st);

// c'_k = m(phase_k) * c_k (make_params, qrusty/src/accel.rs:141-157):
// m = (1, -i, -1, +i)[phase], num-complex's product (ar br - ai bi,
// ar bi + ai br) with every operation rounded on its own (no FMA).
__device__ __forceinline__ double2 make_param(double2 b, uint32_t phase) {
    const uint32_t ph = phase & 3u;
    const double ar = ph == 0 ? 1.0 : (ph == 2 ? -1.0 : 0.0);
    const double ai = ph == 1 ? -1.0 : (ph == 3 ? 1.0 : 0.0);
    return make_double2(__dsub_rn(__dmul_rn(ar, b.x), __dmul_rn(ai, b.y)),
                        __dadd_rn(__dmul_rn(ar, b.y), __dmul_rn(ai, b.x)));
}

// Device error codes written to the error word.
enum : int { kErrNone = 0, kErrMbarTimeout = 1, kErrCsrPos = 2 };

// num-complex 0.4 arithmetic with every operation an explicit round-to-nearest
// intrinsic (no FMA contraction): a * b = (ar br - ai bi, ar bi + ai br).
// a*x + b*y is the axpby of qrusty/src/accel.rs:374-379.
__device__ __forceinline__ double2 cx_axpby(double ar, double ai, double2 x, double br, double bi,
                                            double2 y) {
    const double ur = __dsub_rn(__dmul_rn(ar, x.x), __dmul_rn(ai, x.y));
    const double ui = __dadd_rn(__dmul_rn(ar, x.y), __dmul_rn(ai, x.x));
    const double vr = __dsub_rn(__dmul_rn(br, y.x), __dmul_rn(bi, y.y));
    const double vi = __dadd_rn(__dmul_rn(br, y.y), __dmul_rn(bi, y.x));
    return make_double2(__dadd_rn(ur, vr), __dadd_rn(ui, vi));
}
__device__ __forceinline__ float2 cx_axpby(float ar, float ai, float2 x, float br, float bi,
                                           float2 y) {
    const float ur = __fsub_rn(__fmul_rn(ar, x.x), __fmul_rn(ai, x.y));
    const float ui = __fadd_rn(__fmul_rn(ar, x.y), __fmul_rn(ai, x.x));
    const float vr = __fsub_rn(__fmul_rn(br, y.x), __fmul_rn(bi, y.y));
    const float vi = __fadd_rn(__fmul_rn(br, y.y), __fmul_rn(bi, y.x));
    return make_float2(__fadd_rn(ur, vr), __fadd_rn(ui, vi));
}

// sub-groups of one per-tile factor table of the compensated-complex64 kernel
constexpr uint32_t kTabCap = 512;

// log2 of the thread count of the compensated-complex64 kernels (the
// single-operator kernels and the batched kernel, see qr_apply.cu).
constexpr int kC64ThreadBits = 9;

// Records msg as the calling thread's last error (qr_last_error) and returns code.
int set_error(int code, const char *msg);

// Per-process launch counter (all launches issued through this library).
void count_launch(uint64_t k = 1);

// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) for kernel fn on the
// current device, only when `bytes` exceeds what was set before: steady-state
// launches (and launches inside a stream capture) make no attribute calls.
cudaError_t ensure_dyn_smem(const void *fn, size_t bytes);

// Kernel launchers (qr_apply.cu / qr_csr.cu).
cudaError_t launch_apply(int dtype, const ApplyArgs &a, int amps, int threads, int nsm,
                         cudaStream_t st);
cudaError_t launch_diag(int dtype, int n, int db, uint64_t ntiles, const uint64_t *bin_zlo,
                        const uint32_t *bin_off, uint32_t nbins, const uint64_t *tz,
                        const double *tc, void *out, cudaStream_t st);

// CSR fill.  Per group g (x masks ascending): the sigma values of its
// position formula, and either a class table -- the term-order fold of
// the group's +-c'_k for each of the 2^(d+1) sign classes of a row, class
// bit 0 = parity(r & z0), bit j+1 = parity(r & beta_j) -- or, when the z
// span has rank > kCsrMaxRank, the term range to fold per row.
constexpr int kCsrMaxRank = 4;
constexpr uint32_t kCsrFold = 0xffffffffu;
// Fold-mode groups: the longest leading run of terms whose z differences
// span rank <= kCsrPrefixRank is folded per class on the host (table of
// 2^(rank+1) entries); rows add only the terms after it.
constexpr int kCsrPrefixRank = 10;
struct CsrGroup {
    uint64_t z0;
    uint64_t beta[kCsrMaxRank];
    uint32_t d;       // rank of the z differences, or kCsrFold
    uint32_t tab;     // first class-table entry (2^(d+1) entries)
    uint32_t zparts;  // fold mode: bit 0 every c'_k.re is +-0, bit 1 every c'_k.im is +-0
    uint32_t pre;     // fold mode: prefix terms (bits 0-23) folded per class, prefix rank << 24
    uint32_t k0, k1;  // terms [k0, k1) in group-stable order (fold mode)
};
static_assert(sizeof(CsrGroup) == 64, "CsrGroup layout");

struct CsrArgs {
    uint64_t N, G;
    int n;                    // qubits: row bits
    const uint64_t *gx;       // G, ascending
    const CsrGroup *grp;      // G
    const uint64_t *pmask;    // G: bits b with a nonzero sigma_{g,b}
    const int32_t *sig;       // G x n: sigma_{g,b} (0 where b is not in pmask)
    const uint32_t *fold;     // groups in fold mode
    uint32_t nfold;
    const double2 *ctab;      // class tables
    uint32_t nctab;           // class-table entries
    const uint64_t *tz;       // terms in group-stable order (fold mode)
    const double *tc;         // 2 doubles per term
    const uint64_t *pbeta;    // nfold x kCsrPrefixRank: prefix span bases (fold mode)
    const double2 *ptab;      // prefix class tables (fold mode)
    double2 *fvals;           // nfold x nrows fold-mode values, or null (written in place)
    uint64_t *indptr, *indices;
    double *data;
    uint64_t row0, nrows;     // rows to fill
    int *err;                 // device error word (bad position => kErrCsrPos)
    int wide;                 // 64-bit row words (the n > 32 kernels) forced (test hook)
};
cudaError_t launch_csr_fill(const CsrArgs &a, int nsm, cudaStream_t st);

// qr_group.cu: term grouping on the device.  Buffers sized for T terms (the
// group counts are bounded by T).
struct TermGroupsOut {
    uint32_t *order;     // T: input index of each term, stably sorted by x (CSR order)
    uint64_t *tz;        // T: z of the terms in CSR order
    uint64_t *gx;        // G: distinct x, ascending
    uint32_t *goff;      // G + 1: CSR group g = terms [goff[g], goff[g + 1]) in CSR order
    uint32_t *mmap;      // T: merged string of each input term
    uint32_t *mm_off;    // M + 1: merged string m folds terms mm_terms[mm_off[m] ..]
    uint32_t *mm_terms;  // T: input indices, per merged string in input order
    uint64_t *mx, *mz;   // M: merged strings, first-occurrence order
    uint8_t *madj;       // M: popc(x & z) & 1 (adjoint sign)
    uint32_t *ag_off;    // Ga + 1: x-groups of the merged strings (first-occurrence order)
    uint32_t *ag_mem;    // M: merged indices per x-group, ascending
};
struct TermGroupCounts {
    uint64_t G = 0, M = 0, Ga = 0;
};
// Synchronises st; returns the counts.
cudaError_t group_terms(int n, uint64_t T, const uint64_t *x, const uint64_t *z,
                        const TermGroupsOut &o, TermGroupCounts *cnt, cudaStream_t st);

struct CsrStructOut {
    uint64_t *pmask;  // G
    int32_t *sig;     // G x n
    CsrGroup *grp;    // G
    uint16_t *coord;  // T: span coordinates of each term (CSR order)
    uint32_t *fold;   // <= G: fold-mode groups
    uint64_t *pbeta;  // <= G x kCsrPrefixRank
};
struct CsrStructCounts {
    uint64_t nctab = 0, nptab = 0;
    uint32_t nfold = 0;
};
// Mask-only CSR tables; synchronises st and returns the table sizes.
cudaError_t csr_structure(int n, uint64_t G, const uint64_t *gx, const uint32_t *goff,
                          const uint64_t *tz, const CsrStructOut &o, CsrStructCounts *cnt,
                          cudaStream_t st);
// Coefficient-dependent CSR tables (tc, zero-part flags, class and prefix
// tables) from the raw coefficients: stream-ordered, no synchronisation.
cudaError_t csr_values(uint64_t G, uint64_t T, const uint32_t *order, const double2 *coef,
                       const uint8_t *phase, double2 *tc, CsrGroup *grp, const uint16_t *coord,
                       double2 *ctab, double2 *ptab, cudaStream_t st);
cudaError_t launch_csr_spmv(uint64_t nrows, uint64_t ncols, const uint64_t *indptr,
                            const uint64_t *indices, const double *data, const double *v,
                            double *y, int nsm, cudaStream_t st);

// qr_vec.cu (op: 0 axpby, 1 axpy, 2 ax, 3 precond2)
cudaError_t launch_vec_op(int op, int f32, uint64_t len, const void *x, const void *y, void *z,
                          const double *a, const double *b, double tol, int nsm, cudaStream_t st);
cudaError_t launch_csr_diag(uint64_t nd, const uint64_t *indptr, const uint64_t *indices,
                            const double *data, double *out, int nsm, cudaStream_t st);
cudaError_t launch_op_diag(uint64_t N, uint32_t nt, const uint64_t *tz, const double *tc, void *out,
                           int f32, int nsm, cudaStream_t st);

// qr_reduce.cu
uint32_t vdot_blocks(uint64_t N, int nsm);
cudaError_t launch_vdot(int dtype, uint64_t N, const void *a, const void *b, int nstates,
                        double2 *partial, uint32_t nblk, double2 *out, cudaStream_t st);
cudaError_t launch_term_grad(int dtype, uint64_t N, int nstates, const uint64_t *sx,
                             const uint64_t *sz, uint32_t nstr, const void *psi, const void *g,
                             double2 *partial, uint32_t nchunk, uint64_t chunk, double2 *R,
                             uint64_t T, const uint32_t *map, const uint8_t *phase, double2 *out,
                             cudaStream_t st);
// Tiled complex64 term gradients (n >= 12): strings sorted by partner tile
// x >> 12 (sx, sz; perm = merged index of each), batches of <= 8 strings of
// one partner tile as (first, count), largest first; partial holds nstr x
// nchunk entries; counter: 8 bytes of device scratch (the work counter).
cudaError_t launch_term_grad_tiles(uint64_t N, int nstates, const uint64_t *sx, const uint64_t *sz,
                                   const uint32_t *perm, const uint2 *batches, uint32_t nbatch,
                                   uint32_t nstr, const void *psi, const void *g,
                                   double2 *partial, uint32_t nchunk, double2 *R, uint64_t T,
                                   const uint32_t *map, const uint8_t *phase, double2 *out,
                                   unsigned long long *counter, int nsm, cudaStream_t st);

}  // namespace qr
