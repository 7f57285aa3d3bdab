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

// Rank of column r ^ x_g in row r: g + sum of sigma_{g,b} over the bits b
// of r in the group's position mask (sig: the group's row of the table).
__device__ __forceinline__ int32_t csr_pos(uint64_t r, uint32_t g, uint64_t pm,
                                           const int32_t *sig) {
    int32_t pos = (int32_t)g;
    for (uint64_t m = r & pm; m; m &= m - 1) pos += sig[__ffsll((long long)m) - 1];
    return pos;
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
__device__ __forceinline__ uint32_t csr_class(const CsrGroup &d, uint64_t r) {
    uint32_t c = (uint32_t)__popcll(r & d.z0) & 1u;
#pragma unroll
    for (int j = 0; j < kCsrMaxRank; ++j)
        if ((uint32_t)j < d.d) c |= ((uint32_t)__popcll(r & d.beta[j]) & 1u) << (j + 1);
    return c;
}

constexpr int kCsrThreads = 256;
constexpr uint32_t kCsrSmemSig = 12288;  // sigma entries staged in shared memory (48 KB)

// Class-table groups.  G <= 256: thread t owns group g = t % G of row t / G
// in every pass of 256 / G consecutive rows, so its descriptor and position
// mask stay in registers and no per-entry division is needed.  G > 256: one
// row per pass, threads stride the groups.  Fold-mode groups are left to
// csr_fold_kernel, so no lane of a warp waits on another's long fold.
__global__ void __launch_bounds__(kCsrThreads) csr_fill_kernel(const CsrArgs a) {
    extern __shared__ int32_t s_sig[];
    const uint32_t G = (uint32_t)a.G;
    const uint64_t nsig = (uint64_t)G * (uint32_t)a.n;
    const bool staged = nsig <= kCsrSmemSig;
    if (staged)
        for (uint32_t i = threadIdx.x; i < nsig; i += kCsrThreads) s_sig[i] = a.sig[i];
    __syncthreads();
    const int32_t *sig = staged ? s_sig : a.sig;
    if (G <= (uint32_t)kCsrThreads) {
        const uint32_t rpp = kCsrThreads / G;
        const uint32_t t = threadIdx.x;
        if (t >= rpp * G) return;  // no barrier follows
        const uint32_t rs = t / G, g = t - rs * G;
        const CsrGroup d = a.grp[g];
        if (d.d == kCsrFold) return;
        const uint64_t xg = a.gx[g], pm = a.pmask[g];
        const int32_t *sg = sig + (size_t)g * (uint32_t)a.n;
        const uint64_t npass = (a.nrows + rpp - 1) / rpp;
        for (uint64_t p = blockIdx.x; p < npass; p += gridDim.x) {
            const uint64_t rr = p * rpp + rs;
            if (rr >= a.nrows) break;
            const uint64_t r = a.row0 + rr;
            csr_store(a, rr, csr_pos(r, g, pm, sg), r ^ xg, a.ctab[d.tab + csr_class(d, r)]);
        }
    } else {
        for (uint64_t rr = blockIdx.x; rr < a.nrows; rr += gridDim.x) {
            const uint64_t r = a.row0 + rr;
            for (uint32_t g = threadIdx.x; g < G; g += kCsrThreads) {
                const CsrGroup d = a.grp[g];
                if (d.d == kCsrFold) continue;
                const int32_t pos = csr_pos(r, g, a.pmask[g], sig + (size_t)g * (uint32_t)a.n);
                csr_store(a, rr, pos, r ^ a.gx[g], a.ctab[d.tab + csr_class(d, r)]);
            }
        }
    }
}

// Fold-mode groups (z span wider than kCsrMaxRank): one thread per row, all
// lanes of a warp on the same group, the group's +-c'_k folded in input-term
// order from the first term (make_row's fold), terms read warp-uniformly.
__global__ void __launch_bounds__(kCsrThreads) csr_fold_kernel(const CsrArgs a) {
    for (uint32_t f = blockIdx.y; f < a.nfold; f += gridDim.y) {
        const uint32_t g = a.fold[f];
        const CsrGroup d = a.grp[g];
        const uint64_t xg = a.gx[g], pm = a.pmask[g];
        const int32_t *sg = a.sig + (size_t)g * (uint32_t)a.n;
        for (uint64_t rr = blockIdx.x * (uint64_t)kCsrThreads + threadIdx.x; rr < a.nrows;
             rr += (uint64_t)gridDim.x * kCsrThreads) {
            const uint64_t r = a.row0 + rr;
            const uint32_t k0 = d.k0, k1 = d.k1;
            const bool neg0 = (__popcll(r & a.tz[k0]) & 1) != 0;
            double vr = neg0 ? -a.tc[2 * k0] : a.tc[2 * k0];
            double vi = neg0 ? -a.tc[2 * k0 + 1] : a.tc[2 * k0 + 1];
            for (uint32_t k = k0 + 1; k < k1; ++k) {
                const bool neg = (__popcll(r & a.tz[k]) & 1) != 0;
                vr = __dadd_rn(vr, neg ? -a.tc[2 * k] : a.tc[2 * k]);
                vi = __dadd_rn(vi, neg ? -a.tc[2 * k + 1] : a.tc[2 * k + 1]);
            }
            csr_store(a, rr, csr_pos(r, g, pm, sg), r ^ xg, make_double2(vr, vi));
        }
    }
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
    const uint64_t rpp = a.G <= (uint64_t)kCsrThreads ? (uint64_t)kCsrThreads / a.G : 1;
    uint64_t g = (a.nrows + rpp - 1) / rpp;
    if (g > (uint64_t)nsm * 8) g = (uint64_t)nsm * 8;
    const uint64_t nsig = a.G * (uint64_t)a.n;
    const size_t smem = nsig <= kCsrSmemSig ? (size_t)nsig * sizeof(int32_t) : 0;
    csr_fill_kernel<<<(unsigned)g, kCsrThreads, smem, st>>>(a);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || a.nfold == 0) return e;
    uint64_t gx = (a.nrows + kCsrThreads - 1) / kCsrThreads;
    const uint32_t gy = a.nfold < 65535u ? a.nfold : 65535u;
    uint64_t cap = ((uint64_t)nsm * 8 + gy - 1) / gy;
    if (cap < 1) cap = 1;
    if (gx > cap) gx = cap;
    csr_fold_kernel<<<dim3((unsigned)gx, gy), kCsrThreads, 0, st>>>(a);
    count_launch();
    return cudaGetLastError();
}

// y = A v, complex128.  One warp per row; lanes stride the row's entries and
// the partial sums are combined with a butterfly.  Replaces
// spmat_dot_densevec (qrusty/src/accel.rs:338-370).
__global__ void __launch_bounds__(256) csr_spmv_kernel(uint64_t nrows, uint64_t ncols,
                                                       const uint64_t *indptr,
                                                       const uint64_t *indices,
                                                       const double2 *data, const double2 *v,
                                                       double2 *y) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x / 32);
    for (uint64_t r = blockIdx.x * (uint64_t)(blockDim.x / 32) + (threadIdx.x / 32); r < nrows;
         r += warps) {
        const uint64_t j0 = indptr[r], j1 = indptr[r + 1];
        double sr = 0.0, si = 0.0;
        for (uint64_t j = j0 + lane; j < j1; j += 32) {
            const uint64_t c = indices[j];
            if (c >= ncols) continue;  // out-of-range column: skipped
            const double2 d = data[j];
            const double2 x = v[c];
            sr = fma(d.x, x.x, fma(-d.y, x.y, sr));
            si = fma(d.x, x.y, fma(d.y, x.x, si));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sr += __shfl_xor_sync(0xffffffffu, sr, o);
            si += __shfl_xor_sync(0xffffffffu, si, o);
        }
        if (lane == 0) y[r] = make_double2(sr, si);
    }
}

cudaError_t launch_csr_spmv(uint64_t nrows, uint64_t ncols, const uint64_t *indptr,
                            const uint64_t *indices, const double *data, const double *v,
                            double *y, int nsm, cudaStream_t st) {
    if (nrows == 0) return cudaSuccess;
    uint64_t g = (nrows + 7) / 8;
    if (g > (uint64_t)nsm * 32) g = (uint64_t)nsm * 32;
    csr_spmv_kernel<<<(unsigned)g, 256, 0, st>>>(nrows, ncols, indptr, indices,
                                                 reinterpret_cast<const double2 *>(data),
                                                 reinterpret_cast<const double2 *>(v),
                                                 reinterpret_cast<double2 *>(y));
    count_launch();
    return cudaGetLastError();
}

}  // namespace qr
