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
#include "qr_common.cuh"

namespace qr {

__global__ void __launch_bounds__(256) csr_indptr_kernel(uint64_t N, uint64_t G,
                                                         uint64_t *indptr) {
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r <= N;
         r += (uint64_t)gridDim.x * blockDim.x)
        indptr[r] = r * G;
}

__global__ void __launch_bounds__(256) csr_fill_kernel(const CsrArgs a) {
    const uint64_t total = a.nrows * a.G;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < total;
         e += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t rr = e / a.G;
        const uint64_t g = e - rr * a.G;
        const uint64_t r = a.row0 + rr;
        int64_t pos = (int64_t)g;
        for (uint32_t k = a.eoff[g]; k < a.eoff[g + 1]; ++k)
            if ((r >> a.ebit[k]) & 1ull) pos += a.esig[k];
        // left fold in input-term order; first term taken as-is
        const uint32_t k0 = a.goff[g], k1 = a.goff[g + 1];
        double vr, vi;
        {
            const bool neg = (__popcll(r & a.tz[k0]) & 1) != 0;
            vr = neg ? -a.tc[2 * k0] : a.tc[2 * k0];
            vi = neg ? -a.tc[2 * k0 + 1] : a.tc[2 * k0 + 1];
        }
        for (uint32_t k = k0 + 1; k < k1; ++k) {
            const bool neg = (__popcll(r & a.tz[k]) & 1) != 0;
            const double cr = neg ? -a.tc[2 * k] : a.tc[2 * k];
            const double ci = neg ? -a.tc[2 * k + 1] : a.tc[2 * k + 1];
            vr = __dadd_rn(vr, cr);
            vi = __dadd_rn(vi, ci);
        }
        if (pos < 0 || (uint64_t)pos >= a.G) {  // cannot happen for a valid trie table
            atomicExch(a.err, kErrCsrPos);
            continue;
        }
        const uint64_t o = rr * a.G + (uint64_t)pos;
        a.indices[o] = r ^ a.gx[g];
        reinterpret_cast<double2 *>(a.data)[o] = make_double2(vr, vi);
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
    const uint64_t total = a.nrows * a.G;
    if (total == 0) return cudaSuccess;
    uint64_t g = (total + 255) / 256;
    if (g > (uint64_t)nsm * 16) g = (uint64_t)nsm * 16;
    csr_fill_kernel<<<(unsigned)g, 256, 0, st>>>(a);
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
