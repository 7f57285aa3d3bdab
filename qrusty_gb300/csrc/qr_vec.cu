// qr_vec.cu -- the vector helpers of qrusty's eigensolver loop, on sm_103a.
//
//   axpby  z = a x + b y      qrusty/src/accel.rs:374-379
//   axpy   z = a x + y        qrusty/src/accel.rs:381-386
//   ax     z = a x            qrusty/src/accel.rs:388-393
//   precond2  out = dx / reg(diag - e, tol)      pyqrusty/src/lib.rs:457-469
//             (reg :436-440)
//   precond   the same with diag = SpMat.diagonal()   pyqrusty/src/lib.rs:442-455
//   SpMat.diagonal()          pyqrusty/src/lib.rs:118-125 (sprs diag().to_dense())
//   the operator's diagonal without a CSR (the x = 0 terms folded in input
//   order, exactly the value make_row places in column r of row r).
//
// complex128 arithmetic is num-complex 0.4's, operation for operation, with
// every multiply, add and divide an explicit round-to-nearest intrinsic so
// the compiler cannot contract a * b + c into one FMA (Rust never does):
//   a * b = (ar br - ai bi, ar bi + ai br)
//   a / b = ((ar br + ai bi) / (br^2 + bi^2), (ai br - ar bi) / (br^2 + bi^2))
// complex64 runs the same sequence in FP32 with the scalars rounded to float.
//
// All element-wise kernels are HBM-bound streams: grid-stride over 16-byte
// elements (one complex128 or two complex64), four elements in flight per
// thread, grid = 8 CTAs of 256 threads per SM.
#include "../../include/qrusty_gpu.h"
#include "qr_common.cuh"

namespace qr {

namespace {

constexpr int kVecThreads = 256;
constexpr int kVecUnroll = 4;

enum VecOp { kAxpby = 0, kAxpy = 1, kAx = 2, kPrecond = 3 };

struct VecScalars {
    double ar, ai, br, bi;  // a, b (axpby / axpy / ax); e for precond
    double tol;
};

template <typename R> struct C2;
template <> struct C2<double> {
    using T = double2;
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
    static __device__ __forceinline__ double norm(double a, double b) { return hypot(a, b); }
};
template <> struct C2<float> {
    using T = float2;
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
    static __device__ __forceinline__ float norm(float a, float b) { return hypotf(a, b); }
};

template <typename R>
__device__ __forceinline__ typename C2<R>::T cmul(R ar, R ai, typename C2<R>::T x) {
    using O = C2<R>;
    typename C2<R>::T r;
    r.x = O::sub(O::mul(ar, x.x), O::mul(ai, x.y));
    r.y = O::add(O::mul(ar, x.y), O::mul(ai, x.x));
    return r;
}

template <typename R, int OP>
__device__ __forceinline__ typename C2<R>::T vec_elem(typename C2<R>::T x, typename C2<R>::T y,
                                                      R ar, R ai, R br, R bi, R tol) {
    using O = C2<R>;
    typename C2<R>::T r;
    if (OP == kAx) return cmul<R>(ar, ai, x);
    if (OP == kAxpy) {
        r = cmul<R>(ar, ai, x);
        r.x = O::add(r.x, y.x);
        r.y = O::add(r.y, y.y);
        return r;
    }
    if (OP == kAxpby) {
        const typename C2<R>::T u = cmul<R>(ar, ai, x), v = cmul<R>(br, bi, y);
        r.x = O::add(u.x, v.x);
        r.y = O::add(u.y, v.y);
        return r;
    }
    // precond: x = diag, y = dx, (ar, ai) = e
    R dr = O::sub(x.x, ar), di = O::sub(x.y, ai);
    if (O::norm(dr, di) < tol) {
        dr = tol;
        di = R(0);
    }
    const R ns = O::add(O::mul(dr, dr), O::mul(di, di));
    r.x = O::div(O::add(O::mul(y.x, dr), O::mul(y.y, di)), ns);
    r.y = O::div(O::sub(O::mul(y.y, dr), O::mul(y.x, di)), ns);
    return r;
}

// complex128: one element per 16-byte word.
template <int OP>
__global__ void __launch_bounds__(kVecThreads) vec_c128(uint64_t len, const double2 *__restrict__ x,
                                                        const double2 *__restrict__ y,
                                                        double2 *z, VecScalars s) {
    const uint64_t stride = (uint64_t)gridDim.x * kVecThreads;
    uint64_t i = blockIdx.x * (uint64_t)kVecThreads + threadIdx.x;
    const bool Y = OP != kAx;
    for (; i + (kVecUnroll - 1) * stride < len; i += kVecUnroll * stride) {
        double2 xv[kVecUnroll], yv[kVecUnroll];
#pragma unroll
        for (int u = 0; u < kVecUnroll; ++u) {
            xv[u] = __ldcs(x + i + u * stride);
            yv[u] = Y ? __ldcs(y + i + u * stride) : make_double2(0.0, 0.0);
        }
#pragma unroll
        for (int u = 0; u < kVecUnroll; ++u)
            __stcs(z + i + u * stride,
                   vec_elem<double, OP>(xv[u], yv[u], s.ar, s.ai, s.br, s.bi, s.tol));
    }
    for (; i < len; i += stride) {
        const double2 yv = Y ? y[i] : make_double2(0.0, 0.0);
        z[i] = vec_elem<double, OP>(x[i], yv, s.ar, s.ai, s.br, s.bi, s.tol);
    }
}

// complex64: two elements per 16-byte word (all three pointers 16-byte
// aligned and len even; the host sends anything else to vec_c64_scalar).
template <int OP>
__global__ void __launch_bounds__(kVecThreads) vec_c64(uint64_t npair, const float4 *__restrict__ x,
                                                       const float4 *__restrict__ y, float4 *z,
                                                       VecScalars s) {
    const float ar = (float)s.ar, ai = (float)s.ai, br = (float)s.br, bi = (float)s.bi,
                tol = (float)s.tol;
    const uint64_t stride = (uint64_t)gridDim.x * kVecThreads;
    const bool Y = OP != kAx;
    for (uint64_t i = blockIdx.x * (uint64_t)kVecThreads + threadIdx.x; i < npair; i += stride) {
        const float4 xv = __ldcs(x + i);
        const float4 yv = Y ? __ldcs(y + i) : make_float4(0.f, 0.f, 0.f, 0.f);
        const float2 lo = vec_elem<float, OP>(make_float2(xv.x, xv.y), make_float2(yv.x, yv.y), ar,
                                              ai, br, bi, tol);
        const float2 hi = vec_elem<float, OP>(make_float2(xv.z, xv.w), make_float2(yv.z, yv.w), ar,
                                              ai, br, bi, tol);
        __stcs(z + i, make_float4(lo.x, lo.y, hi.x, hi.y));
    }
}

template <int OP>
__global__ void __launch_bounds__(kVecThreads) vec_c64_scalar(uint64_t len, const float2 *x,
                                                              const float2 *y, float2 *z,
                                                              VecScalars s) {
    const float ar = (float)s.ar, ai = (float)s.ai, br = (float)s.br, bi = (float)s.bi,
                tol = (float)s.tol;
    for (uint64_t i = blockIdx.x * (uint64_t)kVecThreads + threadIdx.x; i < len;
         i += (uint64_t)gridDim.x * kVecThreads) {
        const float2 yv = OP != kAx ? y[i] : make_float2(0.f, 0.f);
        z[i] = vec_elem<float, OP>(x[i], yv, ar, ai, br, bi, tol);
    }
}

unsigned vec_grid(uint64_t units, int nsm) {
    const uint64_t want = (units + kVecThreads - 1) / kVecThreads;
    const uint64_t cap = (uint64_t)(nsm > 0 ? nsm : 1) * 8;
    return (unsigned)(want < cap ? (want ? want : 1) : cap);
}

template <int OP>
cudaError_t launch_vec(int f32, uint64_t len, const void *x, const void *y, void *z,
                       const VecScalars &s, int nsm, cudaStream_t st) {
    if (len == 0) return cudaSuccess;
    if (!f32) {
        vec_c128<OP><<<vec_grid(len, nsm), kVecThreads, 0, st>>>(
            len, static_cast<const double2 *>(x), static_cast<const double2 *>(y),
            static_cast<double2 *>(z), s);
    } else {
        const bool aligned = ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y) |
                               reinterpret_cast<uintptr_t>(z)) & 15u) == 0 && (len & 1) == 0;
        if (aligned) {
            vec_c64<OP><<<vec_grid(len / 2, nsm), kVecThreads, 0, st>>>(
                len / 2, static_cast<const float4 *>(x), static_cast<const float4 *>(y),
                static_cast<float4 *>(z), s);
        } else {
            vec_c64_scalar<OP><<<vec_grid(len, nsm), kVecThreads, 0, st>>>(
                len, static_cast<const float2 *>(x), static_cast<const float2 *>(y),
                static_cast<float2 *>(z), s);
        }
    }
    count_launch();
    return cudaGetLastError();
}

// Diagonal of a CSR matrix (rows sorted or not): one warp per row, the first
// stored entry whose column equals the row, else 0 -- sprs diag().to_dense()
// for matrices whose rows hold each column at most once.
__global__ void __launch_bounds__(256) csr_diag_kernel(uint64_t nd, const uint64_t *indptr,
                                                       const uint64_t *indices,
                                                       const double2 *data, double2 *out) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t w0 = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t r = w0; r < nd; r += nw) {
        const uint64_t lo = indptr[r], hi = indptr[r + 1];
        double2 v = make_double2(0.0, 0.0);
        for (uint64_t j = lo; j < hi; j += 32) {
            const bool hit = j + lane < hi && indices[j + lane] == r;
            const uint32_t m = __ballot_sync(0xffffffffu, hit);
            if (m) {
                v = data[j + (__ffs(m) - 1)];
                break;
            }
        }
        if (lane == 0) out[r] = v;
    }
}

// Operator diagonal: the t1 - t0 terms with x = 0 (input order), folded per
// row as make_row folds them: v = s_0 c'_0, then v = v + s_k c'_k, with
// s_k = -1 when popc(r & z_k) is odd (negation of both parts).  Terms are
// staged through shared memory in chunks; each thread owns rows.
constexpr int kDiagChunk = 512;

__global__ void __launch_bounds__(256) op_diag_kernel(uint64_t N, uint32_t nt, const uint64_t *tz,
                                                      const double2 *tc, void *out, int f32) {
    __shared__ uint64_t s_z[kDiagChunk];
    __shared__ double2 s_c[kDiagChunk];
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    // every thread of the block runs the same number of outer iterations so
    // the chunk barriers stay uniform
    const uint64_t base0 = blockIdx.x * (uint64_t)blockDim.x;
    for (uint64_t base = base0; base < N; base += stride) {
        const uint64_t r = base + threadIdx.x;
        double vr = 0.0, vi = 0.0;
        for (uint32_t c0 = 0; c0 < nt; c0 += kDiagChunk) {
            const uint32_t cn = min((uint32_t)kDiagChunk, nt - c0);
            __syncthreads();
            for (uint32_t k = threadIdx.x; k < cn; k += blockDim.x) {
                s_z[k] = tz[c0 + k];
                s_c[k] = tc[c0 + k];
            }
            __syncthreads();
            for (uint32_t k = 0; k < cn; ++k) {
                const bool neg = (__popcll(r & s_z[k]) & 1) != 0;
                const double cr = neg ? -s_c[k].x : s_c[k].x;
                const double ci = neg ? -s_c[k].y : s_c[k].y;
                if (c0 + k == 0) {
                    vr = cr;
                    vi = ci;
                } else {
                    vr = __dadd_rn(vr, cr);
                    vi = __dadd_rn(vi, ci);
                }
            }
        }
        if (r < N) {
            if (f32)
                static_cast<float2 *>(out)[r] = make_float2((float)vr, (float)vi);
            else
                static_cast<double2 *>(out)[r] = make_double2(vr, vi);
        }
    }
}

}  // namespace

cudaError_t launch_vec_op(int op, int f32, uint64_t len, const void *x, const void *y, void *z,
                          const double *a, const double *b, double tol, int nsm, cudaStream_t st) {
    VecScalars s{};
    if (a) {
        s.ar = a[0];
        s.ai = a[1];
    }
    if (b) {
        s.br = b[0];
        s.bi = b[1];
    }
    s.tol = tol;
    switch (op) {
        case kAxpby: return launch_vec<kAxpby>(f32, len, x, y, z, s, nsm, st);
        case kAxpy: return launch_vec<kAxpy>(f32, len, x, y, z, s, nsm, st);
        case kAx: return launch_vec<kAx>(f32, len, x, y, z, s, nsm, st);
        case kPrecond: return launch_vec<kPrecond>(f32, len, x, y, z, s, nsm, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_csr_diag(uint64_t nd, const uint64_t *indptr, const uint64_t *indices,
                            const double *data, double *out, int nsm, cudaStream_t st) {
    if (nd == 0) return cudaSuccess;
    uint64_t blocks = (nd * 32 + 255) / 256;
    const uint64_t cap = (uint64_t)nsm * 8;
    if (blocks > cap) blocks = cap;
    csr_diag_kernel<<<(unsigned)blocks, 256, 0, st>>>(nd, indptr, indices,
                                                      reinterpret_cast<const double2 *>(data),
                                                      reinterpret_cast<double2 *>(out));
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_op_diag(uint64_t N, uint32_t nt, const uint64_t *tz, const double *tc, void *out,
                           int f32, int nsm, cudaStream_t st) {
    if (N == 0) return cudaSuccess;
    uint64_t blocks = (N + 255) / 256;
    const uint64_t cap = (uint64_t)nsm * 8;
    if (blocks > cap) blocks = cap;
    op_diag_kernel<<<(unsigned)blocks, 256, 0, st>>>(N, nt, tz,
                                                     reinterpret_cast<const double2 *>(tc), out, f32);
    count_launch();
    return cudaGetLastError();
}

}  // namespace qr
