/*
 * qrusty_gpu.h -- C ABI of the GB300 (sm_103a) Pauli-operator hot path.
 *
 * Drop-in boundary for qrusty's rowwise SparsePauliOp -> CSR construction
 * and for the Pauli-sum product H*psi.  Plain pointers and sizes only; no
 * CUDA, C++ or torch types appear in the signatures (streams are passed as
 * `void*` holding a cudaStream_t, NULL = the legacy default stream).
 *
 * Conventions
 *  - Every function returns QR_OK (0) or a negative QR_E* code and never
 *    aborts; qr_last_error() returns the message of the calling thread's
 *    last failure.
 *  - Terms are (x, z, phase, coeff) exactly as qrusty's make_params consumes
 *    them (qrusty/src/accel.rs:141-157): bit q of x is set for X/Y on qubit
 *    q, bit q of z for Y/Z, phase = (base_phase + #Y) mod 4 with base_phase
 *    from the label prefix (qrusty/src/lib.rs:125-181).  Matrix entry
 *    (r, r ^ x) of a term is c' * (-1)^popcount(r & z) with
 *    c' = (1, -i, -1, +i)[phase] * coeff.
 *  - Complex numbers are interleaved (re, im): complex128 = 2 doubles,
 *    complex64 = 2 floats.
 *  - Device pointers are raw CUDA allocations on the device the operator
 *    was created on.  Host pointers may be pageable or pinned.
 *  - A handle must not be used by two host threads at once.
 *  - Calls taking a stream are asynchronous with respect to the host unless
 *    stated otherwise.
 */
#ifndef QRUSTY_GPU_H
#define QRUSTY_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    QR_OK = 0,
    QR_EINVAL = -1,   /* bad argument (sizes, masks, phase, null pointer)   */
    QR_ECUDA = -2,    /* a CUDA runtime call failed                         */
    QR_ENOMEM = -3,   /* device or host allocation failed                   */
    QR_EKERNEL = -4,  /* a kernel reported an error (bounded wait expired)  */
    QR_ESTATE = -5    /* wrong device / handle state                        */
};

enum { QR_MEM_DEVICE = 0, QR_MEM_HOST = 1 };

/* Arithmetic of qr_apply: plain complex128, or complex64 amplitudes with
 * FP32 arithmetic and compensated (two-sum) accumulation. */
enum { QR_C128 = 0, QR_C64C = 1 };

typedef struct qr_op qr_op;

typedef struct {
    int32_t n;            /* qubits                                        */
    int32_t tile_bits;    /* amplitude-tile width used by qr_apply         */
    uint64_t nterms;      /* input terms, in input order                   */
    uint64_t ngroups;     /* distinct x masks (= nnz per CSR row)          */
    uint64_t nmerged;     /* distinct (x, z) strings after FP64 merging    */
    uint64_t nblocks;     /* distinct partner tiles x >> tile_bits         */
    uint64_t nfat;        /* complex128 plan: groups evaluated term by term */
    uint64_t nsub;        /* complex64 plan: rank <= 2 sub-groups          */
    int32_t has_diag;     /* x = 0 group held as a precomputed diagonal    */
    int32_t device;       /* CUDA device the operator lives on             */
} qr_op_info;

/* Create an operator from T terms (replaces SparsePauliOp::new,
 * qrusty/src/lib.rs:354-376, plus make_params, qrusty/src/accel.rs:141-157).
 * Validates 1 <= n <= 63, T >= 1, masks within n bits, phase <= 3.
 * Uploads the terms to the current CUDA device and groups them there
 * (qr_op_get_groups); synchronous.  The grouping kernels run on the legacy
 * default stream with scratch from the stream-ordered allocator, so, like
 * cudaMalloc, this is not to be called while a stream of the device is
 * being captured into a CUDA graph. */
int qr_op_create(int32_t n, uint64_t nterms, const uint64_t *x, const uint64_t *z,
                 const uint8_t *phase, const double *coeff, qr_op **out);

/* Release the operator and its device memory (synchronous). */
int qr_op_destroy(qr_op *op);

int qr_op_get_info(const qr_op *op, qr_op_info *info);

/* The operator's term grouping, computed on the device at creation by a
 * stable radix sort on x (replaces the per-row sort by x of make_row,
 * qrusty/src/accel.rs:188-208, and the merging of equal (x, z) strings of
 * the FP64 simplification).  *ngroups receives the number of groups; the
 * host buffers, each may be NULL (a first call with all NULL sizes them):
 *   gx[ngroups]       distinct x masks, ascending (the CSR column groups);
 *   goff[ngroups + 1] group g is order[goff[g] .. goff[g + 1]);
 *   order[nterms]     input index of each term, stably sorted by x;
 *   mmap[nterms]      merged (x, z) string of each input term, the strings
 *                     numbered in order of first occurrence.
 * Synchronous. */
int qr_op_get_groups(const qr_op *op, uint64_t *ngroups, uint64_t *gx, uint32_t *goff,
                     uint32_t *order, uint32_t *mmap);

/* CSR size of the operator's matrix (replaces the nnz pass of
 * make_unsafe_vectors_chunked, qrusty/src/accel.rs:309-319):
 * nrows = 2^n, nnz = nrows * ngroups. */
int qr_csr_size(const qr_op *op, uint64_t *nrows, uint64_t *nnz);

/* Fill caller-owned CSR arrays: indptr[nrows+1], indices[nnz],
 * data[2*nnz] (complex128).  Replaces make_unsafe_vectors_chunked
 * (qrusty/src/accel.rs:267-336) / to_matrix_rowwise_unsafe_chunked
 * (qrusty/src/lib.rs:558-571): per row, columns r ^ x ascending, values
 * summed over equal columns in input-term order, explicit zeros kept.
 * mem = QR_MEM_DEVICE: device pointers, asynchronous on `stream`
 * (16-byte aligned indices/data take the staged bulk-store path).
 * mem = QR_MEM_HOST: host pointers; built on the device and copied back,
 * synchronous.
 * Groups whose z masks span rank > 4 are folded per row into a value
 * buffer of (such groups) x rows x 16 bytes kept with the operator: the
 * first call that needs it (or a larger one) allocates it, so that call
 * synchronises the device; qr_op_destroy frees it. */
int qr_csr_build(qr_op *op, uint64_t *indptr, uint64_t *indices, double *data,
                 int32_t mem, void *stream);

/* y = H psi (adjoint = 0) or y = H^dagger psi (adjoint = 1) for nstates
 * state vectors stored back to back (state s at offset s * 2^n).
 * Replaces CSR build + spmat_dot_densevec (qrusty/src/accel.rs:338-370)
 * with a matrix-free kernel.  dtype = QR_C128 (double2) or QR_C64C
 * (float2).  psi and y are device pointers and must not overlap.
 * QR_C128 computes in FP64 throughout.  QR_C64C keeps amplitudes and
 * products in FP32 and accumulates each amplitude's sum with compensated
 * (two-sum) additions; its relative error against the FP64 result is about
 * 2.5e-7 on a 26-qubit, 10,000-term operator (the tests bound it by 1e-6). */
int qr_apply(qr_op *op, int32_t dtype, const void *psi, void *y, int32_t nstates,
             int32_t adjoint, void *stream);

/* y = alpha * (H psi) + beta * v, fused into the apply kernel's store: the
 * eigensolver residual H psi - theta psi (alpha = 1, beta = -theta, v = psi)
 * without a second pass over y.  alpha, beta: host (re, im) doubles.  The
 * combination is qrusty's axpby (qrusty/src/accel.rs:374-379) applied to
 * the value qr_apply would store, with num-complex arithmetic (complex128) or
 * its FP32 form (QR_C64C), so the result equals qr_apply followed by
 * qr_axpby bit for bit.  v may be psi or y itself (not a shifted view of y);
 * y must not overlap psi. */
int qr_apply_axpby(qr_op *op, int32_t dtype, const double *alpha, const void *psi,
                   const double *beta, const void *v, void *y, int32_t nstates, void *stream);

/* Synchronise `stream` and report any error a kernel of this operator
 * recorded on the device (e.g. an expired bounded wait).  The error word is
 * cleared after it is reported. */
int qr_check(qr_op *op, void *stream);

/* As qr_apply with HOST psi / y (synchronous): copies psi to a device
 * staging buffer and applies.  When y is page-locked host memory
 * (cudaHostAlloc / cudaHostRegister) the kernel writes each output tile
 * straight into it, overlapping the write-back with the computation;
 * otherwise y goes to a device staging buffer and is copied back.  With
 * several states whose host ranges of psi and y do not overlap, the copy of
 * state s + 1 runs on a second stream while state s is computed.  Staging
 * buffers are owned by the operator and reused across calls. */
int qr_apply_host(qr_op *op, int32_t dtype, const void *psi_host, void *y_host,
                  int32_t nstates, int32_t adjoint);

/* y = A v for a CSR matrix given by device arrays (replaces
 * spmat_dot_densevec, qrusty/src/accel.rs:338-370, and its binding
 * pyqrusty/src/lib.rs:476-491).  complex128; each row's products are summed
 * by 8 lanes (lane-strided partial sums, then a butterfly), so the result
 * matches a storage-order sum to rounding, not bit for bit.  v has ncols
 * entries; a column index >= ncols is skipped.  indptr must be a valid
 * non-decreasing row-pointer array over data / indices. */
int qr_csr_spmv(uint64_t nrows, uint64_t ncols, const uint64_t *indptr,
                const uint64_t *indices, const double *data, const double *v, double *y,
                void *stream);

/* Replace the coefficients of the operator's T terms (same order and
 * meaning as in qr_op_create); terms, masks and phases are unchanged.
 * Cached plans are rebuilt on next use (synchronous).  Replaces building a
 * new SparsePauliOp (qrusty/src/lib.rs:354-376) when only c changes, as in
 * gradient-based coefficient optimisation. */
int qr_op_set_coeffs(qr_op *op, const double *coeff);

/* qr_op_set_coeffs with the coefficients in DEVICE memory (T (re, im)
 * doubles, same order and meaning), asynchronous on `stream`, with no host
 * synchronisation: for training loops whose coefficients live on the GPU.
 * Replaces building a new SparsePauliOp (qrusty/src/lib.rs:354-376) like
 * qr_op_set_coeffs.  Kernels on `stream` recompute c' (make_params,
 * qrusty/src/accel.rs:141-157), the merged sums and every coefficient table
 * of the plans already built (qr_apply / qr_apply_axpby / qr_expect /
 * batches of this operator, and their diagonals), with the same FP64
 * operations in the same order as a host build, so results are bit for bit
 * those of an operator created with these coefficients.  Work on other
 * streams that reads the operator must be ordered after it by the caller;
 * `coeff` may be reused once the stream has passed this call.  A batch keeps
 * its graph (its tables are rewritten in place).  Host-side consumers of the
 * coefficients -- a plan built later, qr_csr_build, qr_op_diagonal -- fetch
 * them once (synchronous).  The first call uploads the operator's fold
 * structure (synchronous). */
int qr_op_set_coeffs_device(qr_op *op, const double *coeff, void *stream);

/* TEST HOOKS -- not for production use; no reference counterpart.  They let
 * the test suite reach code that ordinary inputs do not:
 *  - flags & QR_TEST_FORCE_WIDE: this operator's CSR fill and compensated
 *    complex64 apply kernels use the 64-bit row-word instantiations that
 *    operators with n > 32 need, at any n (results are identical);
 *  - wait_ns: bound of every mbarrier wait of this operator's apply kernels
 *    (0 = the default 2 s; otherwise at least 1 ms);
 *  - withhold_step >= 0: in this operator's apply kernels, CTA 0 never
 *    issues the partner-tile copy of that step of its ring, so the wait for
 *    it runs out after wait_ns.  The kernel then stops computing, waits for
 *    the copies it did issue, records the error word and returns; qr_check
 *    reports QR_EKERNEL.  -1 = off.
 * Hooks stay set until changed; (0, 0, -1) restores normal operation. */
enum { QR_TEST_FORCE_WIDE = 1 };
int qr_op_set_test_hooks(qr_op *op, uint32_t flags, uint64_t wait_ns, int64_t withhold_step);

/* out[s] = <a_s, b_s> = sum_r conj(a_s[r]) * b_s[r] for nstates states of
 * 2^n amplitudes, accumulated in FP64 (complex128 out: 2 doubles per state,
 * device pointer).  dtype QR_C128 or QR_C64C (inputs complex64).  New: no
 * reference counterpart (qrusty leaves inner products to numpy). */
int qr_vdot(int32_t n, int32_t dtype, const void *a, const void *b, int32_t nstates,
            double *out, void *stream);

/* Allocation-free variant of qr_vdot.  No counterpart in the reference.
 *
 * For callers that cannot allocate device memory while they run: hosts whose
 * device memory is reserved up front by another allocator (a framework's
 * caching allocator or a fixed per-process budget), and latency-critical
 * loops that must not take the synchronisation or pool growth that
 * cudaMalloc / cudaMallocAsync can bring.  Same inputs, output and FP64
 * result as qr_vdot; the per-block partial sums live in a fixed
 * 256 KiB (QR_VDOT_NOALLOC_MAX_PARTIALS double2 entries) __device__ array that
 * every GPU loading this library holds until process exit, and no call
 * allocates or frees anything.
 *  - The first call on a device looks up that array's device address
 *    (cudaGetSymbolAddress, with the device current) and caches it; make
 *    that first call before any stream capture.
 *  - nstates may be at most QR_VDOT_NOALLOC_MAX_PARTIALS (QR_EINVAL
 *    otherwise); the block count per state shrinks as nstates grows.
 *  - All calls share the one array: calls whose kernels overlap on the GPU
 *    (other streams, other host threads) race and must be serialised by the
 *    caller. */
#define QR_VDOT_NOALLOC_MAX_PARTIALS 16384
int qr_vdot_noalloc(int32_t n, int32_t dtype, const void *a, const void *b, int32_t nstates,
                    double *out, void *stream);

/* out[s] = <psi_s| H |psi_s> in FP64 (2 doubles per state, device pointer);
 * H psi is formed in an operator-owned device buffer.  New: no reference
 * counterpart (spmat_dot_densevec + numpy vdot in qrusty's sandbox). */
int qr_expect(qr_op *op, int32_t dtype, const void *psi, int32_t nstates, double *out,
              void *stream);

/* Gradient of the coefficients of y = H(c) psi: for every INPUT term k,
 * out[k] = sum_s <P_k psi_s, g_s> (complex128, 2 doubles per term, device
 * pointer), where P_k = (1, -i, -1, +i)[phase_k] X^x_k Z^z_k is the term
 * without its coefficient and g the upstream gradient.  For real
 * coefficients the gradient is Re(out[k]).  FP32 products for QR_C64C,
 * FP64 accumulation across threads and tiles, every sum in a fixed order
 * (repeated calls and graph replays give the same bits).  Scratch is taken
 * from the stream-ordered allocator on `stream`.  New: no reference
 * counterpart (used by the autograd backward). */
int qr_term_grad(qr_op *op, int32_t dtype, const void *psi, const void *g, int32_t nstates,
                 double *out, void *stream);

/* Batched H psi: many operators, each with its own states, behind ONE graph
 * launch per call.  Compensated complex64 only.  New: no reference
 * counterpart (qrusty applies one operator at a time).
 *
 * qr_batch_create: ops[i] (all on the current device, n <= 32) with
 * nstates[i] states each.  The operators must outlive the batch.  When an
 * operator's coefficients change (qr_op_set_coeffs), the next
 * qr_batch_apply synchronises `stream`, rebuilds the plan tables and makes
 * its graph again before launching.
 * qr_batch_apply: psi[i] / y[i] are device pointers to operator i's
 * nstates[i] complex64 states (back to back).  The first call times, on the
 * given buffers (y is overwritten), (a) one persistent kernel over a work list
 * of (operator, state, amplitude tile) items, (b) a graph of one apply
 * kernel per operator on four parallel branches and, when the batch has
 * both, (c) the persistent kernel over the small operators (fewer work items
 * than half the SMs) beside per-operator kernels for the large ones; it
 * keeps the fastest, captured in a CUDA graph, and every call launches that
 * graph on `stream`.  A call whose pointers differ from the
 * previous call's synchronises `stream` first (and, for (b), captures the
 * graph again). */
typedef struct qr_batch qr_batch;
int qr_batch_create(int32_t nops, qr_op *const *ops, const int32_t *nstates, qr_batch **out);
int qr_batch_destroy(qr_batch *b);
int qr_batch_apply(qr_batch *b, const void *const *psi, void *const *y, void *stream);
/* Mode the first apply chose: 0 persistent work-list kernel, 1 graph of
 * per-operator kernels, 2 both (form (c) above); -1 before the first apply.
 * qr_batch_set_mode fixes it instead (-1 restores the choice by timing);
 * only before the first apply. */
int qr_batch_mode(const qr_batch *b);
int qr_batch_set_mode(qr_batch *b, int32_t mode);
/* Tile width the autotuner chose (log2 amplitudes; 0 before the first apply). */
int qr_batch_tile_bits(const qr_batch *b);

/* Vector helpers of the eigensolver loop, element-wise over len complex
 * elements of device memory (dtype QR_C128: complex128, arithmetic
 * bit-identical to num-complex's; QR_C64C: complex64, the same sequence in
 * FP32 with the scalars rounded to float).  Scalars a, b, e are host
 * pointers to (re, im) doubles.  z / out may be the same buffer as an input.
 *
 * qr_axpby: z = a x + b y      -- qrusty/src/accel.rs:374-379 (axpby),
 *                                  pyqrusty/src/lib.rs:523-535
 * qr_axpy:  z = a x + y        -- qrusty/src/accel.rs:381-386 (axpy)
 * qr_ax:    z = a x            -- qrusty/src/accel.rs:388-393 (ax)
 * qr_precond2: out = dx / reg(diag - e, tol), where reg(v) = tol + 0i when
 *           |v| < tol (|v| = hypot) and v otherwise -- pyqrusty/src/lib.rs:
 *           457-469 (precond2), :580-592 (binding) and :436-440 (reg). */
int qr_axpby(int32_t dtype, uint64_t len, const double *a, const void *x, const double *b,
             const void *y, void *z, void *stream);
int qr_axpy(int32_t dtype, uint64_t len, const double *a, const void *x, const void *y, void *z,
            void *stream);
int qr_ax(int32_t dtype, uint64_t len, const double *a, const void *x, void *z, void *stream);
int qr_precond2(int32_t dtype, uint64_t len, const void *diag, const void *dx, const double *e,
                double tol, void *out, void *stream);

/* Diagonal of a device CSR matrix (complex128 data): out[r] = the stored
 * entry of row r at column r, 0 if none, for r < min(nrows, ncols) --
 * SpMat.diagonal(), pyqrusty/src/lib.rs:118-125 (sprs diag().to_dense());
 * with it, qr_precond2 is pyqrusty's precond (pyqrusty/src/lib.rs:442-455). */
int qr_csr_diagonal(uint64_t nrows, uint64_t ncols, const uint64_t *indptr,
                    const uint64_t *indices, const double *data, double *out, void *stream);

/* Diagonal of H without building the CSR: out[r] = the terms with x = 0
 * folded in input order as make_row folds them (qrusty/src/accel.rs:
 * 171-210), so for QR_C128 it equals the diagonal of qr_csr_build's matrix
 * bit for bit; QR_C64C rounds that FP64 value to complex64.  2^n elements. */
int qr_op_diagonal(qr_op *op, int32_t dtype, void *out, void *stream);

/* On-disk CSR formats.  Paths ending in ".gz" are gzip streams (zlib is
 * loaded at run time), as qrusty/src/util.rs:324-367 opens them.  Arrays are
 * host (mem = QR_MEM_HOST) or device (QR_MEM_DEVICE, staged through pinned
 * buffers on `stream`) memory; every call is synchronous.
 *
 * rawio -- qrusty/src/rawio.rs:128-179 (rawio::write / rawio::read): mark
 * "MI" in the writer's byte order, u64 storage (0 CSR, 1 CSC), rows, cols,
 * then (u64 length, words) for indptr, indices and data (complex128).  A file
 * from a machine of the other byte order is swapped on reading.
 * qr_rawio_info reads the sizes (nnz = data length), qr_rawio_read fills
 * caller-owned arrays of those sizes. */
typedef struct {
    uint64_t storage;     /* 0 = CSR, 1 = CSC                              */
    uint64_t nrows, ncols;
    uint64_t indptr_len;  /* entries of indptr                             */
    uint64_t nnz;         /* entries of indices and of data                */
    int32_t byte_swapped; /* file written with the other byte order       */
} qr_csr_file_info;
int qr_rawio_info(const char *path, qr_csr_file_info *info);
int qr_rawio_read(const char *path, uint64_t *indptr, uint64_t *indices, double *data, int32_t mem,
                  void *stream);
int qr_rawio_write(const char *path, uint64_t storage, uint64_t nrows, uint64_t ncols,
                   const uint64_t *indptr, uint64_t indptr_len, const uint64_t *indices,
                   const double *data, uint64_t nnz, int32_t mem, void *stream);

/* MatrixMarket -- SpMat.matrixmarket_write / matrixmarket_write_symmetric /
 * matrixmarket_read (pyqrusty/src/lib.rs:216-260, sprs::io).  Writing: a CSR
 * matrix as "coordinate complex <symmetry>" (symmetry 0 general,
 * 1 symmetric, 2 skew-symmetric, 3 hermitian; the symmetric kinds write the
 * lower triangle, skew the strict lower triangle), 1-based, rows in order,
 * values as the shortest decimal that reads back to the same double, no
 * exponent.  Reading: coordinate files of real / integer / complex / pattern
 * field and any of the four symmetries, mirrored entries added, converted
 * to CSR with columns ascending and duplicates summed in file order;
 * qr_mm_open parses into a handle, qr_mm_fetch copies it out,
 * qr_mm_close frees it. */
typedef struct qr_csr_file qr_csr_file;
int qr_mm_write(const char *path, uint64_t nrows, uint64_t ncols, const uint64_t *indptr,
                const uint64_t *indices, const double *data, int32_t symmetry, int32_t mem,
                void *stream);
int qr_mm_open(const char *path, qr_csr_file **out, uint64_t *nrows, uint64_t *ncols,
               uint64_t *nnz);
int qr_mm_fetch(const qr_csr_file *f, uint64_t *indptr, uint64_t *indices, double *data,
                int32_t mem, void *stream);
int qr_mm_close(qr_csr_file *f);

/* Message of the calling thread's last failure ("" if none).  Copies at
 * most len-1 bytes plus a terminating NUL; returns the full length. */
int qr_last_error(char *buf, size_t len);

/* Number of kernel launches this library has issued in the process (for
 * launch accounting by callers and benchmarks). */
uint64_t qr_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* QRUSTY_GPU_H */
