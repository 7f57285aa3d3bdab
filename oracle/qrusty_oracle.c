/*
 * qrusty_oracle.c -- CPU restatement of qrusty's rowwise Pauli-sum path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle and the timed
 * CPU baseline ("port" of the reference's rayon path).  Only tests/, the
 * smoke() check and bench.py's CPU-baseline / reference arm may load it.
 * The GPU product path never calls it and has no CPU fallback.
 *
 * Parity status: pinned.  The reference (Rust + pyo3) cannot be compiled
 * here, so this restatement is pinned against the reference's own
 * known-answer tests and fixtures (label-parse goldens, the 2x2 Pauli
 * matrices, I+2X, and "rowwise == kron exactly" on the H2/H4/H6 fixture
 * Hamiltonians) -- see tests/test_oracle_pins.py.
 *
 * Every function cites the reference source it restates (paths relative
 * to the qrusty repository).
 *
 * Arithmetic follows num-complex 0.4: (a*b) = (ar*br - ai*bi, ar*bi + ai*br),
 * a+b component-wise, -a component-wise.  Build with -ffp-contract=off so
 * that no fused multiply-add changes a rounding (aarch64 gcc contracts by
 * default; Rust never does).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include <stdatomic.h>

typedef struct { double re, im; } cplx;

static inline cplx c_mul(cplx a, cplx b) {
    cplx r;
    r.re = a.re * b.re - a.im * b.im;
    r.im = a.re * b.im + a.im * b.re;
    return r;
}
static inline cplx c_add(cplx a, cplx b) { cplx r = {a.re + b.re, a.im + b.im}; return r; }
static inline cplx c_neg(cplx a) { cplx r = {-a.re, -a.im}; return r; }

/* ------------------------------------------------------------------ */
/* Label parsing: qrusty/src/lib.rs:125-149 (Pauli::parse_label),       */
/* x/z masks lib.rs:161-176, phase lib.rs:179-181.                       */
/* Grammar ^([+-]?)1?([ij]?)([IXYZ]+)$ ; characters reversed so that     */
/* qubit 0 is the rightmost letter.                                      */
/* Returns 0 on success, -1 on a malformed label.                        */
/* letters_out receives qubit-ordered letters ('I','X','Y','Z').         */
/* ------------------------------------------------------------------ */
int or_parse_label(const char *s, int *base_phase, int *nqubits, char *letters_out, int cap)
{
    const char *p = s;
    int neg = 0, imag = 0;
    if (*p == '+' || *p == '-') { neg = (*p == '-'); ++p; }
    if (*p == '1') ++p;
    if (*p == 'i' || *p == 'j') { imag = 1; ++p; }
    const char *q = p;
    while (*q == 'I' || *q == 'X' || *q == 'Y' || *q == 'Z') ++q;
    if (*q != '\0' || q == p) return -1;
    int n = (int)(q - p);
    if (n > cap) return -1;
    for (int i = 0; i < n; ++i) letters_out[i] = p[n - 1 - i];
    *nqubits = n;
    *base_phase = imag + (neg ? 2 : 0);
    return 0;
}

/* Masks and phase of one parsed label (lib.rs:161-181, SimplePauli::x/z
 * lib.rs:80-91): x bit q <=> X or Y at qubit q; z bit q <=> Y or Z;
 * phase = (base + #Y) mod 4.  n <= 64. */
void or_label_masks(const char *letters, int n, int base_phase,
                    uint64_t *x, uint64_t *z, int *phase)
{
    uint64_t xm = 0, zm = 0;
    int ny = 0;
    for (int i = 0; i < n; ++i) {
        char c = letters[i];
        if (c == 'X' || c == 'Y') xm |= (uint64_t)1 << i;
        if (c == 'Y' || c == 'Z') zm |= (uint64_t)1 << i;
        if (c == 'Y') ++ny;
    }
    *x = xm; *z = zm; *phase = (base_phase + ny) % 4;
}

/* ------------------------------------------------------------------ */
/* make_params: qrusty/src/accel.rs:141-157.                              */
/* c'_k = m(phase % 4) * c_k with m = 1, -i, -1, +i.                     */
/* coeff / cprime are interleaved (re, im) arrays of length 2*T.         */
/* ------------------------------------------------------------------ */
void or_make_params(size_t T, const uint8_t *phase, const double *coeff, double *cprime)
{
    static const cplx m[4] = {{1.0, 0.0}, {0.0, -1.0}, {-1.0, 0.0}, {0.0, 1.0}};
    for (size_t k = 0; k < T; ++k) {
        cplx c = {coeff[2 * k], coeff[2 * k + 1]};
        cplx r = c_mul(m[phase[k] % 4], c);
        cprime[2 * k] = r.re;
        cprime[2 * k + 1] = r.im;
    }
}

/* ------------------------------------------------------------------ */
/* make_row: qrusty/src/accel.rs:171-210.                                 */
/* For row r: per term (col = r ^ x_k, val = odd(popcount(r & z_k)) ?    */
/* -c'_k : c'_k); STABLE sort by col (Rust sort_by is stable); left      */
/* fold merging equal columns, summing in term order starting from the  */
/* first value; explicit zeros kept.  Returns the number of entries.     */
/* work must hold 2*T entries of ent_t.                                  */
/* ------------------------------------------------------------------ */
typedef struct { uint64_t col; cplx val; } ent_t;

static void merge_sort_stable(ent_t *a, ent_t *tmp, size_t n)
{
    /* bottom-up stable merge sort by col */
    for (size_t w = 1; w < n; w <<= 1) {
        for (size_t lo = 0; lo < n; lo += 2 * w) {
            size_t mid = lo + w < n ? lo + w : n;
            size_t hi = lo + 2 * w < n ? lo + 2 * w : n;
            size_t i = lo, j = mid, k = lo;
            while (i < mid && j < hi) {
                if (a[j].col < a[i].col) tmp[k++] = a[j++];
                else tmp[k++] = a[i++];
            }
            while (i < mid) tmp[k++] = a[i++];
            while (j < hi) tmp[k++] = a[j++];
        }
        memcpy(a, tmp, n * sizeof(ent_t));
    }
}

static size_t make_row_impl(size_t T, const uint64_t *z, const uint64_t *x, const cplx *cp,
                            uint64_t row, uint64_t *cols, cplx *vals, ent_t *work)
{
    ent_t *v = work, *tmp = work + T;
    for (size_t k = 0; k < T; ++k) {
        v[k].col = row ^ x[k];
        v[k].val = (__builtin_popcountll(row & z[k]) % 2 == 1) ? c_neg(cp[k]) : cp[k];
    }
    merge_sort_stable(v, tmp, T);
    size_t cnt = 0;
    uint64_t prev = v[0].col;
    cplx sum = v[0].val;
    for (size_t k = 1; k < T; ++k) {
        if (v[k].col == prev) {
            sum = c_add(sum, v[k].val);
        } else {
            cols[cnt] = prev; vals[cnt] = sum; ++cnt;
            prev = v[k].col; sum = v[k].val;
        }
    }
    cols[cnt] = prev; vals[cnt] = sum; ++cnt;
    return cnt;
}

size_t or_make_row(size_t T, const uint64_t *z, const uint64_t *x, const double *cprime,
                   uint64_t row, uint64_t *cols, double *vals)
{
    ent_t *work = (ent_t *)malloc(2 * T * sizeof(ent_t));
    size_t c = make_row_impl(T, z, x, (const cplx *)cprime, row, cols, (cplx *)vals, work);
    free(work);
    return c;
}

/* ------------------------------------------------------------------ */
/* Chunked parallel CSR assembly: qrusty/src/accel.rs:267-336            */
/* (make_unsafe_vectors_chunked).  Rows are cut into chunks of `step`;   */
/* chunks run in parallel (rayon par_iter -> a pthread pool pulling      */
/* chunk indices from an atomic counter); each chunk concatenates its    */
/* rows; indptr is a serial prefix sum (accel.rs:309-319); indices/data  */
/* are the concatenation of the chunks (accel.rs:322-325).               */
/* ------------------------------------------------------------------ */
typedef struct {
    size_t nnz;
    uint64_t *row_nnz;  /* per row */
    uint64_t *cols;     /* per-chunk buffers, concatenated at fetch */
    cplx *vals;
    uint64_t **chunk_cols;
    cplx **chunk_vals;
    uint64_t *chunk_nnz;
    size_t nchunks, step, dim;
} csr_handle;

typedef struct {
    size_t T; const uint64_t *z, *x; const cplx *cp;
    size_t dim, step, nchunks;
    uint64_t row_lo;
    atomic_size_t next;
    csr_handle *h;
} build_ctx;

static void *build_worker(void *arg)
{
    build_ctx *c = (build_ctx *)arg;
    ent_t *work = (ent_t *)malloc(2 * c->T * sizeof(ent_t));
    uint64_t *rc = (uint64_t *)malloc(c->T * sizeof(uint64_t));
    cplx *rv = (cplx *)malloc(c->T * sizeof(cplx));
    for (;;) {
        size_t ch = atomic_fetch_add(&c->next, 1);
        if (ch >= c->nchunks) break;
        size_t lo = ch * c->step, hi = lo + c->step < c->dim ? lo + c->step : c->dim;
        size_t cap = (hi - lo) * c->T, used = 0;
        uint64_t *cc = (uint64_t *)malloc((cap ? cap : 1) * sizeof(uint64_t));
        cplx *cv = (cplx *)malloc((cap ? cap : 1) * sizeof(cplx));
        for (size_t r = lo; r < hi; ++r) {
            size_t k = make_row_impl(c->T, c->z, c->x, c->cp, c->row_lo + (uint64_t)r, rc, rv, work);
            memcpy(cc + used, rc, k * sizeof(uint64_t));
            memcpy(cv + used, rv, k * sizeof(cplx));
            c->h->row_nnz[r] = k;
            used += k;
        }
        c->h->chunk_cols[ch] = cc;
        c->h->chunk_vals[ch] = cv;
        c->h->chunk_nnz[ch] = used;
    }
    free(work); free(rc); free(rv);
    return NULL;
}

static void run_pool(int nthreads, void *(*fn)(void *), void *ctx)
{
    if (nthreads <= 1) { fn(ctx); return; }
    pthread_t *th = (pthread_t *)malloc(nthreads * sizeof(pthread_t));
    for (int i = 0; i < nthreads; ++i) pthread_create(&th[i], NULL, fn, ctx);
    for (int i = 0; i < nthreads; ++i) pthread_join(th[i], NULL);
    free(th);
}

/* Builds rows [row_lo, row_hi) of the CSR of sum_k c'_k P_k (the whole
 * 2^n x 2^n matrix when the range is [0, 2^n); a row range is the bounded
 * sample the CPU baseline times).  Returns an opaque handle; or_csr_nnz()
 * gives nnz; or_csr_fetch() performs the final indptr pass + concatenation
 * into caller buffers; or_csr_free() frees. */
void *or_csr_build(size_t T, int n, const uint64_t *z, const uint64_t *x, const double *cprime,
                   uint64_t row_lo, uint64_t row_hi, size_t step, int nthreads)
{
    csr_handle *h = (csr_handle *)calloc(1, sizeof(csr_handle));
    (void)n;
    size_t dim = (size_t)(row_hi - row_lo);
    if (step == 0) step = 1;
    h->dim = dim; h->step = step;
    h->nchunks = (dim + step - 1) / step;
    h->row_nnz = (uint64_t *)malloc(dim * sizeof(uint64_t));
    h->chunk_cols = (uint64_t **)calloc(h->nchunks, sizeof(uint64_t *));
    h->chunk_vals = (cplx **)calloc(h->nchunks, sizeof(cplx *));
    h->chunk_nnz = (uint64_t *)calloc(h->nchunks, sizeof(uint64_t));
    build_ctx c;
    c.T = T; c.z = z; c.x = x; c.cp = (const cplx *)cprime;
    c.dim = dim; c.step = step; c.nchunks = h->nchunks; c.h = h; c.row_lo = row_lo;
    atomic_init(&c.next, 0);
    run_pool(nthreads, build_worker, &c);
    size_t nnz = 0;
    for (size_t i = 0; i < h->nchunks; ++i) nnz += h->chunk_nnz[i];
    h->nnz = nnz;
    return h;
}

size_t or_csr_nnz(void *hv) { return ((csr_handle *)hv)->nnz; }

void or_csr_fetch(void *hv, uint64_t *indptr, uint64_t *indices, double *data)
{
    csr_handle *h = (csr_handle *)hv;
    uint64_t nnz = 0;
    for (size_t r = 0; r < h->dim; ++r) { indptr[r] = nnz; nnz += h->row_nnz[r]; }
    indptr[h->dim] = nnz;
    size_t off = 0;
    for (size_t ch = 0; ch < h->nchunks; ++ch) {
        memcpy(indices + off, h->chunk_cols[ch], h->chunk_nnz[ch] * sizeof(uint64_t));
        memcpy(data + 2 * off, h->chunk_vals[ch], h->chunk_nnz[ch] * sizeof(cplx));
        off += h->chunk_nnz[ch];
    }
}

void or_csr_free(void *hv)
{
    csr_handle *h = (csr_handle *)hv;
    for (size_t ch = 0; ch < h->nchunks; ++ch) { free(h->chunk_cols[ch]); free(h->chunk_vals[ch]); }
    free(h->chunk_cols); free(h->chunk_vals); free(h->chunk_nnz); free(h->row_nnz); free(h);
}

/* ------------------------------------------------------------------ */
/* CSR * dense vector: qrusty/src/accel.rs:338-370 (spmat_dot_densevec). */
/* Chunks of `step` (1024 in the reference) rows in parallel; per row    */
/* sum_j data_j * v[indices_j] in storage order (sprs dot_dense,         */
/* accel.rs:359), accumulated from zero.                                 */
/* ------------------------------------------------------------------ */
typedef struct {
    size_t nrows, step, nchunks;
    const uint64_t *indptr, *indices; const cplx *data; const cplx *v; cplx *y;
    atomic_size_t next;
} spmv_ctx;

static void *spmv_worker(void *arg)
{
    spmv_ctx *c = (spmv_ctx *)arg;
    for (;;) {
        size_t ch = atomic_fetch_add(&c->next, 1);
        if (ch >= c->nchunks) break;
        size_t lo = ch * c->step, hi = lo + c->step < c->nrows ? lo + c->step : c->nrows;
        for (size_t r = lo; r < hi; ++r) {
            cplx s = {0.0, 0.0};
            for (uint64_t j = c->indptr[r]; j < c->indptr[r + 1]; ++j)
                s = c_add(s, c_mul(c->data[j], c->v[c->indices[j]]));
            c->y[r] = s;
        }
    }
    return NULL;
}

void or_spmv(size_t nrows, const uint64_t *indptr, const uint64_t *indices, const double *data,
             const double *v, double *y, size_t step, int nthreads)
{
    spmv_ctx c;
    c.nrows = nrows; c.step = step ? step : 1024; c.nchunks = (nrows + c.step - 1) / c.step;
    c.indptr = indptr; c.indices = indices; c.data = (const cplx *)data;
    c.v = (const cplx *)v; c.y = (cplx *)y;
    atomic_init(&c.next, 0);
    run_pool(nthreads, spmv_worker, &c);
}

/* ------------------------------------------------------------------ */
/* Matrix-free restatement of CSR-build + SpMV, row for row: for each    */
/* row in [row_lo, row_hi) build the row exactly as make_row does        */
/* (accel.rs:171-210) and dot it with psi as spmat_dot_densevec does     */
/* (accel.rs:359).  Identical arithmetic to the CSR route, without       */
/* materialising the matrix; used where the CSR does not fit in RAM and  */
/* for row samples at large n.  Not qrusty's method as such.             */
/* y has (row_hi - row_lo) entries.                                      */
/* ------------------------------------------------------------------ */
typedef struct {
    size_t T; const uint64_t *z, *x; const cplx *cp;
    uint64_t row_lo, row_hi; size_t step, nchunks;
    const cplx *psi; cplx *y;
    atomic_size_t next;
} mf_ctx;

static void *mf_worker(void *arg)
{
    mf_ctx *c = (mf_ctx *)arg;
    ent_t *work = (ent_t *)malloc(2 * c->T * sizeof(ent_t));
    uint64_t *rc = (uint64_t *)malloc(c->T * sizeof(uint64_t));
    cplx *rv = (cplx *)malloc(c->T * sizeof(cplx));
    for (;;) {
        size_t ch = atomic_fetch_add(&c->next, 1);
        if (ch >= c->nchunks) break;
        uint64_t lo = c->row_lo + ch * c->step;
        uint64_t hi = lo + c->step < c->row_hi ? lo + c->step : c->row_hi;
        for (uint64_t r = lo; r < hi; ++r) {
            size_t k = make_row_impl(c->T, c->z, c->x, c->cp, r, rc, rv, work);
            cplx s = {0.0, 0.0};
            for (size_t j = 0; j < k; ++j) s = c_add(s, c_mul(rv[j], c->psi[rc[j]]));
            c->y[r - c->row_lo] = s;
        }
    }
    free(work); free(rc); free(rv);
    return NULL;
}

void or_apply_rows(size_t T, const uint64_t *z, const uint64_t *x, const double *cprime,
                   uint64_t row_lo, uint64_t row_hi, const double *psi, double *y, int nthreads)
{
    mf_ctx c;
    c.T = T; c.z = z; c.x = x; c.cp = (const cplx *)cprime;
    c.row_lo = row_lo; c.row_hi = row_hi; c.step = 64;
    c.nchunks = (row_hi - row_lo + c.step - 1) / c.step;
    c.psi = (const cplx *)psi; c.y = (cplx *)y;
    atomic_init(&c.next, 0);
    run_pool(nthreads, mf_worker, &c);
}

/* ------------------------------------------------------------------ */
/* Per-term coefficient gradient, FP64 definition check (no reference   */
/* counterpart: qrusty has no gradients).  out[k] = <P_k psi, g> =      */
/* sum_r conj(m(phase_k) (-1)^popc(r & z_k) psi[r ^ x_k]) g[r].         */
/* ------------------------------------------------------------------ */
typedef struct {
    size_t T, N; const uint64_t *x, *z; const uint8_t *phase;
    const cplx *psi, *g; cplx *out;
    atomic_size_t next;
} tg_ctx;

static void *tg_worker(void *arg)
{
    static const cplx m[4] = {{1.0, 0.0}, {0.0, -1.0}, {-1.0, 0.0}, {0.0, 1.0}};
    tg_ctx *c = (tg_ctx *)arg;
    for (;;) {
        size_t k = atomic_fetch_add(&c->next, 1);
        if (k >= c->T) break;
        cplx s = {0.0, 0.0};
        for (size_t r = 0; r < c->N; ++r) {
            cplx p = c->psi[r ^ c->x[k]];
            cplx v = {p.re * c->g[r].re + p.im * c->g[r].im, p.re * c->g[r].im - p.im * c->g[r].re};
            if (__builtin_popcountll(r & c->z[k]) & 1) v = c_neg(v);
            s = c_add(s, v);
        }
        cplx u = m[c->phase[k] % 4];
        cplx uc = {u.re, -u.im};
        c->out[k] = c_mul(uc, s);
    }
    return NULL;
}

void or_term_grad(size_t T, int n, const uint64_t *z, const uint64_t *x, const uint8_t *phase,
                  const double *psi, const double *g, double *out, int nthreads)
{
    tg_ctx c;
    c.T = T; c.N = (size_t)1 << n; c.x = x; c.z = z; c.phase = phase;
    c.psi = (const cplx *)psi; c.g = (const cplx *)g; c.out = (cplx *)out;
    atomic_init(&c.next, 0);
    run_pool(nthreads, tg_worker, &c);
}

/* ------------------------------------------------------------------ */
/* Vector helpers of the eigensolver loop, element-wise:               */
/*   op 0 axpby z = a x + b y   qrusty/src/accel.rs:374-379            */
/*   op 1 axpy  z = a x + y     qrusty/src/accel.rs:381-386            */
/*   op 2 ax    z = a x         qrusty/src/accel.rs:388-393            */
/*   op 3 precond2 z = y / reg(x - a, tol)  pyqrusty/src/lib.rs:457-469 */
/*        reg(v) = tol + 0i if |v| < tol else v  (:436-440), |v| = hypot */
/* num-complex 0.4 arithmetic: a*b as c_mul, a/b = ((ar br + ai bi)/n,  */
/* (ai br - ar bi)/n) with n = br^2 + bi^2.  f32 = 1: the same sequence */
/* in float with the scalars rounded to float (complex64 data).         */
/* ------------------------------------------------------------------ */
#include <math.h>

#define OR_VEC_BODY(R, HYPOT)                                                     \
    do {                                                                          \
        const R *X = (const R *)x, *Y = (const R *)y;                             \
        R *Z = (R *)z;                                                            \
        const R ar = (R)a[0], ai = (R)a[1];                                       \
        const R br = b ? (R)b[0] : (R)0, bi = b ? (R)b[1] : (R)0, tl = (R)tol;    \
        for (size_t i = 0; i < len; ++i) {                                        \
            const R xr = X[2 * i], xi = X[2 * i + 1];                             \
            const R yr = op != 2 ? Y[2 * i] : (R)0, yi = op != 2 ? Y[2 * i + 1] : (R)0; \
            R zr, zi;                                                             \
            if (op == 3) {                                                        \
                R dr = xr - ar, di = xi - ai;                                     \
                if (HYPOT(dr, di) < tl) { dr = tl; di = (R)0; }                   \
                const R ns = dr * dr + di * di;                                   \
                zr = (yr * dr + yi * di) / ns;                                    \
                zi = (yi * dr - yr * di) / ns;                                    \
            } else {                                                              \
                const R ur = ar * xr - ai * xi, ui = ar * xi + ai * xr;           \
                if (op == 2) { zr = ur; zi = ui; }                                \
                else if (op == 1) { zr = ur + yr; zi = ui + yi; }                 \
                else {                                                            \
                    const R vr = br * yr - bi * yi, vi = br * yi + bi * yr;       \
                    zr = ur + vr; zi = ui + vi;                                   \
                }                                                                 \
            }                                                                     \
            Z[2 * i] = zr; Z[2 * i + 1] = zi;                                     \
        }                                                                         \
    } while (0)

void or_vec(int op, int f32, size_t len, const void *x, const void *y, void *z,
            const double *a, const double *b, double tol)
{
    if (f32) OR_VEC_BODY(float, hypotf);
    else OR_VEC_BODY(double, hypot);
}

/* Diagonal of the operator's matrix, rows [row0, row0 + nrows): the value */
/* make_row (qrusty/src/accel.rs:171-210) places at column r of row r --    */
/* the terms with x = 0 in input order, left-folded from the first; 0 when  */
/* no term has x = 0 (the row then stores no diagonal entry).               */
void or_op_diagonal(size_t T, const uint64_t *z, const uint64_t *x, const double *cprime,
                    uint64_t row0, uint64_t nrows, double *out)
{
    const cplx *cp = (const cplx *)cprime;
    for (uint64_t i = 0; i < nrows; ++i) {
        const uint64_t r = row0 + i;
        cplx v = {0.0, 0.0};
        int first = 1;
        for (size_t k = 0; k < T; ++k) {
            if (x[k] != 0) continue;
            cplx t = cp[k];
            if (__builtin_popcountll(r & z[k]) & 1) t = c_neg(t);
            if (first) { v = t; first = 0; }
            else v = c_add(v, t);
        }
        out[2 * i] = v.re;
        out[2 * i + 1] = v.im;
    }
}
