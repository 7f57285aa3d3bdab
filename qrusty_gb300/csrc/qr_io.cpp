// qr_io.cpp -- qrusty's on-disk CSR formats, read into and written from host
// or device arrays.
//
//   rawio        qrusty/src/rawio.rs:128-179 (write / read): 2-byte mark "MI"
//                in the writer's byte order, u64 storage (0 CSR, 1 CSC),
//                u64 rows, u64 cols, then three (u64 length, raw array)
//                records: indptr (u64), indices (u64), data (complex128).  A
//                reader whose byte order differs sees the mark reversed and
//                swaps every word.
//   MatrixMarket pyqrusty/src/lib.rs:216-260 (matrixmarket_write / _read /
//                _write_symmetric over sprs::io): coordinate format, complex
//                field on output, 1-based indices, entries in CSR order,
//                values in the shortest decimal that reads back to the same
//                double, without exponent (Rust's f64 Display); input of
//                real / integer / complex / pattern fields and general /
//                symmetric / skew-symmetric / hermitian storage, duplicates
//                summed in file order when converted to CSR.
//   ".gz" paths are gzip streams, as qrusty/src/util.rs:324-367
//   (with_input_file / with_output_file); zlib is loaded at run time.
//
// Device arrays (mem = QR_MEM_DEVICE) move through two pinned 32 MiB staging
// buffers, so a CSR built on the GPU goes to disk without a full host copy.
#include <cuda_runtime.h>
#include <dlfcn.h>

#include <algorithm>
#include <charconv>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/qrusty_gpu.h"

namespace qr {
int set_error(int code, const char *msg);
}

namespace {

using qr::set_error;

int fail_msg(int code, const std::string &m) { return set_error(code, m.c_str()); }

// ---------------------------------------------------------------- zlib (run time)
struct Zlib {
    void *(*gzopen)(const char *, const char *) = nullptr;
    int (*gzread)(void *, void *, unsigned) = nullptr;
    int (*gzwrite)(void *, const void *, unsigned) = nullptr;
    int (*gzclose)(void *) = nullptr;
    bool ok = false;
};

const Zlib &zlib() {
    static Zlib z;
    static std::once_flag once;
    std::call_once(once, [] {
        void *h = dlopen("libz.so.1", RTLD_NOW | RTLD_LOCAL);
        if (!h) h = dlopen("libz.so", RTLD_NOW | RTLD_LOCAL);
        if (!h) return;
        z.gzopen = reinterpret_cast<void *(*)(const char *, const char *)>(dlsym(h, "gzopen"));
        z.gzread = reinterpret_cast<int (*)(void *, void *, unsigned)>(dlsym(h, "gzread"));
        z.gzwrite = reinterpret_cast<int (*)(void *, const void *, unsigned)>(dlsym(h, "gzwrite"));
        z.gzclose = reinterpret_cast<int (*)(void *)>(dlsym(h, "gzclose"));
        z.ok = z.gzopen && z.gzread && z.gzwrite && z.gzclose;
    });
    return z;
}

bool is_gz(const char *path) {
    const size_t n = strlen(path);
    return n >= 3 && strcmp(path + n - 3, ".gz") == 0;
}

// Byte stream over a plain file or a gzip file.
class Stream {
  public:
    ~Stream() { close(); }
    int open(const char *path, bool write) {
        gz_ = is_gz(path);
        if (gz_) {
            if (!zlib().ok) return fail_msg(QR_EINVAL, std::string(path) + ": gzip needs libz.so.1");
            g_ = zlib().gzopen(path, write ? "wb6" : "rb");
            if (!g_) return fail_msg(QR_EINVAL, std::string(path) + ": cannot open");
        } else {
            f_ = fopen(path, write ? "wb" : "rb");
            if (!f_)
                return fail_msg(QR_EINVAL, std::string(path) + ": " + strerror(errno));
        }
        path_ = path;
        return QR_OK;
    }
    int close() {
        int rc = QR_OK;
        if (f_ && fclose(f_) != 0) rc = fail_msg(QR_EINVAL, path_ + ": close failed");
        if (g_ && zlib().gzclose(g_) != 0) rc = fail_msg(QR_EINVAL, path_ + ": close failed");
        f_ = nullptr;
        g_ = nullptr;
        return rc;
    }
    int write(const void *p, size_t n) {
        const char *c = static_cast<const char *>(p);
        while (n) {
            const unsigned k = (unsigned)std::min<size_t>(n, 1u << 30);
            const size_t w = gz_ ? (size_t)std::max(0, zlib().gzwrite(g_, c, k)) : fwrite(c, 1, k, f_);
            if (w != k) return fail_msg(QR_EINVAL, path_ + ": write failed");
            c += k;
            n -= k;
        }
        return QR_OK;
    }
    // Reads up to n bytes; returns the count (0 at end of file), -1 on error.
    long long read_some(void *p, size_t n) {
        if (gz_) return zlib().gzread(g_, p, (unsigned)std::min<size_t>(n, 1u << 30));
        const size_t r = fread(p, 1, n, f_);
        if (r == 0 && ferror(f_)) return -1;
        return (long long)r;
    }
    int read_exact(void *p, size_t n) {
        char *c = static_cast<char *>(p);
        while (n) {
            const long long r = read_some(c, n);
            if (r <= 0) return fail_msg(QR_EINVAL, path_ + ": unexpected end of file");
            c += r;
            n -= (size_t)r;
        }
        return QR_OK;
    }
    const std::string &path() const { return path_; }

  private:
    FILE *f_ = nullptr;
    void *g_ = nullptr;
    bool gz_ = false;
    std::string path_;
};

// ---------------------------------------------------------------- staging
constexpr size_t kStage = 32u << 20;

struct Pinned {
    void *p[2] = {nullptr, nullptr};
    ~Pinned() {
        for (void *q : p)
            if (q) cudaFreeHost(q);
    }
    int alloc() {
        for (auto &q : p)
            if (cudaHostAlloc(&q, kStage, cudaHostAllocDefault) != cudaSuccess)
                return fail_msg(QR_ENOMEM, "pinned staging allocation failed");
        return QR_OK;
    }
};

// Write n bytes from host or device memory.
int write_array(Stream &s, const void *src, size_t n, int32_t mem, cudaStream_t st) {
    if (mem == QR_MEM_HOST || n == 0) return s.write(src, n);
    Pinned pin;
    int rc = pin.alloc();
    if (rc) return rc;
    cudaEvent_t ev[2];
    cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming);
    const char *d = static_cast<const char *>(src);
    size_t off = 0;
    int cur = 0;
    size_t len[2] = {0, 0};
    // prefetch chunk 0; then copy chunk i+1 while chunk i is written
    len[0] = std::min(kStage, n);
    if (cudaMemcpyAsync(pin.p[0], d, len[0], cudaMemcpyDeviceToHost, st) != cudaSuccess)
        rc = fail_msg(QR_ECUDA, "device-to-host copy failed");
    cudaEventRecord(ev[0], st);
    while (!rc && off < n) {
        const size_t next = off + len[cur];
        if (next < n) {
            len[cur ^ 1] = std::min(kStage, n - next);
            if (cudaMemcpyAsync(pin.p[cur ^ 1], d + next, len[cur ^ 1], cudaMemcpyDeviceToHost,
                                st) != cudaSuccess) {
                rc = fail_msg(QR_ECUDA, "device-to-host copy failed");
                break;
            }
            cudaEventRecord(ev[cur ^ 1], st);
        }
        if (cudaEventSynchronize(ev[cur]) != cudaSuccess) {
            rc = fail_msg(QR_ECUDA, "device-to-host copy failed");
            break;
        }
        rc = s.write(pin.p[cur], len[cur]);
        off = next;
        cur ^= 1;
    }
    cudaStreamSynchronize(st);
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    return rc;
}

void swap8(void *p, size_t count) {
    unsigned char *b = static_cast<unsigned char *>(p);
    for (size_t i = 0; i < count; ++i, b += 8)
        for (int k = 0; k < 4; ++k) std::swap(b[k], b[7 - k]);
}

// Read n bytes (8-byte words, swapped if asked) into host or device memory.
int read_array(Stream &s, void *dst, size_t n, bool swap, int32_t mem, cudaStream_t st) {
    if (mem == QR_MEM_HOST || n == 0) {
        int rc = s.read_exact(dst, n);
        if (!rc && swap) swap8(dst, n / 8);
        return rc;
    }
    Pinned pin;
    int rc = pin.alloc();
    if (rc) return rc;
    cudaEvent_t ev[2];
    cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming);
    bool used[2] = {false, false};
    char *d = static_cast<char *>(dst);
    int cur = 0;
    for (size_t off = 0; off < n && !rc; off += kStage, cur ^= 1) {
        const size_t len = std::min(kStage, n - off);
        if (used[cur] && cudaEventSynchronize(ev[cur]) != cudaSuccess) {
            rc = fail_msg(QR_ECUDA, "host-to-device copy failed");
            break;
        }
        rc = s.read_exact(pin.p[cur], len);
        if (rc) break;
        if (swap) swap8(pin.p[cur], len / 8);
        if (cudaMemcpyAsync(d + off, pin.p[cur], len, cudaMemcpyHostToDevice, st) != cudaSuccess) {
            rc = fail_msg(QR_ECUDA, "host-to-device copy failed");
            break;
        }
        cudaEventRecord(ev[cur], st);
        used[cur] = true;
    }
    cudaStreamSynchronize(st);
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    return rc;
}

// ---------------------------------------------------------------- rawio
uint16_t mark() {
    const unsigned char b[2] = {'M', 'I'};
    uint16_t m;
    memcpy(&m, b, 2);
    return m;
}

int read_u64(Stream &s, bool swap, uint64_t *v) {
    int rc = s.read_exact(v, 8);
    if (!rc && swap) swap8(v, 1);
    return rc;
}

struct RawHeader {
    bool swap = false;
    uint64_t storage = 0, rows = 0, cols = 0;
};

int raw_header(Stream &s, RawHeader *h) {
    uint16_t m = 0;
    int rc = s.read_exact(&m, 2);
    if (rc) return rc;
    h->swap = m != mark();
    if ((rc = read_u64(s, h->swap, &h->storage))) return rc;
    if (h->storage > 1) return fail_msg(QR_EINVAL, "rawio::read: bad storage found");
    if ((rc = read_u64(s, h->swap, &h->rows))) return rc;
    return read_u64(s, h->swap, &h->cols);
}

int skip(Stream &s, uint64_t bytes) {
    std::vector<char> buf(1 << 20);
    while (bytes) {
        const size_t k = (size_t)std::min<uint64_t>(bytes, buf.size());
        int rc = s.read_exact(buf.data(), k);
        if (rc) return rc;
        bytes -= k;
    }
    return QR_OK;
}

// ---------------------------------------------------------------- MatrixMarket
// f64 as Rust's Display prints it: shortest round-trip digits, fixed notation
// (at most ~330 characters).
char *put_f64(char *p, char *end, double v) {
    if (v != v) {
        memcpy(p, "NaN", 3);
        return p + 3;
    }
    if (v == __builtin_inf() || v == -__builtin_inf()) {
        const char *s = v > 0 ? "inf" : "-inf";
        const size_t n = strlen(s);
        memcpy(p, s, n);
        return p + n;
    }
    return std::to_chars(p, end, v, std::chars_format::fixed).ptr;
}

char *put_u64(char *p, char *end, uint64_t v) { return std::to_chars(p, end, v).ptr; }

enum Sym { kGeneral = 0, kSymmetric = 1, kSkew = 2, kHermitian = 3 };

const char *sym_name(int s) {
    switch (s) {
        case kSymmetric: return "symmetric";
        case kSkew: return "skew-symmetric";
        case kHermitian: return "hermitian";
        default: return "general";
    }
}

// Entries of rows [r0, r1) kept by the symmetry mode (lower triangle for
// the symmetric kinds, strictly lower for skew), formatted as text.
void format_rows(const uint64_t *indptr, const uint64_t *indices, const double *data, uint64_t r0,
                 uint64_t r1, int sym, std::string *out, uint64_t *count) {
    std::string &s = *out;
    uint64_t c = 0;
    // fixed notation of a double takes up to ~330 characters (1e-308, 1e308)
    char buf[1024];
    for (uint64_t r = r0; r < r1; ++r) {
        for (uint64_t j = indptr[r]; j < indptr[r + 1]; ++j) {
            const uint64_t col = indices[j];
            if (sym != kGeneral && (col > r || (sym == kSkew && col == r))) continue;
            char *p = buf, *e = buf + sizeof(buf);
            p = put_u64(p, e, r + 1);
            *p++ = ' ';
            p = put_u64(p, e, col + 1);
            *p++ = ' ';
            p = put_f64(p, e, data[2 * j]);
            *p++ = ' ';
            p = put_f64(p, e, data[2 * j + 1]);
            *p++ = '\n';
            s.append(buf, (size_t)(p - buf));
            ++c;
        }
    }
    *count = c;
}

int mm_write(const char *path, uint64_t nrows, uint64_t ncols, const uint64_t *indptr,
             const uint64_t *indices, const double *data, int32_t mem, void *stream, int sym) {
    if (!path || !indptr || (nrows && (!indices || !data)))
        return set_error(QR_EINVAL, "matrixmarket_write: null argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // host view of the arrays
    std::vector<uint64_t> h_ptr, h_idx;
    std::vector<double> h_dat;
    if (mem == QR_MEM_DEVICE) {
        h_ptr.resize(nrows + 1);
        if (cudaMemcpyAsync(h_ptr.data(), indptr, (nrows + 1) * 8, cudaMemcpyDeviceToHost, st) !=
                cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return set_error(QR_ECUDA, "matrixmarket_write: copy failed");
        const uint64_t nnz = h_ptr[nrows];
        h_idx.resize(nnz);
        h_dat.resize(2 * nnz);
        if (cudaMemcpyAsync(h_idx.data(), indices, nnz * 8, cudaMemcpyDeviceToHost, st) !=
                cudaSuccess ||
            cudaMemcpyAsync(h_dat.data(), data, nnz * 16, cudaMemcpyDeviceToHost, st) !=
                cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return set_error(QR_ECUDA, "matrixmarket_write: copy failed");
        indptr = h_ptr.data();
        indices = h_idx.data();
        data = h_dat.data();
    } else if (mem != QR_MEM_HOST) {
        return set_error(QR_EINVAL, "matrixmarket_write: mem must be QR_MEM_DEVICE or QR_MEM_HOST");
    }
    for (uint64_t r = 0; r < nrows; ++r)
        if (indptr[r + 1] < indptr[r])
            return set_error(QR_EINVAL, "matrixmarket_write: indptr is not non-decreasing");
    // format row chunks in parallel, write them in order
    unsigned nth = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    const uint64_t nnz = nrows ? indptr[nrows] : 0;
    if (nnz < (1u << 16)) nth = 1;
    std::vector<uint64_t> cut(nth + 1, nrows);
    cut[0] = 0;
    for (unsigned i = 1; i < nth; ++i) {
        const uint64_t want = nnz / nth * i;
        cut[i] = (uint64_t)(std::lower_bound(indptr, indptr + nrows + 1, want) - indptr);
        if (cut[i] > nrows) cut[i] = nrows;
        if (cut[i] < cut[i - 1]) cut[i] = cut[i - 1];
    }
    std::vector<std::string> text(nth);
    std::vector<uint64_t> count(nth, 0);
    std::vector<std::thread> pool;
    for (unsigned i = 0; i < nth; ++i)
        pool.emplace_back(format_rows, indptr, indices, data, cut[i], cut[i + 1], sym, &text[i],
                          &count[i]);
    for (auto &th : pool) th.join();
    uint64_t total = 0;
    for (uint64_t c : count) total += c;
    Stream s;
    int rc = s.open(path, true);
    if (rc) return rc;
    std::string head = std::string("%%MatrixMarket matrix coordinate complex ") + sym_name(sym) + "\n";
    char buf[96];
    char *p = buf, *e = buf + sizeof(buf);
    p = put_u64(p, e, nrows);
    *p++ = ' ';
    p = put_u64(p, e, ncols);
    *p++ = ' ';
    p = put_u64(p, e, total);
    *p++ = '\n';
    head.append(buf, (size_t)(p - buf));
    rc = s.write(head.data(), head.size());
    for (unsigned i = 0; i < nth && !rc; ++i) rc = s.write(text[i].data(), text[i].size());
    const int rc2 = s.close();
    return rc ? rc : rc2;
}

// Line reader over a Stream.
class Lines {
  public:
    explicit Lines(Stream &s) : s_(s), buf_(1 << 20) {}
    // Next line without its newline; false at end of file or on a read error.
    bool next(std::string &line) {
        line.clear();
        for (;;) {
            if (pos_ == len_) {
                const long long r = s_.read_some(buf_.data(), buf_.size());
                if (r <= 0) {
                    err_ = r < 0;
                    return !line.empty();
                }
                len_ = (size_t)r;
                pos_ = 0;
            }
            const char *b = buf_.data() + pos_;
            const void *nl = memchr(b, '\n', len_ - pos_);
            if (nl) {
                const size_t k = (size_t)(static_cast<const char *>(nl) - b);
                line.append(b, k);
                pos_ += k + 1;
                if (!line.empty() && line.back() == '\r') line.pop_back();
                return true;
            }
            line.append(b, len_ - pos_);
            pos_ = len_;
        }
    }
    bool error() const { return err_; }

  private:
    Stream &s_;
    std::vector<char> buf_;
    size_t pos_ = 0, len_ = 0;
    bool err_ = false;
};

std::string lower(std::string v) {
    for (auto &ch : v) ch = (char)tolower((unsigned char)ch);
    return v;
}

}  // namespace

// In-memory CSR read from a file, held between qr_mm_open and qr_mm_close.
struct qr_csr_file {
    uint64_t nrows = 0, ncols = 0;
    std::vector<uint64_t> indptr, indices;
    std::vector<double> data;
};

namespace {

int mm_parse(const char *path, qr_csr_file *f) {
    Stream s;
    int rc = s.open(path, false);
    if (rc) return rc;
    Lines in(s);
    std::string line;
    auto bad = [&](const std::string &why) {
        return fail_msg(QR_EINVAL, std::string("matrixmarket_read: ") + path + ": " + why);
    };
    if (!in.next(line)) return bad("empty file");
    // %%MatrixMarket matrix coordinate <field> <symmetry>
    char w[5][64] = {{0}};
    if (sscanf(line.c_str(), "%63s %63s %63s %63s %63s", w[0], w[1], w[2], w[3], w[4]) != 5 ||
        lower(w[0]) != "%%matrixmarket" || lower(w[1]) != "matrix")
        return bad("missing %%MatrixMarket matrix header");
    if (lower(w[2]) != "coordinate") return bad("only the coordinate format is supported");
    const std::string field = lower(w[3]), symm = lower(w[4]);
    int nval;
    if (field == "complex") nval = 2;
    else if (field == "real" || field == "integer" || field == "double") nval = 1;
    else if (field == "pattern") nval = 0;
    else return bad("unsupported field " + field);
    int sym;
    if (symm == "general") sym = kGeneral;
    else if (symm == "symmetric") sym = kSymmetric;
    else if (symm == "skew-symmetric") sym = kSkew;
    else if (symm == "hermitian") sym = kHermitian;
    else return bad("unsupported symmetry " + symm);
    // size line after comments
    unsigned long long rows = 0, cols = 0, nent = 0;
    for (;;) {
        if (!in.next(line)) return bad("missing size line");
        size_t k = line.find_first_not_of(" \t");
        if (k == std::string::npos || line[k] == '%') continue;
        if (sscanf(line.c_str(), "%llu %llu %llu", &rows, &cols, &nent) != 3)
            return bad("malformed size line");
        break;
    }
    struct Trip {
        uint64_t r, c;
        double re, im;
    };
    std::vector<Trip> t;
    t.reserve(sym == kGeneral ? nent : 2 * nent);
    uint64_t seen = 0;
    while (seen < nent && in.next(line)) {
        const char *p = line.c_str();
        while (*p == ' ' || *p == '\t') ++p;
        if (*p == 0 || *p == '%') continue;
        char *q;
        const unsigned long long i = strtoull(p, &q, 10);
        if (q == p) return bad("malformed entry");
        p = q;
        const unsigned long long j = strtoull(p, &q, 10);
        if (q == p) return bad("malformed entry");
        p = q;
        double re = 1.0, im = 0.0;
        if (nval >= 1) {
            re = strtod(p, &q);
            if (q == p) return bad("malformed entry");
            p = q;
        }
        if (nval == 2) {
            im = strtod(p, &q);
            if (q == p) return bad("malformed entry");
        }
        if (i < 1 || j < 1 || i > rows || j > cols) return bad("entry index out of range");
        t.push_back({i - 1, j - 1, re, im});
        if (sym != kGeneral && i != j) {
            if (sym == kSymmetric) t.push_back({j - 1, i - 1, re, im});
            else if (sym == kSkew) t.push_back({j - 1, i - 1, -re, -im});
            else t.push_back({j - 1, i - 1, re, -im});
        }
        ++seen;
    }
    if (in.error()) return bad("read error");
    if (seen < nent) return bad("fewer entries than the size line states");
    // CSR: rows ascending, columns ascending, duplicates summed in file order
    std::stable_sort(t.begin(), t.end(), [](const Trip &a, const Trip &b) {
        return a.r != b.r ? a.r < b.r : a.c < b.c;
    });
    f->nrows = rows;
    f->ncols = cols;
    f->indptr.assign(rows + 1, 0);
    f->indices.clear();
    f->data.clear();
    for (size_t k = 0; k < t.size(); ++k) {
        if (k > 0 && t[k].r == t[k - 1].r && t[k].c == t[k - 1].c) {
            f->data[f->data.size() - 2] += t[k].re;
            f->data[f->data.size() - 1] += t[k].im;
            continue;
        }
        f->indices.push_back(t[k].c);
        f->data.push_back(t[k].re);
        f->data.push_back(t[k].im);
        f->indptr[t[k].r + 1]++;
    }
    for (uint64_t r = 0; r < rows; ++r) f->indptr[r + 1] += f->indptr[r];
    return QR_OK;
}

int copy_out(void *dst, const void *src, size_t n, int32_t mem, cudaStream_t st) {
    if (n == 0) return QR_OK;
    if (mem == QR_MEM_HOST) {
        memcpy(dst, src, n);
        return QR_OK;
    }
    if (cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return set_error(QR_ECUDA, "host-to-device copy failed");
    return QR_OK;
}

}  // namespace

extern "C" {

int qr_rawio_info(const char *path, qr_csr_file_info *info) {
    if (!path || !info) return set_error(QR_EINVAL, "qr_rawio_info: null argument");
    Stream s;
    int rc = s.open(path, false);
    if (rc) return rc;
    RawHeader h;
    if ((rc = raw_header(s, &h))) return rc;
    uint64_t lp = 0, li = 0, ld = 0;
    if ((rc = read_u64(s, h.swap, &lp)) || (rc = skip(s, lp * 8)) ||
        (rc = read_u64(s, h.swap, &li)) || (rc = skip(s, li * 8)) ||
        (rc = read_u64(s, h.swap, &ld)))
        return rc;
    info->storage = h.storage;
    info->nrows = h.rows;
    info->ncols = h.cols;
    info->indptr_len = lp;
    info->nnz = ld;
    info->byte_swapped = h.swap ? 1 : 0;
    if (li != ld) return set_error(QR_EINVAL, "rawio: indices and data lengths differ");
    return QR_OK;
}

int qr_rawio_read(const char *path, uint64_t *indptr, uint64_t *indices, double *data, int32_t mem,
                  void *stream) {
    if (!path) return set_error(QR_EINVAL, "qr_rawio_read: null argument");
    if (mem != QR_MEM_DEVICE && mem != QR_MEM_HOST)
        return set_error(QR_EINVAL, "qr_rawio_read: mem must be QR_MEM_DEVICE or QR_MEM_HOST");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Stream s;
    int rc = s.open(path, false);
    if (rc) return rc;
    RawHeader h;
    if ((rc = raw_header(s, &h))) return rc;
    uint64_t lp = 0, li = 0, ld = 0;
    if ((rc = read_u64(s, h.swap, &lp))) return rc;
    if (lp && !indptr) return set_error(QR_EINVAL, "qr_rawio_read: null argument");
    if ((rc = read_array(s, indptr, lp * 8, h.swap, mem, st))) return rc;
    if ((rc = read_u64(s, h.swap, &li))) return rc;
    if (li && !indices) return set_error(QR_EINVAL, "qr_rawio_read: null argument");
    if ((rc = read_array(s, indices, li * 8, h.swap, mem, st))) return rc;
    if ((rc = read_u64(s, h.swap, &ld))) return rc;
    if (ld != li) return set_error(QR_EINVAL, "rawio: indices and data lengths differ");
    if (ld && !data) return set_error(QR_EINVAL, "qr_rawio_read: null argument");
    return read_array(s, data, ld * 16, h.swap, mem, st);
}

int qr_rawio_write(const char *path, uint64_t storage, uint64_t nrows, uint64_t ncols,
                   const uint64_t *indptr, uint64_t indptr_len, const uint64_t *indices,
                   const double *data, uint64_t nnz, int32_t mem, void *stream) {
    if (!path || (indptr_len && !indptr) || (nnz && (!indices || !data)))
        return set_error(QR_EINVAL, "qr_rawio_write: null argument");
    if (storage > 1) return set_error(QR_EINVAL, "qr_rawio_write: storage must be 0 (CSR) or 1 (CSC)");
    if (mem != QR_MEM_DEVICE && mem != QR_MEM_HOST)
        return set_error(QR_EINVAL, "qr_rawio_write: mem must be QR_MEM_DEVICE or QR_MEM_HOST");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Stream s;
    int rc = s.open(path, true);
    if (rc) return rc;
    const uint16_t m = mark();
    const uint64_t hdr[3] = {storage, nrows, ncols};
    if ((rc = s.write(&m, 2)) || (rc = s.write(hdr, sizeof(hdr))) ||
        (rc = s.write(&indptr_len, 8)) ||
        (rc = write_array(s, indptr, indptr_len * 8, mem, st)) || (rc = s.write(&nnz, 8)) ||
        (rc = write_array(s, indices, nnz * 8, mem, st)) || (rc = s.write(&nnz, 8)) ||
        (rc = write_array(s, data, nnz * 16, mem, st))) {
        s.close();
        return rc;
    }
    return s.close();
}

int qr_mm_write(const char *path, uint64_t nrows, uint64_t ncols, const uint64_t *indptr,
                const uint64_t *indices, const double *data, int32_t symmetry, int32_t mem,
                void *stream) {
    if (symmetry < 0 || symmetry > 3)
        return set_error(QR_EINVAL,
                         "matrixmarket_write_symmetric: unrecognized mode (0 general, 1 symmetric, "
                         "2 skew-symmetric, 3 hermitian)");
    return mm_write(path, nrows, ncols, indptr, indices, data, mem, stream, symmetry);
}

int qr_mm_open(const char *path, qr_csr_file **out, uint64_t *nrows, uint64_t *ncols,
               uint64_t *nnz) {
    if (!path || !out) return set_error(QR_EINVAL, "qr_mm_open: null argument");
    *out = nullptr;
    qr_csr_file *f = new (std::nothrow) qr_csr_file;
    if (!f) return set_error(QR_ENOMEM, "qr_mm_open: out of memory");
    int rc;
    try {
        rc = mm_parse(path, f);
    } catch (const std::bad_alloc &) {
        rc = set_error(QR_ENOMEM, "qr_mm_open: out of memory");
    }
    if (rc) {
        delete f;
        return rc;
    }
    if (nrows) *nrows = f->nrows;
    if (ncols) *ncols = f->ncols;
    if (nnz) *nnz = f->indices.size();
    *out = f;
    return QR_OK;
}

int qr_mm_fetch(const qr_csr_file *f, uint64_t *indptr, uint64_t *indices, double *data,
                int32_t mem, void *stream) {
    if (!f || !indptr || (!f->indices.empty() && (!indices || !data)))
        return set_error(QR_EINVAL, "qr_mm_fetch: null argument");
    if (mem != QR_MEM_DEVICE && mem != QR_MEM_HOST)
        return set_error(QR_EINVAL, "qr_mm_fetch: mem must be QR_MEM_DEVICE or QR_MEM_HOST");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int rc = copy_out(indptr, f->indptr.data(), f->indptr.size() * 8, mem, st);
    if (!rc) rc = copy_out(indices, f->indices.data(), f->indices.size() * 8, mem, st);
    if (!rc) rc = copy_out(data, f->data.data(), f->data.size() * 8, mem, st);
    return rc;
}

int qr_mm_close(qr_csr_file *f) {
    delete f;
    return QR_OK;
}

}  // extern "C"
