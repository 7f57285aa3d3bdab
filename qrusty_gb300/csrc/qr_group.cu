// qr_group.cu -- term preparation and grouping on the device.
//
//   * Stable LSD radix sort of (u64 key, u32 index) pairs, 8-bit digits, and
//     device-wide exclusive scans: the primitives of everything below.
//   * group_terms: the terms sorted stably by x and cut into groups of equal x
//     in ascending order (the sort of make_row, qrusty/src/accel.rs:188-208);
//     the FP64 simplification -- terms with equal (x, z) merged into one
//     string, strings numbered in first-occurrence order, each string's input
//     terms listed in input order for the fold of merge_coeffs_kernel; and the
//     merged strings cut into groups of equal x, numbered in first-occurrence
//     order (the apply plan's x-groups).
//   * CSR tables over the ascending x groups: the position trie (for each
//     group and bit b, the size of the sibling subtree at b: the row's entry
//     for that group lands at r * G + rank(r ^ x_g), the rank built from these
//     sizes), each group's GF(2) span of z differences, and the sign-class fold
//     tables (the additions of make_row, qrusty/src/accel.rs:188-208, in term
//     order, once per sign class).  The fold tables depend on the
//     coefficients and are rebuilt by csr_values after every update; the rest
//     depends only on the masks.
// Every sum of coefficients here is the same sequence of FP64 additions, in
// the same order, as the reference's, so the tables are bit-identical to it.
#include <utility>

#include "qr_common.cuh"

namespace qr {

// ---------------------------------------------------------------- scans
constexpr int kScanThreads = 512;
constexpr int kScanPer = 4;
constexpr uint32_t kScanTile = kScanThreads * kScanPer;

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T x) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    return x;
}

// Exclusive scan of one value per thread over the block; *total = block sum.
template <typename T>
__device__ T block_excl_scan(T v, T *sh, T *total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const T inc = warp_incl_scan(v);
    if (lane == 31) sh[w] = inc;
    __syncthreads();
    if (w == 0) {
        T t = lane < nw ? sh[lane] : T(0);
        t = warp_incl_scan(t);
        if (lane < nw) sh[lane] = t;
    }
    __syncthreads();
    const T pre = (w ? sh[w - 1] : T(0)) + inc - v;
    *total = sh[nw - 1];
    __syncthreads();
    return pre;
}

template <typename T>
__global__ void __launch_bounds__(kScanThreads) scan_reduce_kernel(const T *in, uint64_t n,
                                                                   T *bsum) {
    __shared__ T sh[32];
    const uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanPer;
    T s = 0;
#pragma unroll
    for (int j = 0; j < kScanPer; ++j)
        if (base + j < n) s += in[base + j];
    T tot;
    block_excl_scan(s, sh, &tot);
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

// Exclusive scan of bsum[0, nb) in place; bsum[nb] = the total.
template <typename T>
__global__ void __launch_bounds__(kScanThreads) scan_top_kernel(T *bsum, uint32_t nb) {
    __shared__ T sh[32];
    T carry = 0;
    for (uint32_t c0 = 0; c0 < nb; c0 += kScanTile) {
        const uint32_t i0 = c0 + threadIdx.x * kScanPer;
        T v[kScanPer], s = 0;
#pragma unroll
        for (int j = 0; j < kScanPer; ++j) {
            v[j] = (i0 + j < nb) ? bsum[i0 + j] : T(0);
            s += v[j];
        }
        T tot;
        T run = carry + block_excl_scan(s, sh, &tot);
#pragma unroll
        for (int j = 0; j < kScanPer; ++j) {
            if (i0 + j < nb) bsum[i0 + j] = run;
            run += v[j];
        }
        carry += tot;
    }
    if (threadIdx.x == 0) bsum[nb] = carry;
}

template <typename T>
__global__ void __launch_bounds__(kScanThreads) scan_down_kernel(const T *in, uint64_t n,
                                                                 const T *bsum, uint32_t nb,
                                                                 T *out) {
    __shared__ T sh[32];
    const uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanPer;
    T v[kScanPer], s = 0;
#pragma unroll
    for (int j = 0; j < kScanPer; ++j) {
        v[j] = (base + j < n) ? in[base + j] : T(0);
        s += v[j];
    }
    T tot;
    T run = bsum[blockIdx.x] + block_excl_scan(s, sh, &tot);
#pragma unroll
    for (int j = 0; j < kScanPer; ++j) {
        if (base + j < n) out[base + j] = run;
        run += v[j];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = bsum[nb];
}

// out[i] = sum of in[0, i) for i <= n (out has n + 1 entries; in == out allowed).
template <typename T>
cudaError_t scan_excl(const T *in, T *out, uint64_t n, cudaStream_t st) {
    const uint64_t nb64 = (n + kScanTile - 1) / kScanTile;
    if (nb64 >= (1ull << 31)) return cudaErrorInvalidValue;
    const uint32_t nb = nb64 ? (uint32_t)nb64 : 1u;
    T *bsum = nullptr;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&bsum), (nb + 1) * sizeof(T), st);
    if (e != cudaSuccess) return e;
    scan_reduce_kernel<T><<<nb, kScanThreads, 0, st>>>(in, n, bsum);
    scan_top_kernel<T><<<1, kScanThreads, 0, st>>>(bsum, nb);
    scan_down_kernel<T><<<nb, kScanThreads, 0, st>>>(in, n, bsum, nb, out);
    count_launch(3);
    e = cudaGetLastError();
    cudaFreeAsync(bsum, st);
    return e;
}

// ---------------------------------------------------------------- radix sort
constexpr int kSortThreads = 256;
constexpr int kSortPer = 8;
constexpr uint32_t kSortTile = kSortThreads * kSortPer;
constexpr int kSortWarps = kSortThreads / 32;

// counts[d * nblk + blk] = number of keys of tile blk with digit d.
__global__ void __launch_bounds__(kSortThreads) radix_count_kernel(const uint64_t *key, uint64_t n,
                                                                   int shift, uint32_t nblk,
                                                                   uint32_t *counts) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint64_t base = (uint64_t)blockIdx.x * kSortTile;
#pragma unroll
    for (int j = 0; j < kSortPer; ++j) {
        const uint64_t i = base + (uint64_t)j * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(uint32_t)(key[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    counts[(uint64_t)threadIdx.x * nblk + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter of tile blk: a key's place is the digit's offset for the
// tile, plus the keys of that digit in earlier rounds, earlier warps of this
// round and lower lanes of its warp (tile order = input order).
__global__ void __launch_bounds__(kSortThreads) radix_scatter_kernel(
    const uint64_t *key, const uint32_t *val, uint64_t n, int shift, uint32_t nblk,
    const uint32_t *offs, uint64_t *okey, uint32_t *oval) {
    __shared__ uint32_t run[256];
    __shared__ uint32_t wc[kSortWarps][256];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    run[threadIdx.x] = offs[(uint64_t)threadIdx.x * nblk + blockIdx.x];
#pragma unroll
    for (int v = 0; v < kSortWarps; ++v) wc[v][threadIdx.x] = 0;
    __syncthreads();
    const uint64_t base = (uint64_t)blockIdx.x * kSortTile;
    const uint32_t below = (1u << lane) - 1u;
    for (int j = 0; j < kSortPer; ++j) {
        const uint64_t i = base + (uint64_t)j * kSortThreads + threadIdx.x;
        const bool ok = i < n;
        uint64_t k = 0;
        uint32_t v = 0, d = 256u + (uint32_t)lane;  // out-of-range lanes match nobody
        if (ok) {
            k = key[i];
            v = val[i];
            d = (uint32_t)(k >> shift) & 255u;
        }
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const uint32_t rk = __popc(peers & below);
        if (ok && rk == 0) wc[w][d] = __popc(peers);
        __syncthreads();
        if (ok) {
            uint32_t pos = run[d] + rk;
            for (int u = 0; u < w; ++u) pos += wc[u][d];
            okey[pos] = k;
            oval[pos] = v;
        }
        __syncthreads();
        uint32_t t = 0;
#pragma unroll
        for (int u = 0; u < kSortWarps; ++u) {
            t += wc[u][threadIdx.x];
            wc[u][threadIdx.x] = 0;
        }
        run[threadIdx.x] += t;
        __syncthreads();
    }
}

// Stable sort of (key, val) by key bits [0, bits), LSD.  The sorted pairs end
// in whichever of (*key, *val) / (key2, val2) the last pass wrote; the
// pointers are swapped so that *key and *val hold them.
cudaError_t radix_sort(uint64_t **key, uint32_t **val, uint64_t *key2, uint32_t *val2, uint64_t n,
                       int bits, cudaStream_t st) {
    if (n <= 1 || bits <= 0) return cudaSuccess;
    if (n > 0xffffffffull) return cudaErrorInvalidValue;
    const uint32_t nblk = (uint32_t)((n + kSortTile - 1) / kSortTile);
    uint32_t *counts = nullptr;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&counts),
                                    ((uint64_t)256 * nblk + 1) * sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    uint64_t *ka = *key, *kb = key2;
    uint32_t *va = *val, *vb = val2;
    for (int shift = 0; shift < bits; shift += 8) {
        radix_count_kernel<<<nblk, kSortThreads, 0, st>>>(ka, n, shift, nblk, counts);
        count_launch();
        e = cudaGetLastError();
        if (e == cudaSuccess) e = scan_excl<uint32_t>(counts, counts, (uint64_t)256 * nblk, st);
        if (e != cudaSuccess) break;
        radix_scatter_kernel<<<nblk, kSortThreads, 0, st>>>(ka, va, n, shift, nblk, counts, kb, vb);
        count_launch();
        e = cudaGetLastError();
        if (e != cudaSuccess) break;
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    cudaFreeAsync(counts, st);
    *key = ka;
    *val = va;
    return e;
}

// ---------------------------------------------------------------- grouping
static unsigned grid_of(uint64_t n, unsigned threads = 256) {
    const uint64_t g = (n + threads - 1) / threads;
    return g == 0 ? 1u : (g > 8192u ? 8192u : (unsigned)g);
}

#define GRID_STRIDE(i, n)                                                         \
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < (n); \
         i += (uint64_t)gridDim.x * blockDim.x)

__global__ void iota_kernel(uint32_t *v, uint64_t n) {
    GRID_STRIDE(i, n) v[i] = (uint32_t)i;
}

__global__ void gather_u64_kernel(const uint64_t *src, const uint32_t *idx, uint64_t n,
                                  uint64_t *dst) {
    GRID_STRIDE(i, n) dst[i] = src[idx[i]];
}

// H[i] = 1 where sorted position i starts a run of equal keys (ka, and kb
// when given) of the items P[i].
__global__ void head_kernel(const uint32_t *P, const uint64_t *ka, const uint64_t *kb, uint64_t n,
                            uint32_t *H) {
    GRID_STRIDE(i, n) {
        uint32_t h = 1;
        if (i > 0) {
            const uint32_t p = P[i], q = P[i - 1];
            h = (ka[p] != ka[q]) || (kb && kb[p] != kb[q]);
        }
        H[i] = h;
    }
}

// Runs: start[s] = first sorted position of run s, start[nrun] = n; isfirst
// (item order, zeroed by the caller) marks each run's first item.
__global__ void run_start_kernel(const uint32_t *H, const uint32_t *S, const uint32_t *P,
                                 uint64_t n, uint32_t *start, uint32_t *isfirst) {
    GRID_STRIDE(i, n) {
        if (H[i]) {
            start[S[i]] = (uint32_t)i;
            if (isfirst) isfirst[P[i]] = 1;
        }
        if (i == 0) start[S[n]] = (uint32_t)n;
    }
}

// Run s becomes group R[first item of s] (first-occurrence numbering).
__global__ void run_group_kernel(const uint32_t *start, const uint32_t *P, const uint32_t *R,
                                 uint64_t nrun, uint32_t *gid, uint32_t *glen) {
    GRID_STRIDE(s, nrun) {
        const uint32_t g = R[P[start[s]]];
        gid[s] = g;
        glen[g] = start[s + 1] - start[s];
    }
}

// Every sorted position: its item's group (map), its place in the group's
// member list (members in sorted = item order), the group's first item (rep).
__global__ void run_scatter_kernel(const uint32_t *H, const uint32_t *S, const uint32_t *start,
                                   const uint32_t *P, const uint32_t *gid, const uint32_t *goff,
                                   uint64_t n, uint32_t *map, uint32_t *members, uint32_t *rep) {
    GRID_STRIDE(i, n) {
        const uint32_t s = S[i] + H[i] - 1u;
        const uint32_t g = gid[s];
        const uint32_t item = P[i];
        if (map) map[item] = g;
        members[goff[g] + (uint32_t)i - start[s]] = item;
        if (H[i]) rep[g] = item;
    }
}

__global__ void merged_strings_kernel(const uint32_t *rep, const uint64_t *x, const uint64_t *z,
                                      uint64_t M, uint64_t *mx, uint64_t *mz, uint8_t *madj) {
    GRID_STRIDE(g, M) {
        const uint32_t k = rep[g];
        const uint64_t a = x[k], b = z[k];
        mx[g] = a;
        mz[g] = b;
        madj[g] = (uint8_t)(__popcll(a & b) & 1);
    }
}

__global__ void csr_groups_kernel(const uint32_t *start, const uint32_t *P, const uint64_t *x,
                                  uint64_t G, uint64_t *gx, uint32_t *goff) {
    GRID_STRIDE(g, G + 1) {
        goff[g] = start[g];
        if (g < G) gx[g] = x[P[start[g]]];
    }
}

struct Scratch {
    cudaStream_t st;
    void *p[16] = {};
    int k = 0;
    cudaError_t e = cudaSuccess;
    template <typename T>
    T *get(uint64_t count) {
        void *q = nullptr;
        if (e == cudaSuccess) e = cudaMallocAsync(&q, (count ? count : 1) * sizeof(T), st);
        if (e == cudaSuccess) p[k++] = q;
        return static_cast<T *>(q);
    }
    ~Scratch() {
        for (int i = 0; i < k; ++i) cudaFreeAsync(p[i], st);
    }
};

#define GR_TRY(call)                          \
    do {                                      \
        cudaError_t e_ = (call);              \
        if (e_ != cudaSuccess) return e_;     \
    } while (0)
#define GR_LAUNCH()                           \
    do {                                      \
        count_launch();                       \
        GR_TRY(cudaGetLastError());           \
    } while (0)

// Runs of equal keys among items sorted stably by key (P: item at each
// sorted position), numbered by first occurrence.  Writes goff (ngroups + 1),
// members (n), rep (ngroups) and, when given, map (n); returns ngroups.
static cudaError_t group_runs(const uint32_t *P, const uint64_t *ka, const uint64_t *kb, uint64_t n,
                              uint32_t *goff, uint32_t *members, uint32_t *rep, uint32_t *map,
                              uint64_t *ngroups, cudaStream_t st) {
    Scratch sc{st};
    uint32_t *H = sc.get<uint32_t>(n), *S = sc.get<uint32_t>(n + 1);
    uint32_t *start = sc.get<uint32_t>(n + 1), *isfirst = sc.get<uint32_t>(n + 1);
    uint32_t *R = sc.get<uint32_t>(n + 1), *gid = sc.get<uint32_t>(n);
    GR_TRY(sc.e);
    head_kernel<<<grid_of(n), 256, 0, st>>>(P, ka, kb, n, H);
    GR_LAUNCH();
    GR_TRY(scan_excl<uint32_t>(H, S, n, st));
    GR_TRY(cudaMemsetAsync(isfirst, 0, n * sizeof(uint32_t), st));
    run_start_kernel<<<grid_of(n), 256, 0, st>>>(H, S, P, n, start, isfirst);
    GR_LAUNCH();
    GR_TRY(scan_excl<uint32_t>(isfirst, R, n, st));
    uint32_t nrun = 0;
    GR_TRY(cudaMemcpyAsync(&nrun, S + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GR_TRY(cudaStreamSynchronize(st));
    // group lengths in group order (goff doubles as their buffer), then offsets
    run_group_kernel<<<grid_of(nrun), 256, 0, st>>>(start, P, R, nrun, gid, goff);
    GR_LAUNCH();
    GR_TRY(scan_excl<uint32_t>(goff, goff, nrun, st));
    run_scatter_kernel<<<grid_of(n), 256, 0, st>>>(H, S, start, P, gid, goff, n, map, members,
                                                   rep);
    GR_LAUNCH();
    *ngroups = nrun;
    return cudaSuccess;
}

cudaError_t group_terms(int n, uint64_t T, const uint64_t *x, const uint64_t *z,
                        const TermGroupsOut &o, TermGroupCounts *cnt, cudaStream_t st) {
    Scratch sc{st};
    uint64_t *ka = sc.get<uint64_t>(T), *kb = sc.get<uint64_t>(T);
    uint32_t *va = sc.get<uint32_t>(T), *vb = sc.get<uint32_t>(T);
    uint32_t *H = sc.get<uint32_t>(T), *S = sc.get<uint32_t>(T + 1);
    uint32_t *start = sc.get<uint32_t>(T + 1), *rep = sc.get<uint32_t>(T);
    GR_TRY(sc.e);
    // (1) terms stably by x: the CSR order and the ascending x groups
    GR_TRY(cudaMemcpyAsync(ka, x, T * sizeof(uint64_t), cudaMemcpyDeviceToDevice, st));
    iota_kernel<<<grid_of(T), 256, 0, st>>>(va, T);
    GR_LAUNCH();
    uint64_t *k1 = ka;
    uint32_t *v1 = va;
    GR_TRY(radix_sort(&k1, &v1, kb, vb, T, n, st));
    GR_TRY(cudaMemcpyAsync(o.order, v1, T * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
    gather_u64_kernel<<<grid_of(T), 256, 0, st>>>(z, o.order, T, o.tz);
    GR_LAUNCH();
    head_kernel<<<grid_of(T), 256, 0, st>>>(o.order, x, nullptr, T, H);
    GR_LAUNCH();
    GR_TRY(scan_excl<uint32_t>(H, S, T, st));
    run_start_kernel<<<grid_of(T), 256, 0, st>>>(H, S, o.order, T, start, nullptr);
    GR_LAUNCH();
    uint32_t G = 0;
    GR_TRY(cudaMemcpyAsync(&G, S + T, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GR_TRY(cudaStreamSynchronize(st));
    csr_groups_kernel<<<grid_of(G + 1), 256, 0, st>>>(start, o.order, x, G, o.gx, o.goff);
    GR_LAUNCH();
    cnt->G = G;

    // (2) terms by (x, z), ties in input order: z first, then stably by x
    GR_TRY(cudaMemcpyAsync(ka, z, T * sizeof(uint64_t), cudaMemcpyDeviceToDevice, st));
    iota_kernel<<<grid_of(T), 256, 0, st>>>(va, T);
    GR_LAUNCH();
    uint64_t *k2 = ka;
    uint32_t *v2 = va;
    GR_TRY(radix_sort(&k2, &v2, kb, vb, T, n, st));
    uint64_t *kx = (k2 == ka) ? kb : ka;  // the free key buffer
    gather_u64_kernel<<<grid_of(T), 256, 0, st>>>(x, v2, T, kx);
    GR_LAUNCH();
    uint32_t *vfree = (v2 == va) ? vb : va;
    uint64_t *k3 = kx;
    uint32_t *v3 = v2;
    GR_TRY(radix_sort(&k3, &v3, k2, vfree, T, n, st));
    uint64_t M = 0;
    GR_TRY(group_runs(v3, x, z, T, o.mm_off, o.mm_terms, rep, o.mmap, &M, st));
    merged_strings_kernel<<<grid_of(M), 256, 0, st>>>(rep, x, z, M, o.mx, o.mz, o.madj);
    GR_LAUNCH();
    cnt->M = M;

    // (3) merged strings stably by x: the apply plan's x-groups
    GR_TRY(cudaMemcpyAsync(ka, o.mx, M * sizeof(uint64_t), cudaMemcpyDeviceToDevice, st));
    iota_kernel<<<grid_of(M), 256, 0, st>>>(va, M);
    GR_LAUNCH();
    uint64_t *k4 = ka;
    uint32_t *v4 = va;
    GR_TRY(radix_sort(&k4, &v4, kb, vb, M, n, st));
    uint64_t Ga = 0;
    GR_TRY(group_runs(v4, o.mx, nullptr, M, o.ag_off, o.ag_mem, rep, nullptr, &Ga, st));
    cnt->Ga = Ga;
    GR_TRY(cudaStreamSynchronize(st));
    return cudaSuccess;
}

// ---------------------------------------------------------------- CSR tables
__device__ __forceinline__ uint32_t lower_bound_u64(const uint64_t *a, uint32_t lo, uint32_t hi,
                                                    uint64_t v) {
    while (lo < hi) {
        const uint32_t mid = lo + ((hi - lo) >> 1);
        if (a[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Position trie over the ascending x masks: at bit b, the groups sharing x_g's
// bits above b form a range; where bit b splits it, sigma_{g,b} is the size of
// the other side (+ when x_g is on the 0-side, - on the 1-side).
__global__ void csr_trie_kernel(const uint64_t *gx, uint32_t G, int n, uint64_t *pmask,
                                int32_t *sig) {
    GRID_STRIDE(g, G) {
        const uint64_t x = gx[g];
        uint64_t pm = 0;
        for (int b = n - 1; b >= 0; --b) {
            const uint64_t pre = (x >> (b + 1)) << (b + 1);  // b + 1 <= 63
            const uint32_t lo = lower_bound_u64(gx, 0, G, pre);
            const uint32_t hi = lower_bound_u64(gx, lo, G, pre + (2ull << b));
            const uint32_t mid = lower_bound_u64(gx, lo, hi, pre | (1ull << b));
            int32_t s = 0;
            if (mid > lo && mid < hi) {
                pm |= 1ull << b;
                s = ((x >> b) & 1) ? -(int32_t)(mid - lo) : (int32_t)(hi - mid);
            }
            sig[g * (uint64_t)n + b] = s;
        }
        pmask[g] = pm;
    }
}

// GF(2) span of tz[k] ^ tz[k0] over k in [k0, k1): basis in insertion order,
// each difference reduced by the basis in descending pivot (msb) order;
// coord[k] = its coordinates (bit i: basis i).  Stops at the first
// difference that would need basis vector DMAX + 1: *used = terms spanned,
// return = -1 then, else the rank.  *nb = basis vectors found.
template <int DMAX>
__device__ int group_span(const uint64_t *tz, uint32_t k0, uint32_t k1, uint64_t *basis,
                          uint16_t *coord, uint32_t *used, int *nb) {
    const uint64_t z0 = tz[k0];
    int cnt = 0;
    int ord[DMAX];  // basis indices by descending value (= descending pivot)
    for (uint32_t k = k0; k < k1; ++k) {
        uint64_t v = tz[k] ^ z0;
        uint32_t c = 0;
        for (int j = 0; j < cnt; ++j) {
            const int i = ord[j];
            const uint64_t bv = basis[i];
            if ((v >> (63 - __clzll(bv))) & 1ull) {
                v ^= bv;
                c |= 1u << i;
            }
        }
        if (v != 0) {
            if (cnt >= DMAX) {
                *used = k - k0;
                *nb = cnt;
                return -1;
            }
            c |= 1u << cnt;
            basis[cnt] = v;
            int p = cnt;
            while (p > 0 && basis[ord[p - 1]] < v) {
                ord[p] = ord[p - 1];
                --p;
            }
            ord[p] = cnt;
            ++cnt;
        }
        coord[k] = (uint16_t)c;
    }
    *used = k1 - k0;
    *nb = cnt;
    return cnt;
}

// Per group: rank-<= kCsrMaxRank span (class table of 2^(d+1) entries) or
// fold mode with the leading terms of span rank <= kCsrPrefixRank folded per
// class (prefix table).  tab and zparts are filled later.
__global__ void csr_span_kernel(uint32_t G, const uint32_t *goff, const uint64_t *tz,
                                CsrGroup *grp, uint16_t *coord, uint64_t *ctsz, uint64_t *ptsz,
                                uint32_t *isfold, uint64_t *gbeta) {
    GRID_STRIDE(g, G) {
        CsrGroup d;
        d.k0 = goff[g];
        d.k1 = goff[g + 1];
        d.z0 = tz[d.k0];
        for (int j = 0; j < kCsrMaxRank; ++j) d.beta[j] = 0;
        d.tab = 0;
        d.zparts = 0;
        d.pre = 0;
        uint64_t basis[kCsrPrefixRank];
        uint32_t used;
        int nb;
        const int r = group_span<kCsrMaxRank>(tz, d.k0, d.k1, basis, coord, &used, &nb);
        if (r >= 0) {
            d.d = (uint32_t)r;
            for (int j = 0; j < r; ++j) d.beta[j] = basis[j];
            ctsz[g] = 2ull << r;
            ptsz[g] = 0;
            isfold[g] = 0;
        } else {
            d.d = kCsrFold;
            group_span<kCsrPrefixRank>(tz, d.k0, d.k1, basis, coord, &used, &nb);
            // the kernel continues the term-order fold after the prefix, so a
            // prefix cut short of a 24-bit count gives the same additions
            const uint32_t m = used < 0xffffffu ? used : 0xffffffu;
            ptsz[g] = 0;
            if (m >= 2) {
                d.pre = m | ((uint32_t)nb << 24);
                ptsz[g] = 2ull << nb;
            }
            for (int j = 0; j < kCsrPrefixRank; ++j)
                gbeta[g * (uint64_t)kCsrPrefixRank + j] = j < nb ? basis[j] : 0ull;
            ctsz[g] = 0;
            isfold[g] = 1;
        }
        grp[g] = d;
    }
}

// Table offsets, fold list and prefix bases from the scanned sizes (foff:
// exclusive scan of the fold flags; a group is in fold mode iff d == kCsrFold).
__global__ void csr_desc_kernel(uint32_t G, CsrGroup *grp, const uint64_t *ctoff,
                                const uint64_t *ptoff, const uint32_t *foff,
                                const uint64_t *gbeta, uint32_t *fold, uint64_t *pbeta) {
    GRID_STRIDE(g, G) {
        if (grp[g].d == kCsrFold) {
            const uint32_t f = foff[g];
            fold[f] = (uint32_t)g;
            grp[g].tab = grp[g].pre ? (uint32_t)ptoff[g] : 0u;
            for (int j = 0; j < kCsrPrefixRank; ++j)
                pbeta[(uint64_t)f * kCsrPrefixRank + j] = gbeta[g * (uint64_t)kCsrPrefixRank + j];
        } else {
            grp[g].tab = (uint32_t)ctoff[g];
        }
    }
}

cudaError_t csr_structure(int n, uint64_t G, const uint64_t *gx, const uint32_t *goff,
                          const uint64_t *tz, const CsrStructOut &o, CsrStructCounts *cnt,
                          cudaStream_t st) {
    if (G == 0 || G > 0xffffffffull) return cudaErrorInvalidValue;
    Scratch sc{st};
    uint64_t *ctsz = sc.get<uint64_t>(G + 1), *ptsz = sc.get<uint64_t>(G + 1);
    uint32_t *foff = sc.get<uint32_t>(G + 1);
    uint64_t *gbeta = sc.get<uint64_t>(G * kCsrPrefixRank);
    GR_TRY(sc.e);
    csr_trie_kernel<<<grid_of(G), 256, 0, st>>>(gx, (uint32_t)G, n, o.pmask, o.sig);
    GR_LAUNCH();
    csr_span_kernel<<<grid_of(G, 128), 128, 0, st>>>((uint32_t)G, goff, tz, o.grp, o.coord, ctsz,
                                                     ptsz, foff, gbeta);
    GR_LAUNCH();
    GR_TRY(scan_excl<uint64_t>(ctsz, ctsz, G, st));
    GR_TRY(scan_excl<uint64_t>(ptsz, ptsz, G, st));
    GR_TRY(scan_excl<uint32_t>(foff, foff, G, st));
    csr_desc_kernel<<<grid_of(G), 256, 0, st>>>((uint32_t)G, o.grp, ctsz, ptsz, foff, gbeta,
                                                o.fold, o.pbeta);
    GR_LAUNCH();
    uint64_t tot[2] = {0, 0};
    uint32_t nfold = 0;
    GR_TRY(cudaMemcpyAsync(&tot[0], ctsz + G, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    GR_TRY(cudaMemcpyAsync(&tot[1], ptsz + G, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    GR_TRY(cudaMemcpyAsync(&nfold, foff + G, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GR_TRY(cudaStreamSynchronize(st));
    cnt->nctab = tot[0];
    cnt->nptab = tot[1];
    cnt->nfold = nfold;
    return cudaSuccess;
}

// Coefficient-dependent CSR data: tc (c'_k in CSR order), the fold groups'
// zero-part flags, and the class / prefix tables: for class c, the term-order
// fold of (-1)^popc(c & (1 | coord_k << 1)) c'_k.
__global__ void csr_tc_kernel(const uint32_t *order, const double2 *coef, const uint8_t *phase,
                              uint64_t T, double2 *tc) {
    GRID_STRIDE(i, T) {
        const uint32_t k = order[i];
        tc[i] = make_param(coef[k], phase[k]);
    }
}

__global__ void __launch_bounds__(128) csr_fold_tables_kernel(uint32_t G, CsrGroup *grp,
                                                              const uint16_t *coord,
                                                              const double2 *tc, double2 *ctab,
                                                              double2 *ptab) {
    for (uint32_t g = blockIdx.x; g < G; g += gridDim.x) {
        const uint32_t d = grp[g].d, tab = grp[g].tab, pre = grp[g].pre;
        const uint32_t k0 = grp[g].k0, k1 = grp[g].k1;
        uint32_t m, ncls;
        double2 *out;
        if (d == kCsrFold) {
            int rz = 1, iz = 1;
            for (uint32_t k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
                const double2 c = tc[k];
                rz &= c.x == 0.0;
                iz &= c.y == 0.0;
            }
            rz = __syncthreads_and(rz);
            iz = __syncthreads_and(iz);
            if (threadIdx.x == 0) grp[g].zparts = (rz ? 1u : 0u) | (iz ? 2u : 0u);
            m = pre & 0xffffffu;
            if (m < 2) continue;
            ncls = 2u << (pre >> 24);
            out = ptab + tab;
        } else {
            m = k1 - k0;
            ncls = 2u << d;
            out = ctab + tab;
        }
        for (uint32_t c = threadIdx.x; c < ncls; c += blockDim.x) {
            double2 v = make_double2(0.0, 0.0);
            for (uint32_t k = k0; k < k0 + m; ++k) {
                const uint32_t sel = 1u | ((uint32_t)coord[k] << 1);
                double2 t = tc[k];
                if (__popc(c & sel) & 1) {
                    t.x = -t.x;
                    t.y = -t.y;
                }
                if (k == k0) {
                    v = t;
                } else {
                    v.x = __dadd_rn(v.x, t.x);
                    v.y = __dadd_rn(v.y, t.y);
                }
            }
            out[c] = v;
        }
    }
}

cudaError_t csr_values(uint64_t G, uint64_t T, const uint32_t *order, const double2 *coef,
                       const uint8_t *phase, double2 *tc, CsrGroup *grp, const uint16_t *coord,
                       double2 *ctab, double2 *ptab, cudaStream_t st) {
    csr_tc_kernel<<<grid_of(T), 256, 0, st>>>(order, coef, phase, T, tc);
    GR_LAUNCH();
    const unsigned gb = G < 4096 ? (unsigned)(G ? G : 1) : 4096u;
    csr_fold_tables_kernel<<<gb, 128, 0, st>>>((uint32_t)G, grp, coord, tc, ctab, ptab);
    GR_LAUNCH();
    return cudaSuccess;
}

}  // namespace qr
