// Device-side building blocks shared by the qmbx kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/qmbx.h"
#include "common.h"
#include "format.h"
#include "profile.h"

#define QMBX_CUDA_TRY(expr)                                                                          \
    do {                                                                                             \
        cudaError_t qmbx_err_ = (expr);                                                              \
        if (qmbx_err_ != cudaSuccess) {                                                              \
            return ::qmbx::fail(QMBX_ERR_CUDA, "%s failed: %s", #expr, cudaGetErrorString(qmbx_err_)); \
        }                                                                                            \
    } while (0)

#define QMBX_LAUNCH_CHECK(what)                                                                          \
    do {                                                                                                 \
        cudaError_t qmbx_err_ = cudaGetLastError();                                                      \
        if (qmbx_err_ != cudaSuccess) {                                                                  \
            return ::qmbx::fail(QMBX_ERR_CUDA, "launch of %s failed: %s", what, cudaGetErrorString(qmbx_err_)); \
        }                                                                                                \
    } while (0)

namespace qmbx {

constexpr int kThreads = 256;

inline unsigned grid_for(int64_t n, int per_block) {
    int64_t g = (n + per_block - 1) / per_block;
    return (unsigned)(g > 0 ? g : 1);
}

// ---------------------------------------------------------------------------
// keys: W big-endian 64-bit words per configuration (see format.h)
// ---------------------------------------------------------------------------

template <int W>
struct Key {
    uint64_t w[W];
};

template <int W>
__device__ __forceinline__ Key<W> load_key(const uint64_t* __restrict__ keys, int64_t i) {
    Key<W> k;
    if constexpr (W == 2) {
        ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(keys) + i);
        k.w[0] = v.x;
        k.w[1] = v.y;
    } else if constexpr (W == 4) {
        ulonglong2 a = __ldg(reinterpret_cast<const ulonglong2*>(keys) + 2 * i);
        ulonglong2 b = __ldg(reinterpret_cast<const ulonglong2*>(keys) + 2 * i + 1);
        k.w[0] = a.x;
        k.w[1] = a.y;
        k.w[2] = b.x;
        k.w[3] = b.y;
    } else {
#pragma unroll
        for (int q = 0; q < W; ++q) k.w[q] = __ldg(keys + i * W + q);
    }
    return k;
}

template <int W>
__device__ __forceinline__ void store_key(uint64_t* __restrict__ keys, int64_t i, const Key<W>& k) {
#pragma unroll
    for (int q = 0; q < W; ++q) keys[i * W + q] = k.w[q];
}

// -1, 0, 1 as a is lexicographically below, equal to or above b
template <int W>
__device__ __forceinline__ int key_cmp(const Key<W>& a, const Key<W>& b) {
#pragma unroll
    for (int q = 0; q < W; ++q) {
        if (a.w[q] != b.w[q]) return a.w[q] < b.w[q] ? -1 : 1;
    }
    return 0;
}

template <int W>
__device__ __forceinline__ bool key_eq(const Key<W>& a, const Key<W>& b) {
    bool e = true;
#pragma unroll
    for (int q = 0; q < W; ++q) e &= a.w[q] == b.w[q];
    return e;
}

// ---------------------------------------------------------------------------
// open-addressing hash set over the keys of a row set
//
// Slots come in buckets of four; bucket j occupies 32 bytes (one L2 sector)
// of the slot array: the four 32-bit fingerprints, then the four 32-bit rows.
// A fingerprint is never all ones, and both words are all ones in an empty
// slot.  A lookup reads the bucket's fingerprints with one 16-byte load (the
// whole sector comes into L1 with it) and reads a row only on a fingerprint
// match, so an unsuccessful lookup costs one load and a successful one finds
// its row in L1.  Linear probing, load factor at most 1/4.
// ---------------------------------------------------------------------------

constexpr uint32_t kEmptyTag = 0xffffffffu;
constexpr uint32_t kEmptyRow = 0xffffffffu;

// Multiply mixing, one 64-bit multiply per key word; the high bits of the
// result depend on every bit of the key and select the bucket.
template <int W>
__host__ __device__ __forceinline__ uint64_t key_hash(const Key<W>& k) {
    uint64_t h = k.w[0] * 0x9E3779B97F4A7C15ull;
    for (int q = 1; q < W; ++q) h = (h ^ (h >> 31) ^ k.w[q]) * 0xBF58476D1CE4E5B9ull;
    return h;
}

struct HashView {
    const uint32_t* slots; // 8 words per bucket (see above)
    const uint64_t* keys;  // keys of the set's rows, n x W
    uint64_t mask;         // slot count - 1 (a power of two minus one)
    int shift;             // 64 - log2(slot count / kBucket)
    const uint32_t* bloom; // optional filter over the keys (NULL: none)
    uint32_t bloom_mask;   // filter words - 1
};

// Blocked Bloom filter over a set's keys: two bits in one 32-bit word per
// key, all taken from a remix of the key's hash.  With 16 filter bits per
// key it rejects ~98 % of absent keys with one 4-byte load, and a lookup
// probes the hash table only when the filter lets the key through.  Sets
// too large for 16 bits per key in 128 KB get no filter: measured on GB300,
// a sparser filter (5 bits per key, ~10 % false positives) made lookups
// slower than the bucket probe alone.
constexpr uint32_t kBloomMaxWords = 32768;  // 128 KB

__host__ __device__ __forceinline__ uint64_t bloom_mix(uint64_t hv) {
    return (hv ^ (hv >> 29)) * 0xBF58476D1CE4E5B9ull;
}
__host__ __device__ __forceinline__ uint32_t bloom_word(uint64_t f, uint32_t mask) { return (uint32_t)(f >> 40) & mask; }
__host__ __device__ __forceinline__ uint32_t bloom_bits(uint64_t f) {
    return (1u << ((f >> 8) & 31)) | (1u << ((f >> 13) & 31));
}

// Filter words for a set of n rows: 16 bits per row rounded up to a power
// of two (at least 256 words); 0 (no filter) above kBloomMaxWords.
inline uint32_t bloom_words_for(int64_t n) {
    if (n <= 0) return 0;
    uint64_t words = 256;
    while (32 * words < 16 * (uint64_t)n && words < kBloomMaxWords) words <<= 1;
    return 32 * words >= 16 * (uint64_t)n ? (uint32_t)words : 0;
}

constexpr int kBucket = 4;

// Word offsets of slot i's fingerprint and row in the slot array.
__host__ __device__ __forceinline__ uint64_t slot_tag_word(uint64_t i) { return (i >> 2) * 8 + (i & 3); }
__host__ __device__ __forceinline__ uint64_t slot_row_word(uint64_t i) { return (i >> 2) * 8 + 4 + (i & 3); }

// Fingerprint of a key: the hash's high word, kept off the empty value.
__host__ __device__ __forceinline__ uint32_t hash_tag(uint64_t hv) {
    const uint32_t t = (uint32_t)(hv >> 32);
    return t == kEmptyTag ? kEmptyTag - 1u : t;
}

// First slot of a key's home bucket, selected by the top bits of its hash.
__host__ __device__ __forceinline__ uint64_t hash_home(uint64_t hv, int shift) {
    return (hv >> shift) * (uint64_t)kBucket;
}

__host__ __device__ __forceinline__ int hash_shift(uint64_t slots) {
    int s = 64;
    for (uint64_t b = slots / kBucket; b > 1; b >>= 1) --s;
    return s;
}

// Row stored for key (the first row holding it), or -1.  Inserts fill the
// probe sequence slot by slot, so a bucket with an empty slot ends an
// unsuccessful search.
template <int W>
__device__ __forceinline__ int64_t hash_find(const HashView& h, const Key<W>& key) {
    const uint64_t hv = key_hash<W>(key);
    if (h.bloom != nullptr) {
        const uint64_t f = bloom_mix(hv);
        const uint32_t bits = bloom_bits(f);
        if ((__ldg(h.bloom + bloom_word(f, h.bloom_mask)) & bits) != bits) return -1;
    }
    const uint32_t fp = hash_tag(hv);
    uint64_t b = hash_home(hv, h.shift);
    for (uint64_t probe = 0; probe <= h.mask; probe += kBucket) {
        const uint32_t* bucket = h.slots + 2 * b;
        const uint4 t4 = __ldg(reinterpret_cast<const uint4*>(bucket));
        // the four fingerprints compared at once: a miss (no match, an empty slot) costs one branch
        const bool open = (t4.x == kEmptyTag) | (t4.y == kEmptyTag) | (t4.z == kEmptyTag) | (t4.w == kEmptyTag);
        unsigned match = (unsigned)(t4.x == fp) | ((unsigned)(t4.y == fp) << 1) | ((unsigned)(t4.z == fp) << 2) |
                         ((unsigned)(t4.w == fp) << 3);
        while (match != 0) {
            const int k = __ffs(match) - 1;
            match &= match - 1;
            const uint32_t row = __ldg(bucket + kBucket + k);
            if (row != kEmptyRow && key_eq<W>(load_key<W>(h.keys, (int64_t)row), key)) return (int64_t)row;
        }
        if (open) return -1;
        b = (b + kBucket) & h.mask;
    }
    return -1;
}

// ---------------------------------------------------------------------------
// term table parts on the device
// ---------------------------------------------------------------------------

struct PartView {
    const ulonglong2* test;    // [W][stride]: (mask, val) per word
    const ulonglong2* apply;   // [W][stride]: (flip, par) per word
    int64_t stride;            // terms in the part (n may be set to 0 to skip a part)
    const double2* coef;
    const float4* coef32;
    const int32_t* orig;
    const float* norm;
    const int2* groups;        // [start, end) of every pivot group
    const uint64_t* single_ne; // [W]
    const uint64_t* pair_ne;   // [64W][W]
    const int4* nonempty;      // (start, end, p, q) of the non-empty groups
    int64_t n_nonempty;
    int64_t n;
    int wide;                  // groups are large: walk each with lanes over its terms
    const uint4* narrow;       // (mask, val, flip, par) >> 32 of every term (tables of <= 32 sites), or NULL
};

inline PartView part_view(const void* table_host, const void* table_dev, int which) {
    const qmbx_table_header* h = header_of(table_host);
    const qmbx_table_part& p = h->part[which];
    const char* base = static_cast<const char*>(table_dev);
    PartView v;
    v.test = reinterpret_cast<const ulonglong2*>(base + p.off_test);
    v.apply = reinterpret_cast<const ulonglong2*>(base + p.off_apply);
    v.stride = p.n;
    v.coef = reinterpret_cast<const double2*>(base + p.off_coef);
    v.coef32 = reinterpret_cast<const float4*>(base + p.off_coef32);
    v.orig = reinterpret_cast<const int32_t*>(base + p.off_orig);
    v.norm = reinterpret_cast<const float*>(base + p.off_norm);
    v.groups = reinterpret_cast<const int2*>(base + p.off_groups);
    v.single_ne = reinterpret_cast<const uint64_t*>(base + p.off_single_ne);
    v.pair_ne = reinterpret_cast<const uint64_t*>(base + p.off_pair_ne);
    v.nonempty = reinterpret_cast<const int4*>(base + p.off_nonempty);
    v.n_nonempty = p.n_nonempty;
    v.n = p.n;
    v.wide = p.wide_groups;
    v.narrow = p.off_narrow != 0 ? reinterpret_cast<const uint4*>(base + p.off_narrow) : nullptr;
    return v;
}

int check_table(const void* table_host, const void* table_dev);

// Workspace of an apply_within call for one value of same_configs (apply.cu).
int apply_within_workspace_for(const void* table_host, int64_t n_i, int64_t n_j, bool same, uint64_t* bytes);

// ---------------------------------------------------------------------------
// the enumeration kernel: every (configuration, term) pair of one or two
// table parts, terms staged through shared memory tile by tile so that all
// threads of a block test the same term at the same time (broadcast reads).
// ---------------------------------------------------------------------------

constexpr int kTermTile = 128;

template <int W>
struct __align__(16) TermTile {
    uint64_t m[kTermTile][4 * W];  // per word: mask, val, flip, par
};

// Copy count terms from t0 into records of 4W words (per word mask, val,
// flip, par) at dst, threads striding over terms one word at a time.
template <int W>
__device__ __forceinline__ void stage_terms(uint64_t* dst, const PartView& part, int64_t t0, int count, int tid,
                                            int nthreads) {
#pragma unroll
    for (int q = 0; q < W; ++q) {
        const ulonglong2* test = part.test + (int64_t)q * part.stride + t0;
        const ulonglong2* apply = part.apply + (int64_t)q * part.stride + t0;
        for (int k = tid; k < count; k += nthreads) {
            ulonglong2* rec = reinterpret_cast<ulonglong2*>(dst + (int64_t)k * 4 * W + 4 * q);
            rec[0] = __ldg(test + k);
            rec[1] = __ldg(apply + k);
        }
    }
}

template <int W>
__device__ __forceinline__ void stage_tile(TermTile<W>& tile, const PartView& part, int64_t t0, int count) {
    stage_terms<W>(&tile.m[0][0], part, t0, count, threadIdx.x, blockDim.x);
}

template <int W>
__device__ __forceinline__ bool term_applies(const uint64_t* t, const Key<W>& c) {
    uint64_t bad = 0;
#pragma unroll
    for (int q = 0; q < W; ++q) bad |= (c.w[q] ^ t[4 * q + 1]) & t[4 * q];
    return bad == 0;
}

template <int W>
__device__ __forceinline__ int term_image(const uint64_t* t, const Key<W>& c, Key<W>& img) {
    int par = 0;
#pragma unroll
    for (int q = 0; q < W; ++q) {
        img.w[q] = c.w[q] ^ t[4 * q + 2];
        par += __popcll(c.w[q] & t[4 * q + 3]);
    }
    return par & 1;
}

// Row sources of the enumeration kernel: packed keys, or raw rows packed on the fly.
template <int W>
struct KeyRows {
    const uint64_t* keys;
    __device__ __forceinline__ Key<W> get(int64_t i) const { return load_key<W>(keys, i); }
};

template <int W>
struct ByteRows {
    const uint8_t* rows;
    int nq;
    __device__ __forceinline__ Key<W> get(int64_t i) const {
        Key<W> k;
        const uint8_t* r = rows + i * nq;
#pragma unroll
        for (int q = 0; q < W; ++q) {
            uint64_t w = 0;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                int b = 8 * q + j;
                uint64_t byte = b < nq ? (uint64_t)r[b] : 0;
                w |= byte << (8 * (7 - j));
            }
            k.w[q] = w;
        }
        return k;
    }
};

// Test one row against every term of a staged tile: bit k of hit[k / 32] is
// set when term k applies.  Full tiles are tested without bounds checks.
template <int W>
__device__ __forceinline__ void test_tile(const TermTile<W>& tile, int count, const Key<W>& c,
                                          uint32_t (&hit)[kTermTile / 32]) {
    if (count == kTermTile) {
#pragma unroll
        for (int w = 0; w < kTermTile / 32; ++w) {
            uint32_t m = 0;
#pragma unroll
            for (int b = 0; b < 32; ++b) m |= (uint32_t)term_applies<W>(tile.m[32 * w + b], c) << b;
            hit[w] = m;
        }
    } else {
#pragma unroll
        for (int w = 0; w < kTermTile / 32; ++w) {
            uint32_t m = 0;
            for (int b = 0; b < 32 && 32 * w + b < count; ++b) m |= (uint32_t)term_applies<W>(tile.m[32 * w + b], c) << b;
            hit[w] = m;
        }
    }
}

// What a forward walk of apply_within found, kept so that the adjoint
// product on the same rows needs no second walk (qmbx_*_logged): one record
// per (term, walked row) pair whose image was found among the looked-up
// rows, and per walked row the summed diagonal coefficient.  hits == NULL:
// nothing is recorded.
struct HitLog {
    int4* hits;                  // (walked first row, looked-up row, slot | parity << 31, 0)
    unsigned long long* count;   // records found (more than cap: the log is incomplete)
    int64_t cap;
    int2* diag_rows;             // per walk index: (walked first row, looked-up row or -1)
    double2* diag_val;           // per walk index: summed diagonal coefficient (sign folded)
};

// Record n (<= 32) queued hits (int2: slot | parity << 31, looked-up row) of
// the walked row; every lane of the warp calls it.
__device__ __forceinline__ void log_hits(const HitLog& log, int walked, const int2* q, int n, int lane) {
    if (log.hits == nullptr || n <= 0) return;
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(log.count, (unsigned long long)n);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (lane < n && base + lane < (unsigned long long)log.cap) {
        const int2 h = q[lane];
        log.hits[base + lane] = make_int4(walked, h.y, h.x, 0);
    }
}

// One hit recorded by one thread (walks without hit queues).
__device__ __forceinline__ void log_hit(const HitLog& log, int walked, int2 h) {
    if (log.hits == nullptr) return;
    const unsigned long long at = atomicAdd(log.count, 1ull);
    if (at < (unsigned long long)log.cap) log.hits[at] = make_int4(walked, h.y, h.x, 0);
}

// The walked row's diagonal record (walk index u).
__device__ __forceinline__ void log_diag(const HitLog& log, int64_t u, int walked, int64_t pos, double re, double im) {
    if (log.hits == nullptr) return;
    log.diag_rows[u] = make_int2(walked, (int)pos);
    log.diag_val[u] = make_double2(re, im);
}

// Defaults for the optional parts of the visitor protocol: no shared memory,
// no per-block set-up or flush, no hit log.
struct VisitorBase {
    template <class Acc, class K>
    __device__ __forceinline__ void flush(Acc&, int64_t, const K&) const {}
    static constexpr int kShared = 0;
    static constexpr bool kTiledDense = false;  // tiled walks may run as enumerate_dense_kernel (W <= 2)
    static constexpr bool kBatched = false;  // hits are queued and processed by apply_hit with full lanes
    static constexpr bool kStateless = false; // pivot walks: hits carry their row and need no per-row state
    template <class Acc>
    __device__ __forceinline__ void apply_hit(Acc&, int2) const {}
    __device__ __forceinline__ void block_init(int*) const {}
    __device__ __forceinline__ void block_flush(int*) const {}
    // hit-queue drains: record the n hits about to be applied (all lanes call)
    template <class Acc>
    __device__ __forceinline__ void record_hits(const Acc&, const int2*, int, int) const {}
    // one hit applied at once by one lane (serial group walks)
    template <class Acc>
    __device__ __forceinline__ void record_hit(const Acc&, int2) const {}
    // pivot hit-queue drains: the same for (slot | parity << 31, looked-up row, walk index) hits
    __device__ __forceinline__ void record_row_hits(const int4*, int, int) const {}
};

// Visitor protocol:
//   struct V : VisitorBase { struct Acc; init(Acc&, int64_t row, const Key<W>&, int* shared);
//              visit(Acc&, const Key<W>& c, const Key<W>& image, int parity, int64_t slot);
//              visit_diag(Acc&, const Key<W>& c, int parity, int64_t slot);
//              finish(Acc&, int64_t row, const Key<W>&); }
// Rows [0, *n_rows) (or [0, n_max) when n_rows is NULL) of src are visited;
// off holds the terms that change a row, diag the ones that do not.  Each
// thread owns one row: it first tests its row against a whole tile of terms
// (cheap, branch-free, all lanes reading the same term) and then visits only
// the terms that applied.
template <int W, class V, class Src>
__device__ __forceinline__ void enumerate_rows(const V& v, const Src& src, const int* __restrict__ n_rows,
                                               int64_t n_max, const PartView& off, const PartView& diag) {
    __shared__ TermTile<W> tile;
    const int64_t n = n_rows ? (int64_t)*n_rows : n_max;
    if ((int64_t)blockIdx.x * blockDim.x >= n) return;
    const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = row < n;
    Key<W> c;
    if (live) {
        c = src.get(row);
    } else {
#pragma unroll
        for (int q = 0; q < W; ++q) c.w[q] = 0;
    }
    __shared__ int sh[V::kShared > 0 ? V::kShared : 1];
    v.block_init(sh);
    __syncthreads();
    typename V::Acc acc;
    if (live) v.init(acc, row, c, sh);  // init may read per-row data: never for padding lanes
    for (int part = 0; part < 2; ++part) {
        const PartView& pv = part == 0 ? off : diag;
        for (int64_t t0 = 0; t0 < pv.n; t0 += kTermTile) {
            const int count = (int)(pv.n - t0 < kTermTile ? pv.n - t0 : kTermTile);
            __syncthreads();
            stage_tile<W>(tile, pv, t0, count);
            __syncthreads();
            if (!live) continue;
            uint32_t hit[kTermTile / 32];
            test_tile<W>(tile, count, c, hit);
#pragma unroll
            for (int w = 0; w < kTermTile / 32; ++w) {
                uint32_t m = hit[w];
                while (m) {
                    const int k = 32 * w + __ffs(m) - 1;
                    m &= m - 1;
                    Key<W> img;
                    const int parity = term_image<W>(tile.m[k], c, img);
                    if (part == 0) {
                        v.visit(acc, c, img, parity, t0 + k);
                    } else {
                        v.visit_diag(acc, c, parity, t0 + k);
                    }
                }
            }
        }
    }
    if (live) v.finish(acc, row, c);
    __syncthreads();
    v.block_flush(sh);
}

template <int W, class V, class Src>
__global__ void __launch_bounds__(kThreads) enumerate_kernel(V v, Src src, const int* __restrict__ n_rows,
                                                             int64_t n_max, PartView off, PartView diag) {
    enumerate_rows<W>(v, src, n_rows, n_max, off, diag);
}

// The same walk with five resident blocks per SM asked of the compiler (at
// most 48 registers a thread), for visitors with kTiledDense and keys of one
// or two words, which fit that without spills: their row lookups get 40
// warps per SM to hide L2 latency behind instead of 32 (C4 forward walk
// 1.23 -> 1.15 ms on GB300).
template <int W, class V, class Src>
__global__ void __launch_bounds__(kThreads, 5) enumerate_dense_kernel(V v, Src src, const int* __restrict__ n_rows,
                                                                      int64_t n_max, PartView off, PartView diag) {
    enumerate_rows<W>(v, src, n_rows, n_max, off, diag);
}

// The tiled walk of a diagonal part with each row shared by L lanes (lane
// group g = threadIdx.x / L of the block): lane s of a group tests terms s,
// s + L, ... of every staged tile, the group's sums are combined with
// shuffles (the visitor's reduce_lanes<L>), and its first lane finishes the
// row.  For diagonal passes over too few rows to fill the GPU with a thread
// each (C2's 20,000 rows are 79 blocks of 256).  The visitor's init must read
// nothing: it also runs for the lanes past the last row.
template <int W, int L, class V, class Src>
__global__ void __launch_bounds__(kThreads) diag_split_kernel(V v, Src src, const int* __restrict__ n_rows,
                                                              int64_t n_max, PartView diag) {
    static_assert(L == 8, "a row is shared by 8 lanes");
    __shared__ TermTile<W> tile;
    const int64_t n = n_rows ? (int64_t)*n_rows : n_max;
    const int64_t first = (int64_t)blockIdx.x * (kThreads / L);
    if (first >= n) return;  // the whole block is past the last row
    const int sub = threadIdx.x % L;
    const int64_t row = first + threadIdx.x / L;
    const bool live = row < n;
    Key<W> c;
    if (live) {
        c = src.get(row);
    } else {
#pragma unroll
        for (int q = 0; q < W; ++q) c.w[q] = 0;
    }
    typename V::Acc acc;
    v.init(acc, row, c, nullptr);
    for (int64_t t0 = 0; t0 < diag.n; t0 += kTermTile) {
        const int count = (int)(diag.n - t0 < kTermTile ? diag.n - t0 : kTermTile);
        __syncthreads();
        stage_tile<W>(tile, diag, t0, count);
        __syncthreads();
        if (!live) continue;
        for (int k = sub; k < count; k += L) {
            if (term_applies<W>(tile.m[k], c)) {
                Key<W> img;
                v.visit_diag(acc, c, term_image<W>(tile.m[k], c, img), t0 + k);
            }
        }
    }
    v.template reduce_lanes<L>(acc);
    if (live && sub == 0) v.finish(acc, row, c);
}

// Lanes a row of a tiled diagonal pass is shared by: 8 below 40,000 rows
// (C2's 20,000-row pass 40 -> 27 us on GB300), else 1 (the plain tiled
// kernel; at 65,536 rows four lanes a row were slower, 125 -> 163 us).
inline int diag_lanes(int64_t n_rows) { return n_rows < 40000 ? 8 : 1; }

// ---------------------------------------------------------------------------
// the grouped enumeration kernel: one warp per row, visiting only the pivot
// groups whose sites the row occupies (see format.h).  Large groups are
// walked with the lanes over their terms (coalesced term loads); small ones
// with the lanes over groups.  Visitors additionally provide
// reduce(Acc&) (warp-wide, every lane ends with the total) and finish() is
// called by lane 0.  Rows are taken grid-stride, so the grid can be sized to
// the machine.
// ---------------------------------------------------------------------------

constexpr int kWarpsPerBlock = kThreads / 32;

// Parts with at least this many terms are walked by grouped_kernel.
constexpr int64_t kGroupedMinTerms = 2048;

// One term record in registers (loaded with 16-byte vector loads).
template <int W>
struct TermRec {
    uint64_t m[4 * W];
    __device__ __forceinline__ bool applies(const Key<W>& c) const {
        uint64_t bad = 0;
#pragma unroll
        for (int q = 0; q < W; ++q) bad |= (c.w[q] ^ m[4 * q + 1]) & m[4 * q];
        return bad == 0;
    }
    __device__ __forceinline__ int image(const Key<W>& c, Key<W>& img) const {
        int par = 0;
#pragma unroll
        for (int q = 0; q < W; ++q) {
            img.w[q] = c.w[q] ^ m[4 * q + 2];
            par += __popcll(c.w[q] & m[4 * q + 3]);
        }
        return par & 1;
    }
};

// The test pair of every word of term t (into m[4q], m[4q + 1]).
template <int W>
__device__ __forceinline__ void load_test(TermRec<W>& r, const PartView& pv, int64_t t) {
#pragma unroll
    for (int q = 0; q < W; ++q) {
        const ulonglong2 v = __ldg(pv.test + (int64_t)q * pv.stride + t);
        r.m[4 * q] = v.x;
        r.m[4 * q + 1] = v.y;
    }
}

// The apply pair of every word of term t (into m[4q + 2], m[4q + 3]).
template <int W>
__device__ __forceinline__ void load_apply(TermRec<W>& r, const PartView& pv, int64_t t) {
#pragma unroll
    for (int q = 0; q < W; ++q) {
        const ulonglong2 v = __ldg(pv.apply + (int64_t)q * pv.stride + t);
        r.m[4 * q + 2] = v.x;
        r.m[4 * q + 3] = v.y;
    }
}

// The whole record of term t from its narrow form (one 16-byte load; the
// part must have one: W == 1 and pv.narrow set).
template <int W>
__device__ __forceinline__ void load_narrow(TermRec<W>& r, const PartView& pv, int64_t t) {
    const uint4 q = __ldg(pv.narrow + t);
    r.m[0] = (uint64_t)q.x << 32;
    r.m[1] = (uint64_t)q.y << 32;
    r.m[2] = (uint64_t)q.z << 32;
    r.m[3] = (uint64_t)q.w << 32;
}

// Hits of batched visitors wait in a per-warp shared queue until 32 have
// gathered, then every lane processes one: the floating-point work of a hit
// (FP64 on GB300 issues at a small fraction of the FP32 rate) then runs with
// all lanes active instead of once per divergent warp iteration.
// Candidates of a batched walk wait in a per-warp ring: fewer than 32 wait
// between steps, and a step adds at most 32 per term a lane takes (two, or
// kNarrowTerms in the narrow walk of one-word keys).
constexpr int kNarrowTerms = 4;
__host__ __device__ constexpr int cand_ring(int W) { return W == 1 ? (kNarrowTerms > 2 ? 256 : 128) : 128; }

struct HitQueue {
    int2* q;         // 64 entries: (slot | parity << 31, looked-up row)
    int count;       // warp-uniform
    uint64_t* ckey;  // ring of cand_ring(W) candidate images (W words each) waiting for their lookup
    int* cmeta;      // slot | parity << 31 of each candidate
    int ccount;      // warp-uniform: candidates waiting
    int chead;       // warp-uniform: ring position of the oldest waiting candidate
};

template <class V>
__device__ __forceinline__ void queue_drain(const V& v, typename V::Acc& acc, HitQueue& hq, int lane, bool all) {
    v.record_hits(acc, hq.q, all ? hq.count : 32, lane);
    if (all) {
        if (lane < hq.count) v.apply_hit(acc, hq.q[lane]);
        __syncwarp();
        hq.count = 0;
        return;
    }
    v.apply_hit(acc, hq.q[lane]);
    __syncwarp();
    if (lane < hq.count - 32) hq.q[lane] = hq.q[32 + lane];
    __syncwarp();
    hq.count -= 32;
}

template <class V>
__device__ __forceinline__ void queue_push(const V& v, typename V::Acc& acc, HitQueue& hq, int lane, bool hit,
                                           int2 h) {
    const unsigned m = __ballot_sync(0xffffffffu, hit);
    if (m == 0) return;
    if (hit) hq.q[hq.count + __popc(m & ((1u << lane) - 1u))] = h;
    hq.count += __popc(m);
    __syncwarp();
    if (hq.count >= 32) queue_drain(v, acc, hq, lane, false);
}

// Test term t against c; on success either visit it directly or, for a
// batched visitor, probe it and report a hit to queue.
template <int W, bool DIAG, class V>
__device__ __forceinline__ bool test_term(const V& v, typename V::Acc& acc, const Key<W>& c, const PartView& pv,
                                          int64_t t, int2& h) {
    TermRec<W> r;
    bool narrow = false;
    if constexpr (W == 1) narrow = pv.narrow != nullptr;
    if (narrow) {
        load_narrow<W>(r, pv, t);
        if (!r.applies(c)) return false;
    } else {
        load_test<W>(r, pv, t);
        if (!r.applies(c)) return false;
        load_apply<W>(r, pv, t);
    }
    Key<W> img;
    const int par = r.image(c, img);
    if (DIAG) {
        v.visit_diag(acc, c, par, t);
        return false;
    } else if constexpr (V::kBatched) {
        return v.probe(acc, c, img, par, t, h);
    } else {
        v.visit(acc, c, img, par, t);
        return false;
    }
}

// Look up the n (<= 32) oldest queued candidates, one per lane, and queue
// the hits.  The candidates sit in a ring: the flush only advances its head,
// and the __syncwarp orders its reads before the appends that reuse the
// entries.
template <int W, class V>
__device__ __forceinline__ void candidates_flush(const V& v, typename V::Acc& acc, HitQueue& hq, int lane, int n) {
    int2 h = make_int2(0, 0);
    bool hit = false;
    if (lane < n) {
        const int at = (hq.chead + lane) & (cand_ring(W) - 1);
        Key<W> img;  // plain loads: the candidate queue is in shared memory
#pragma unroll
        for (int q = 0; q < W; ++q) img.w[q] = hq.ckey[at * W + q];
        const int64_t pos = hash_find<W>(v.lookup, img);
        if (pos >= 0) {
            hit = true;
            h = make_int2(hq.cmeta[at], (int)pos);
        }
    }
    __syncwarp();
    hq.chead = (hq.chead + n) & (cand_ring(W) - 1);
    hq.ccount -= n;
    queue_push(v, acc, hq, lane, hit, h);
}

// walk_group_lanes of a batched visitor over narrow records (one-word keys,
// every mask in the high half): one 16-byte load a term and 32-bit tests
// against the row's high half; the images are formed in the full word.
template <class V>
__device__ __forceinline__ void walk_group_narrow(const V& v, typename V::Acc& acc, const Key<1>& c,
                                                  const PartView& pv, int2 se, int lane, HitQueue& hq) {
    constexpr int K = kNarrowTerms;
    constexpr int kRing = cand_ring(1);
    const unsigned lt = (1u << lane) - 1u;
    const uint32_t hi = (uint32_t)(c.w[0] >> 32);
    for (int base = se.x; base < se.y; base += 32 * K) {
        // K terms a lane, all records loaded before any is tested
        uint4 q[K];
        bool app[K];
        unsigned m[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int t = base + 32 * k + lane;
            q[k] = make_uint4(0u, 0u, 0u, 0u);
            if (t < se.y) q[k] = __ldg(pv.narrow + t);
        }
        unsigned any = 0;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            app[k] = base + 32 * k + lane < se.y && ((hi ^ q[k].y) & q[k].x) == 0u;
            m[k] = __ballot_sync(0xffffffffu, app[k]);
            any |= m[k];
        }
        if (any == 0) continue;
        // every lane's terms appended in one step, term k of all lanes after term k - 1
        int at0 = hq.chead + hq.ccount;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            if (app[k]) {
                const int at = (at0 + __popc(m[k] & lt)) & (kRing - 1);
                hq.ckey[at] = c.w[0] ^ ((uint64_t)q[k].z << 32);
                hq.cmeta[at] = (base + 32 * k + lane) | ((__popc(hi & q[k].w) & 1) << 31);
            }
            at0 += __popc(m[k]);
        }
        hq.ccount = at0 - hq.chead;
        __syncwarp();
        while (hq.ccount >= 32) candidates_flush<1>(v, acc, hq, lane, 32);
    }
}

// Walk one group: lanes over its terms (warp-uniform bounds, so work can be
// queued).  For batched visitors the applicable terms are first compacted
// into the candidate queue, so that their lookups run with all lanes busy.
template <int W, bool DIAG, class V>
__device__ __forceinline__ void walk_group_lanes(const V& v, typename V::Acc& acc, const Key<W>& c,
                                                 const PartView& pv, int64_t g, int lane, HitQueue& hq) {
    const int2 se = __ldg(pv.groups + g);
    if constexpr (V::kBatched && !DIAG && W == 1) {
        if (pv.narrow != nullptr) {
            walk_group_narrow(v, acc, c, pv, se, lane, hq);
            return;
        }
    }
    if constexpr (V::kBatched && !DIAG) {
        const unsigned lt = (1u << lane) - 1u;
        // two terms per lane per step: both records are loaded before either is tested
        for (int base = se.x; base < se.y; base += 64) {
            const int t0 = base + lane, t1 = base + 32 + lane;
            TermRec<W> r0, r1;
            const bool in0 = t0 < se.y, in1 = t1 < se.y;
            if (in0) load_test<W>(r0, pv, t0);
            if (in1) load_test<W>(r1, pv, t1);
            // the apply pairs are loaded with the test pairs (not after the
            // test), so that no load waits on the test's result
            if (in0) load_apply<W>(r0, pv, t0);
            if (in1) load_apply<W>(r1, pv, t1);
            const bool app0 = in0 && r0.applies(c);
            const bool app1 = in1 && r1.applies(c);
            const unsigned m0 = __ballot_sync(0xffffffffu, app0);
            const unsigned m1 = __ballot_sync(0xffffffffu, app1);
            if ((m0 | m1) == 0) continue;
            // both terms of every lane appended in one step: the first terms, then the second
            const int tail = hq.chead + hq.ccount, n0 = __popc(m0);
#pragma unroll
            for (int half = 0; half < 2; ++half) {
                const bool app = half ? app1 : app0;
                if (app) {
                    const TermRec<W>& rec = half ? r1 : r0;
                    Key<W> img;
                    const int par = rec.image(c, img);
                    const int at = (tail + (half ? n0 + __popc(m1 & lt) : __popc(m0 & lt))) & (cand_ring(W) - 1);
#pragma unroll
                    for (int q = 0; q < W; ++q) hq.ckey[at * W + q] = img.w[q];
                    hq.cmeta[at] = (half ? t1 : t0) | (par << 31);
                }
            }
            hq.ccount += n0 + __popc(m1);
            __syncwarp();
            while (hq.ccount >= 32) candidates_flush<W>(v, acc, hq, lane, 32);
        }
    } else {
        for (int64_t base = se.x; base < se.y; base += 32) {
            const int64_t t = base + lane;
            int2 h = make_int2(0, 0);
            bool hit = false;
            if (t < se.y) hit = test_term<W, DIAG>(v, acc, c, pv, t, h);
            if constexpr (V::kBatched && !DIAG) queue_push(v, acc, hq, lane, hit, h);
        }
    }
}

// Walk one group entirely in this lane (hits processed at once).
template <int W, bool DIAG, class V>
__device__ __forceinline__ void walk_group_serial(const V& v, typename V::Acc& acc, const Key<W>& c,
                                                  const PartView& pv, int64_t g) {
    const int2 se = __ldg(pv.groups + g);
    for (int64_t t = se.x; t < se.y; ++t) {
        int2 h;
        if (test_term<W, DIAG>(v, acc, c, pv, t, h)) {
            v.record_hit(acc, h);
            v.apply_hit(acc, h);
        }
    }
}

// The pivot groups a row can reach, in a fixed order: group 0, the single
// groups of its occupied positions, then for every occupied position p the
// pair groups (p, q) with q occupied.  Warp-uniform state; next() yields one
// group id at a time so the walk has a single call site (small code, few
// registers).
// Word i of a W-word array, selected without indexing the array by a
// runtime value (which would put it in local memory).
template <int W>
__device__ __forceinline__ uint64_t pick_word(const uint64_t (&a)[W], int i) {
    uint64_t r = a[0];
#pragma unroll
    for (int q = 1; q < W; ++q) r = (q == i) ? a[q] : r;
    return r;
}

template <int W>
struct GroupCursor {
    int first;        // -2: group 0 pending; -1: single level; >= 0: pair level with this first position
    int word;         // word of the partner mask being drained
    uint64_t bits;    // partner bits still to yield in `word`
    uint64_t occ[W];  // occupied positions not yet used as `first`

    __device__ __forceinline__ void start(const Key<W>& row) {
        first = -2;
        word = 0;
        bits = 0;
#pragma unroll
        for (int q = 0; q < W; ++q) occ[q] = row.w[q];
    }
    __device__ __forceinline__ uint64_t partners(const Key<W>& row, const PartView& pv, int r) const {
        return pick_word<W>(row.w, r) &
               (first < 0 ? __ldg(pv.single_ne + r) : __ldg(pv.pair_ne + (int64_t)first * W + r));
    }
    __device__ __forceinline__ bool next(int64_t& g, const Key<W>& row, const PartView& pv) {
        if (first == -2) {
            first = -1;
            word = 0;
            bits = partners(row, pv, 0);
            g = 0;
            return true;
        }
#pragma unroll 1
        for (;;) {
            if (bits) {
                const int b = __ffsll((long long)bits) - 1;
                bits &= bits - 1;
                const int kp = 64 * word + b;
                g = first < 0 ? qmbx_single_group(kp) : qmbx_pair_group(W, first, kp);
                return true;
            }
            if (word + 1 < W) {
                ++word;
                bits = partners(row, pv, word);
                continue;
            }
            // next first position (pair level): the lowest occupied position left
            int q = W;
#pragma unroll
            for (int k = W - 1; k >= 0; --k) q = occ[k] ? k : q;
            if (q == W) return false;
            const uint64_t w = pick_word<W>(occ, q);
#pragma unroll
            for (int k = 0; k < W; ++k) occ[k] = (k == q) ? occ[k] & (occ[k] - 1) : occ[k];
            first = 64 * q + (__ffsll((long long)w) - 1);
            word = q;  // partners sit at higher positions
            bits = partners(row, pv, word);
        }
    }
};

// Walk the groups of part pv that row c reaches; with split > 1, only every
// split-th of them, starting at the part-th (a row shared by split warps).
template <int W, bool DIAG, class V>
__device__ __forceinline__ void walk_part(const V& v, typename V::Acc& acc, const Key<W>& c, const PartView& pv,
                                          int lane, HitQueue& hq, int part = 0, int split = 1) {
    if (pv.n == 0) return;
    GroupCursor<W> cur;
    cur.start(c);
    int64_t g;
    int seq = 0;  // groups yielded so far (split walks)
    if (pv.wide) {
#pragma unroll 1
        while (cur.next(g, c, pv)) {
            if (split > 1 && (seq++ % split) != part) continue;
            walk_group_lanes<W, DIAG>(v, acc, c, pv, g, lane, hq);
        }
    } else {
        // small groups: the cursor deals 32 groups to the lanes, one each,
        // then every lane walks its group (all 32 at once)
        int k = 0;
        int64_t mine = -1;
#pragma unroll 1
        while (cur.next(g, c, pv)) {
            if (split > 1 && (seq++ % split) != part) continue;
            if (k == lane) mine = g;
            if (++k == 32) {
                walk_group_serial<W, DIAG>(v, acc, c, pv, mine);
                __syncwarp();
                mine = -1;
                k = 0;
            }
        }
        if (mine >= 0) walk_group_serial<W, DIAG>(v, acc, c, pv, mine);
        __syncwarp();
    }
}

template <int W, class V, class Src>
__global__ void __launch_bounds__(kThreads) grouped_kernel(V v, Src src, const int* __restrict__ n_rows,
                                                           int64_t n_max, PartView off, PartView diag) {
    __shared__ int sh[V::kShared > 0 ? V::kShared : 1];
    __shared__ int2 hitq[kWarpsPerBlock][64];
    __shared__ uint64_t candkey[V::kBatched ? kWarpsPerBlock : 1][cand_ring(W) * W];
    __shared__ int candmeta[V::kBatched ? kWarpsPerBlock : 1][cand_ring(W)];
    v.block_init(sh);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int64_t n = n_rows ? (int64_t)*n_rows : n_max;
    const int64_t stride = (int64_t)gridDim.x * kWarpsPerBlock;
    for (int64_t row = (int64_t)blockIdx.x * kWarpsPerBlock + warp; row < n; row += stride) {
        const Key<W> c = src.get(row);
        typename V::Acc acc;
        v.init(acc, row, c, sh);
        HitQueue hq{hitq[warp], 0, candkey[V::kBatched ? warp : 0], candmeta[V::kBatched ? warp : 0], 0, 0};
        walk_part<W, false>(v, acc, c, off, lane, hq);
        if constexpr (V::kBatched) {
            if (hq.ccount > 0) candidates_flush<W>(v, acc, hq, lane, hq.ccount);
            queue_drain(v, acc, hq, lane, true);
        }
        walk_part<W, true>(v, acc, c, diag, lane, hq);
        v.reduce(acc);
        if (lane == 0) v.finish(acc, row, c);
    }
    __syncthreads();
    v.block_flush(sh);
}

// The grouped walk with each row's groups shared by `split` warps (warp
// item u walks row u / split, every split-th group from the (u % split)-th):
// for visitors whose per-row work adds up across parts of a row (the
// find_relative passes), when there are too few rows to fill the GPU with
// one warp each.  Each part gets its own init / reduce / finish.
template <int W, class V, class Src>
__global__ void __launch_bounds__(kThreads) grouped_split_kernel(V v, Src src, int64_t n, int split, PartView off,
                                                                 PartView diag) {
    __shared__ int sh[V::kShared > 0 ? V::kShared : 1];
    __shared__ int2 hitq[kWarpsPerBlock][64];
    static_assert(!V::kBatched, "split walks serve visitors that handle each term in place");
    v.block_init(sh);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int64_t items = n * split;
    const int64_t stride = (int64_t)gridDim.x * kWarpsPerBlock;
    for (int64_t u = (int64_t)blockIdx.x * kWarpsPerBlock + warp; u < items; u += stride) {
        const int64_t row = u / split;
        const int part = (int)(u - row * split);
        const Key<W> c = src.get(row);
        typename V::Acc acc;
        v.init(acc, row, c, sh);
        HitQueue hq{hitq[warp], 0, nullptr, nullptr, 0, 0};
        walk_part<W, false>(v, acc, c, off, lane, hq, part, split);
        walk_part<W, true>(v, acc, c, diag, lane, hq, part, split);
        v.reduce(acc);
        if (lane == 0) v.finish(acc, row, c);
    }
    __syncthreads();
    v.block_flush(sh);
}

// ---------------------------------------------------------------------------
// the pivot-major enumeration kernel.  A work item is one non-empty pivot
// group and a chunk of kPivotRows rows: the block scans the chunk for the
// rows that occupy the group's pivot positions, stages the group's terms in
// shared memory (slice by slice when they do not fit) and walks them for
// every matching row, one warp per row with lanes over terms.  Term data is
// read once per item from L2 and then from shared memory; only the lookups
// of images go to L2.  Each (row, group) result is handed to v.flush().
// ---------------------------------------------------------------------------

constexpr int kPivotTermBytes = 32768;
constexpr int kPivotRows = 2048;

template <int W>
__device__ __forceinline__ bool has_position(const Key<W>& c, int kp) {
    if (kp < 0) return true;
    uint64_t w = 0;
#pragma unroll
    for (int q = 0; q < W; ++q) w = (q == (kp >> 6)) ? c.w[q] : w;
    return (w >> (kp & 63)) & 1ull;
}

template <int W, class V, class Src>
__global__ void __launch_bounds__(kThreads) pivot_kernel(V v, Src src, const int* __restrict__ n_rows, int64_t n_max,
                                                         PartView pv) {
    // the visitor's own shared memory comes out of the term staging area, so
    // the block stays within the 48 KB of static shared memory
    constexpr int kTerms = (kPivotTermBytes - 4 * V::kShared) / (32 * W);
    // word-major like the table: pair 2q + 0 (mask, val) and 2q + 1 (flip,
    // par) of word q for term k at [2q + j][k], so that lanes reading
    // consecutive terms read consecutive 16-byte pairs (no bank conflicts)
    __shared__ ulonglong2 s_terms[2 * W][kTerms];
    __shared__ int32_t s_rows[kPivotRows];
    __shared__ int s_nrows;
    __shared__ int4 hitq[kWarpsPerBlock][64];
    __shared__ int sh[V::kShared > 0 ? V::kShared : 1];
    v.block_init(sh);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    int4* hq = hitq[warp];
    int hcount = 0;  // warp-uniform; the queue lives across rows and items
    const int64_t n = n_rows ? (int64_t)*n_rows : n_max;
    const int64_t chunks = (n + kPivotRows - 1) / kPivotRows;
    const int64_t items = pv.n_nonempty * chunks;
    for (int64_t item = blockIdx.x; item < items; item += gridDim.x) {
        const int64_t gi = item / chunks;
        const int64_t r0 = (item - gi * chunks) * kPivotRows;
        const int64_t r1 = r0 + kPivotRows < n ? r0 + kPivotRows : n;
        const int4 grp = __ldg(pv.nonempty + gi);
        if (threadIdx.x == 0) s_nrows = 0;
        __syncthreads();
        // rows of the chunk that occupy the pivot positions
        for (int64_t base = r0; base < r1; base += kThreads) {
            const int64_t r = base + threadIdx.x;
            bool m = false;
            if (r < r1) {
                const Key<W> c = src.get(r);
                m = has_position<W>(c, grp.z) && has_position<W>(c, grp.w);
            }
            const unsigned bal = __ballot_sync(0xffffffffu, m);
            int at = 0;
            if (lane == 0 && bal) at = atomicAdd(&s_nrows, __popc(bal));
            at = __shfl_sync(0xffffffffu, at, 0);
            if (m) s_rows[at + __popc(bal & lt)] = (int32_t)(r - r0);
        }
        __syncthreads();
        const int nrows = s_nrows;
        if (nrows > 0) {
            for (int ts = grp.x; ts < grp.y; ts += kTerms) {
                const int cnt = grp.y - ts < kTerms ? grp.y - ts : kTerms;
                __syncthreads();
#pragma unroll
                for (int q = 0; q < W; ++q) {
                    const ulonglong2* test = pv.test + (int64_t)q * pv.stride + ts;
                    const ulonglong2* apply = pv.apply + (int64_t)q * pv.stride + ts;
                    for (int k = threadIdx.x; k < cnt; k += kThreads) {
                        s_terms[2 * q][k] = __ldg(test + k);
                        s_terms[2 * q + 1][k] = __ldg(apply + k);
                    }
                }
                __syncthreads();
                for (int i = warp; i < nrows; i += kWarpsPerBlock) {
                    const int64_t u = r0 + s_rows[i];
                    const Key<W> c = src.get(u);
                    typename V::Acc acc;
                    if constexpr (!V::kStateless) v.init(acc, u, c, sh);
                    for (int b = 0; b < cnt; b += 32) {
                        const int k = b + lane;
                        int4 h = make_int4(0, 0, 0, 0);
                        bool hit = false;
                        if (k < cnt) {
                            TermRec<W> rec;
#pragma unroll
                            for (int q = 0; q < 2 * W; ++q) {
                                const ulonglong2 x = s_terms[q][k];
                                rec.m[2 * q] = x.x;
                                rec.m[2 * q + 1] = x.y;
                            }
                            if (rec.applies(c)) {
                                Key<W> img;
                                const int par = rec.image(c, img);
                                if constexpr (V::kStateless) {
                                    hit = v.probe_row(c, img, par, ts + k, u, h);
                                } else {
                                    v.visit(acc, c, img, par, ts + k);
                                }
                            }
                        }
                        if constexpr (V::kStateless) {
                            // queue the hit; 32 queued hits are applied with all lanes
                            const unsigned m = __ballot_sync(0xffffffffu, hit);
                            if (m) {
                                if (hit) hq[hcount + __popc(m & lt)] = h;
                                hcount += __popc(m);
                                __syncwarp();
                                if (hcount >= 32) {
                                    v.record_row_hits(hq, 32, lane);
                                    v.apply_row_hit(hq[lane]);
                                    __syncwarp();
                                    if (lane < hcount - 32) hq[lane] = hq[32 + lane];
                                    __syncwarp();
                                    hcount -= 32;
                                }
                            }
                        }
                    }
                    if constexpr (!V::kStateless) {
                        v.reduce(acc);
                        if (lane == 0) v.flush(acc, u, c);
                    }
                }
            }
        }
        __syncthreads();
    }
    if constexpr (V::kStateless) {
        v.record_row_hits(hq, hcount, lane);
        if (lane < hcount) v.apply_row_hit(hq[lane]);
    }
    __syncthreads();
    v.block_flush(sh);
}

// Grid for pivot_kernel: a few resident blocks per SM, looping over work items.
int pivot_grid();

// Warps a row's groups are shared by in grouped_split_kernel: enough for
// about two waves of warps over n_rows rows, at most 16 (1 when the rows
// fill the GPU alone).
int row_split(int64_t n_rows);

// Which kernel walks a term part over n_rows rows:
//   pivot    parts of kGroupedMinTerms terms or more whose non-empty groups
//            hold kPivotMeanGroup terms or more on average (when the caller
//            has a pivot-major visitor);
//   grouped  other parts of kGroupedMinTerms terms or more, and smaller parts
//            over fewer than kFewRows rows (kFewWideRows when the part's
//            groups are large), where a thread per row would leave most of
//            the GPU idle;
//   tiled    small parts over more rows (e.g. the diagonal parts, whose
//            groups hold one term or two, over 20,000 rows), and parts of up
//            to kTiledMaxTerms terms in groups of a few terms over
//            kFewWideRows rows or more.
// QMBX_WALK=pivot, grouped or tiled in the environment forces a kernel
// (read at every call; pivot falls back to grouped where it cannot serve).
constexpr int kPivotMeanGroup = 300;
constexpr int64_t kFewRows = 8192;
constexpr int64_t kFewWideRows = 65536;
constexpr int64_t kTiledMaxTerms = 8192;
enum class Walk { kTiled, kGrouped, kPivot };
Walk choose_walk(const PartView& part, int64_t n_rows, bool pivot_ok);

// QMBX_DETERMINISTIC=1 in the environment (read at every call): apply_within
// and its adjoint take only walks whose sums have a fixed order (the gather
// direction, no pivot-major walk), so that repeated calls give identical
// bits.  The scatter and pivot walks add into their outputs with FP64
// atomics, whose order varies from run to run.
bool deterministic_mode();

// Grid for grouped_kernel: enough warps for every row, at most a few waves.
int grouped_grid(int64_t n_rows);

// Lane-sum of a double across the warp (butterfly: every lane gets the total).
__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) x += __shfl_xor_sync(0xffffffffu, x, d);
    return x;
}

// ---------------------------------------------------------------------------
// key utilities implemented in keys.cu (explicitly instantiated for W = 1..4)
// ---------------------------------------------------------------------------

// rows (n x n_qubytes bytes, any alignment) -> keys (n x W words)
template <int W>
int pack_rows(const uint8_t* rows, int64_t n, int n_qubytes, uint64_t* keys, cudaStream_t s);

// keys -> rows; rows beyond *n_rows (when n_rows != NULL) are left untouched
template <int W>
int unpack_rows(const uint64_t* keys, const int* n_rows, int64_t n_max, int n_qubytes, uint8_t* rows,
                cudaStream_t s);

// Scratch of one radix sort of up to n keys.
struct SortScratch {
    uint64_t* keys;
    int32_t* vals;
    int32_t* counts;
    int32_t* scan;
};

template <int W>
SortScratch take_sort_scratch(Arena& ws, int64_t n);

// Stable LSD radix sort of (key, value) pairs in lexicographic key order over
// the first n_bytes row bytes (n_bytes passes of 8 bits).  vals_in == NULL
// sorts the identity permutation.  keys_out/vals_out must not alias the inputs.
template <int W>
int sort_pairs(const uint64_t* keys_in, const int32_t* vals_in, uint64_t* keys_out, int32_t* vals_out, int64_t n,
               int n_bytes, const SortScratch& sc, cudaStream_t s);

// A sorted, de-duplicated row set (all buffers carved by take_rowset).
struct RowSet {
    uint64_t* packed;       // n x W: keys in input row order
    uint64_t* sorted_keys;  // n x W, sorted (with repeats)
    int32_t* perm;          // n: original row of each sorted position
    uint64_t* keys;         // n x W: unique keys (first *count valid)
    int32_t* first;         // n: original row of the first occurrence of each unique key
    int32_t* start;         // n + 1: sorted position where each unique key's run starts
    int* count;             // device int: number of unique keys
    int32_t* head;
    int32_t* pos;
    uint64_t* slots;        // hash set over the unique keys
    uint64_t slot_mask;
    SortScratch sort;
    int64_t n;
    HashView hash() const {
        return HashView{reinterpret_cast<const uint32_t*>(slots), keys, slot_mask, hash_shift(slot_mask + 1), nullptr, 0};
    }
};

template <int W>
RowSet take_rowset(Arena& ws, int64_t n);

template <int W>
int build_rowset(const uint8_t* rows, int n_qubytes, RowSet& out, cudaStream_t s);

// Sort out.n keys by their first n_bytes row bytes and keep the distinct ones
// (out.keys[0 .. *out.count)); builds no hash set.
template <int W>
int sort_unique_keys(const uint64_t* keys, int n_bytes, RowSet& out, cudaStream_t s);

// A de-duplicated row set without sorting: every row's key is inserted in an
// open-addressing hash set whose entries name the first (lowest) row holding
// that key.  first[i] is that row for every row i; unique[0 .. *count) lists
// the first rows (in no particular order: the walks treat rows
// independently).  Lookups (hash()) return first rows, so per-key data is
// stored at the first row's index.
struct HashRows {
    uint64_t* keys;     // n x W, row order
    uint64_t* slots;
    uint64_t slot_mask;
    int32_t* first;     // n
    int32_t* unique;    // n (first *count valid, in no particular order)
    int* count;
    uint32_t* bloom;    // filter over the keys (bloom_words_for(n) words), or NULL
    uint32_t bloom_words;
    int64_t n;
    HashView hash() const {
        return HashView{reinterpret_cast<const uint32_t*>(slots), keys, slot_mask, hash_shift(slot_mask + 1),
                        bloom_words ? bloom : nullptr, bloom_words ? bloom_words - 1 : 0};
    }
};

template <int W>
HashRows take_hashrows(Arena& ws, int64_t n);

template <int W>
int build_hashrows(const uint8_t* rows, int n_qubytes, HashRows& out, cudaStream_t s);

// Rows of a HashRows set visited by the enumeration kernels: walk index u
// is the u-th unique row.
template <int W>
struct UniqueRows {
    const uint64_t* keys;
    const int32_t* unique;
    __device__ __forceinline__ Key<W> get(int64_t u) const { return load_key<W>(keys, __ldg(unique + u)); }
};

// Exclusive prefix sum of n int32 values (in == out allowed); the total goes
// to *total when non-NULL.  scratch holds scan_scratch(n) int32 values.
int64_t scan_scratch(int64_t n);
int exclusive_scan(const int32_t* in, int32_t* out, int64_t n, int* total, int32_t* scratch, cudaStream_t s,
                   int group = kGroupKeys);

}  // namespace qmbx
