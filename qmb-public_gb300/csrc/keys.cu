// Key handling: packing rows into big-endian key words, prefix sums, a stable
// LSD radix sort, and sorted/de-duplicated row sets.
//
// The reference sorts rows with thrust and a byte-wise comparator
// (qmb/_hamiltonian_cuda.cu:245-251, :624-629, :956-961) and de-duplicates
// with torch::unique_dim (:666-674); this file does both with its own
// kernels on 64-bit key words.
#include <cuda_runtime.h>

#include <cstdlib>

#include "device.cuh"

namespace qmbx {

// ---------------------------------------------------------------------------
// pack / unpack
// ---------------------------------------------------------------------------

template <int W>
__global__ void pack_kernel(const uint8_t* __restrict__ rows, int64_t n, int nq, uint64_t* __restrict__ keys) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
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
        keys[i * W + q] = w;
    }
}

template <int W>
__global__ void unpack_kernel(const uint64_t* __restrict__ keys, const int* __restrict__ n_rows, int64_t n_max, int nq,
                              uint8_t* __restrict__ rows) {
    int64_t n = n_rows ? (int64_t)*n_rows : n_max;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint8_t* r = rows + i * nq;
    for (int b = 0; b < nq; ++b) {
        uint64_t w = keys[i * W + (b >> 3)];
        r[b] = (uint8_t)(w >> (8 * (7 - (b & 7))));
    }
}

template <int W>
int pack_rows(const uint8_t* rows, int64_t n, int nq, uint64_t* keys, cudaStream_t s) {
    if (n == 0) return QMBX_OK;
    QMBX_KERNEL(kGroupKeys, s, pack_kernel<W><<<grid_for(n, kThreads), kThreads, 0, s>>>(rows, n, nq, keys));
    QMBX_LAUNCH_CHECK("pack_kernel");
    return QMBX_OK;
}

template <int W>
int unpack_rows(const uint64_t* keys, const int* n_rows, int64_t n_max, int nq, uint8_t* rows, cudaStream_t s) {
    if (n_max == 0) return QMBX_OK;
    QMBX_KERNEL(kGroupKeys, s, unpack_kernel<W><<<grid_for(n_max, kThreads), kThreads, 0, s>>>(keys, n_rows, n_max, nq, rows));
    QMBX_LAUNCH_CHECK("unpack_kernel");
    return QMBX_OK;
}

// ---------------------------------------------------------------------------
// exclusive scan (reduce, scan of block sums, scan with offsets)
// ---------------------------------------------------------------------------

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 8;
constexpr int kScanChunk = kScanThreads * kScanItems;

__global__ void set_zero_kernel(int32_t* p) { *p = 0; }

__global__ void set_int_kernel(int* p, int v) { *p = v; }

__global__ void identity_kernel(const int32_t* __restrict__ in, int32_t* __restrict__ out, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = in ? in[i] : (int32_t)i;
}

__device__ __forceinline__ int32_t block_exclusive_scan(int32_t v, int32_t* s_warp, int32_t* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    int32_t x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        int32_t y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int32_t w = lane < nwarps ? s_warp[lane] : 0;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            int32_t y = __shfl_up_sync(0xffffffffu, w, d);
            if (lane >= d) w += y;
        }
        if (lane < nwarps) s_warp[lane] = w;
    }
    __syncthreads();
    int32_t before = warp > 0 ? s_warp[warp - 1] : 0;
    if (total) *total = s_warp[nwarps - 1];
    __syncthreads();
    return before + x - v;
}

__global__ void scan_reduce_kernel(const int32_t* __restrict__ in, int64_t n, int32_t* __restrict__ sums) {
    __shared__ int32_t s_warp[32];
    int64_t base = (int64_t)blockIdx.x * kScanChunk;
    int32_t acc = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        int64_t i = base + (int64_t)k * kScanThreads + threadIdx.x;
        if (i < n) acc += in[i];
    }
    int32_t total;
    block_exclusive_scan(acc, s_warp, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void scan_sums_kernel(int32_t* __restrict__ sums, int64_t nb, int* __restrict__ total_out) {
    __shared__ int32_t s_warp[32];
    // each thread scans a contiguous run of per-block sums
    int64_t per = (nb + blockDim.x - 1) / blockDim.x;
    int64_t lo = (int64_t)threadIdx.x * per;
    int64_t hi = lo + per < nb ? lo + per : nb;
    int32_t local = 0;
    for (int64_t i = lo; i < hi; ++i) local += sums[i];
    int32_t total;
    int32_t before = block_exclusive_scan(local, s_warp, &total);
    for (int64_t i = lo; i < hi; ++i) {
        int32_t v = sums[i];
        sums[i] = before;
        before += v;
    }
    if (threadIdx.x == 0 && total_out) *total_out = total;
}

__global__ void scan_apply_kernel(const int32_t* __restrict__ in, int32_t* __restrict__ out, int64_t n,
                                  const int32_t* __restrict__ sums) {
    __shared__ int32_t s_warp[32];
    int64_t base = (int64_t)blockIdx.x * kScanChunk + (int64_t)threadIdx.x * kScanItems;
    int32_t v[kScanItems];
    int32_t local = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        int64_t i = base + k;
        v[k] = i < n ? in[i] : 0;
        local += v[k];
    }
    int32_t run = block_exclusive_scan(local, s_warp, nullptr) + sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        int64_t i = base + k;
        if (i < n) out[i] = run;
        run += v[k];
    }
}

// Exclusive scan of up to kScanChunk values in one block (one launch instead of three).
__global__ void scan_single_kernel(const int32_t* __restrict__ in, int32_t* __restrict__ out, int64_t n,
                                   int* __restrict__ total_out) {
    __shared__ int32_t s_warp[32];
    const int64_t base = (int64_t)threadIdx.x * kScanItems;
    int32_t v[kScanItems];
    int32_t local = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t i = base + k;
        v[k] = i < n ? in[i] : 0;
        local += v[k];
    }
    int32_t total;
    int32_t run = block_exclusive_scan(local, s_warp, &total);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t i = base + k;
        if (i < n) out[i] = run;
        run += v[k];
    }
    if (threadIdx.x == 0 && total_out) *total_out = total;
}

int64_t scan_scratch(int64_t n) {
    int64_t nb = (n + kScanChunk - 1) / kScanChunk;
    return nb < 1 ? 1 : nb;
}

int exclusive_scan(const int32_t* in, int32_t* out, int64_t n, int* total, int32_t* scratch, cudaStream_t s,
                   int group) {
    int64_t nb = scan_scratch(n);
    if (n > 0 && n <= kScanChunk) {
        QMBX_KERNEL(group, s, scan_single_kernel<<<1, kScanThreads, 0, s>>>(in, out, n, total));
        QMBX_LAUNCH_CHECK("exclusive_scan");
        return QMBX_OK;
    }
    if (n > 0) QMBX_KERNEL(group, s, scan_reduce_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, scratch));
    else QMBX_KERNEL(group, s, set_zero_kernel<<<1, 1, 0, s>>>(scratch));
    QMBX_KERNEL(group, s, scan_sums_kernel<<<1, kScanThreads, 0, s>>>(scratch, nb, total));
    if (n > 0) QMBX_KERNEL(group, s, scan_apply_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(in, out, n, scratch));
    QMBX_LAUNCH_CHECK("exclusive_scan");
    return QMBX_OK;
}

// ---------------------------------------------------------------------------
// stable LSD radix sort, 8-bit digits
// ---------------------------------------------------------------------------

constexpr int kSortWarps = 8;
constexpr int kSortThreads = kSortWarps * 32;
// items per lane: 16 for large sorts; 8 up to kSortSmall items, so that a
// sort of a few tens of thousands of rows (find_relative's output) spreads
// over twice the blocks while its per-block digit counts still fit the
// one-block scan
constexpr int kSortRounds = 16;
constexpr int kSortRoundsSmall = 8;
constexpr int64_t kSortSmall = int64_t(1) << 20;

__host__ __device__ constexpr int sort_rounds(int64_t n) { return n <= kSortSmall ? kSortRoundsSmall : kSortRounds; }

template <int W>
__device__ __forceinline__ unsigned digit_of(const uint64_t* k, int word, int shift) {
    return (unsigned)(k[word] >> shift) & 0xffu;
}

// counts[d * nblocks + b] = items of block b with digit d (R items per lane)
template <int W, int R>
__global__ void __launch_bounds__(kSortThreads) radix_hist_kernel(const uint64_t* __restrict__ keys, int64_t n,
                                                                 int word, int shift, int32_t* __restrict__ counts,
                                                                 int nblocks) {
    __shared__ int32_t hist[256];
    for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[d] = 0;
    __syncthreads();
    int64_t base = (int64_t)blockIdx.x * kSortThreads * R;
    for (int k = 0; k < R; ++k) {
        int64_t i = base + (int64_t)k * kSortThreads + threadIdx.x;
        if (i < n) {
            unsigned d = (unsigned)(__ldg(keys + i * W + word) >> shift) & 0xffu;
            atomicAdd(&hist[d], 1);
        }
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += blockDim.x) counts[(int64_t)d * nblocks + blockIdx.x] = hist[d];
}

// Scatter with ranks that keep the input order among equal digits: warp w of
// a block owns items [w*32*R, (w+1)*32*R) of the block's tile, visited round
// by round (32 consecutive items per round).
template <int W, int R>
__global__ void __launch_bounds__(kSortThreads) radix_scatter_kernel(const uint64_t* __restrict__ keys_in,
                                                                    const int32_t* __restrict__ vals_in,
                                                                    uint64_t* __restrict__ keys_out,
                                                                    int32_t* __restrict__ vals_out, int64_t n,
                                                                    int word, int shift,
                                                                    const int32_t* __restrict__ offsets, int nblocks) {
    __shared__ int32_t s_cnt[kSortWarps][256];
    __shared__ int32_t s_base[256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int d = threadIdx.x; d < 256; d += blockDim.x) {
        for (int w = 0; w < kSortWarps; ++w) s_cnt[w][d] = 0;
        s_base[d] = offsets[(int64_t)d * nblocks + blockIdx.x];
    }
    __syncthreads();
    const int64_t wbase = (int64_t)blockIdx.x * kSortThreads * R + (int64_t)warp * 32 * R;
    unsigned dig[R];
    int32_t rank[R];
    const unsigned lt_mask = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        int64_t i = wbase + (int64_t)r * 32 + lane;
        bool valid = i < n;
        unsigned d = valid ? (unsigned)(__ldg(keys_in + i * W + word) >> shift) & 0xffu : 256u;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        int leader = __ffs(peers) - 1;
        int b = 0;
        if (lane == leader && valid) {
            b = s_cnt[warp][d];
            s_cnt[warp][d] = b + __popc(peers);
        }
        b = __shfl_sync(0xffffffffu, b, leader);
        dig[r] = d;
        rank[r] = b + __popc(peers & lt_mask);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += blockDim.x) {
        int32_t run = 0;
        for (int w = 0; w < kSortWarps; ++w) {
            int32_t c = s_cnt[w][d];
            s_cnt[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < R; ++r) {
        int64_t i = wbase + (int64_t)r * 32 + lane;
        if (i < n) {
            unsigned d = dig[r];
            int64_t dst = (int64_t)s_base[d] + s_cnt[warp][d] + rank[r];
#pragma unroll
            for (int q = 0; q < W; ++q) keys_out[dst * W + q] = keys_in[i * W + q];
            vals_out[dst] = vals_in ? vals_in[i] : (int32_t)i;
        }
    }
}

template <int W>
static int sort_blocks(int64_t n) {
    const int64_t tile = (int64_t)kSortThreads * sort_rounds(n);
    int64_t nb = (n + tile - 1) / tile;
    return (int)(nb < 1 ? 1 : nb);
}

template <int W>
SortScratch take_sort_scratch(Arena& ws, int64_t n) {
    SortScratch sc;
    int nblocks = sort_blocks<W>(n);
    uint64_t cap = (uint64_t)(n > 0 ? n : 1);
    sc.keys = ws.take<uint64_t>(cap * W);
    sc.vals = ws.take<int32_t>(cap);
    sc.counts = ws.take<int32_t>((uint64_t)256 * nblocks);
    sc.scan = ws.take<int32_t>((uint64_t)scan_scratch((int64_t)256 * nblocks));
    return sc;
}

template <int W>
int sort_pairs(const uint64_t* keys_in, const int32_t* vals_in, uint64_t* keys_out, int32_t* vals_out, int64_t n,
               int n_bytes, const SortScratch& sc, cudaStream_t s) {
    if (n == 0) return QMBX_OK;
    const int nblocks = sort_blocks<W>(n);
    if (n_bytes == 0) {
        QMBX_CUDA_TRY(cudaMemcpyAsync(keys_out, keys_in, n * W * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s));
        QMBX_KERNEL(kGroupKeys, s, identity_kernel<<<grid_for(n, kThreads), kThreads, 0, s>>>(vals_in, vals_out, n));
        QMBX_LAUNCH_CHECK("identity_kernel");
        return QMBX_OK;
    }
    const uint64_t* src_k = keys_in;
    const int32_t* src_v = vals_in;
    for (int p = 0; p < n_bytes; ++p) {
        int b = n_bytes - 1 - p;  // row byte handled by this pass, least significant first
        int word = b >> 3;
        int shift = 8 * (7 - (b & 7));
        bool to_out = ((n_bytes - 1 - p) & 1) == 0;
        uint64_t* dst_k = to_out ? keys_out : sc.keys;
        int32_t* dst_v = to_out ? vals_out : sc.vals;
        const bool small = sort_rounds(n) == kSortRoundsSmall;
        if (small) {
            QMBX_KERNEL(kGroupSort, s, radix_hist_kernel<W, kSortRoundsSmall><<<nblocks, kSortThreads, 0, s>>>(src_k, n, word, shift, sc.counts, nblocks));
        } else {
            QMBX_KERNEL(kGroupSort, s, radix_hist_kernel<W, kSortRounds><<<nblocks, kSortThreads, 0, s>>>(src_k, n, word, shift, sc.counts, nblocks));
        }
        int st = exclusive_scan(sc.counts, sc.counts, (int64_t)256 * nblocks, nullptr, sc.scan, s, kGroupSort);
        if (st != QMBX_OK) return st;
        if (small) {
            QMBX_KERNEL(kGroupSort, s, radix_scatter_kernel<W, kSortRoundsSmall><<<nblocks, kSortThreads, 0, s>>>(src_k, src_v, dst_k, dst_v, n, word, shift, sc.counts, nblocks));
        } else {
            QMBX_KERNEL(kGroupSort, s, radix_scatter_kernel<W, kSortRounds><<<nblocks, kSortThreads, 0, s>>>(src_k, src_v, dst_k, dst_v, n, word, shift, sc.counts, nblocks));
        }
        QMBX_LAUNCH_CHECK("radix sort pass");
        src_k = dst_k;
        src_v = dst_v;
    }
    return QMBX_OK;
}

// ---------------------------------------------------------------------------
// sorted, de-duplicated row sets
// ---------------------------------------------------------------------------

template <int W>
__global__ void head_flags_kernel(const uint64_t* __restrict__ sorted, int64_t n, int32_t* __restrict__ head) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int32_t h = 1;
    if (i > 0) {
        Key<W> a = load_key<W>(sorted, i - 1);
        Key<W> b = load_key<W>(sorted, i);
        h = key_eq<W>(a, b) ? 0 : 1;
    }
    head[i] = h;
}

template <int W>
__global__ void compact_heads_kernel(const uint64_t* __restrict__ sorted, const int32_t* __restrict__ perm,
                                     const int32_t* __restrict__ head, const int32_t* __restrict__ pos, int64_t n,
                                     uint64_t* __restrict__ ukeys, int32_t* __restrict__ first,
                                     int32_t* __restrict__ start, int* __restrict__ count) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (head[i]) {
        int32_t u = pos[i];
        store_key<W>(ukeys, u, load_key<W>(sorted, i));
        first[u] = perm[i];
        start[u] = (int32_t)i;
    }
    if (i == n - 1) {
        int32_t total = pos[i] + head[i];
        *count = total;
        start[total] = (int32_t)n;
    }
}



template <int W>
__global__ void hash_insert_kernel(const uint64_t* __restrict__ keys, const int* __restrict__ count,
                                   uint64_t* __restrict__ slots, uint64_t mask) {
    int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= *count) return;
    Key<W> k = load_key<W>(keys, u);
    uint64_t hv = key_hash<W>(k);
    uint64_t i = hash_home(hv, hash_shift(mask + 1));
    uint32_t* w = reinterpret_cast<uint32_t*>(slots);
    // the keys are unique and the table at most a quarter full, so an empty
    // slot is reached within mask + 1 probes; a slot is claimed on its row
    // word, then given its fingerprint
    for (uint64_t probe = 0; probe <= mask; ++probe) {
        if (atomicCAS(w + slot_row_word(i), kEmptyRow, (uint32_t)u) == kEmptyRow) {
            w[slot_tag_word(i)] = hash_tag(hv);
            return;
        }
        i = (i + 1) & mask;
    }
}

template <int W>
RowSet take_rowset(Arena& ws, int64_t n) {
    RowSet out;
    uint64_t cap = (uint64_t)(n > 0 ? n : 1);
    out.n = n;
    out.packed = ws.take<uint64_t>(cap * W);
    out.sorted_keys = ws.take<uint64_t>(cap * W);
    out.perm = ws.take<int32_t>(cap);
    out.keys = ws.take<uint64_t>(cap * W);
    out.first = ws.take<int32_t>(cap);
    out.start = ws.take<int32_t>(cap + 1);
    out.count = ws.take<int>(1);
    out.head = ws.take<int32_t>(cap);
    out.pos = ws.take<int32_t>(cap);
    uint64_t slots = 64;
    while (slots < 4 * cap) slots <<= 1;
    out.slots = ws.take<uint64_t>(slots);
    out.slot_mask = slots - 1;
    out.sort = take_sort_scratch<W>(ws, n);
    return out;
}

template <int W>
int build_rowset(const uint8_t* rows, int nq, RowSet& out, cudaStream_t s) {
    const int64_t n = out.n;
    if (n == 0) {
        QMBX_KERNEL(kGroupKeys, s, set_int_kernel<<<1, 1, 0, s>>>(out.count, 0));
        QMBX_CUDA_TRY(cudaMemsetAsync(out.slots, 0xff, (out.slot_mask + 1) * sizeof(uint64_t), s));
        QMBX_LAUNCH_CHECK("set_int_kernel");
        return QMBX_OK;
    }
    int st;
    if ((st = pack_rows<W>(rows, n, nq, out.packed, s)) != QMBX_OK) return st;
    if ((st = sort_pairs<W>(out.packed, nullptr, out.sorted_keys, out.perm, n, nq, out.sort, s)) != QMBX_OK) return st;
    QMBX_KERNEL(kGroupKeys, s, head_flags_kernel<W><<<grid_for(n, kThreads), kThreads, 0, s>>>(out.sorted_keys, n, out.head));
    if ((st = exclusive_scan(out.head, out.pos, n, nullptr, out.sort.scan, s)) != QMBX_OK) return st;
    QMBX_KERNEL(kGroupKeys, s, compact_heads_kernel<W><<<grid_for(n, kThreads), kThreads, 0, s>>>(out.sorted_keys, out.perm, out.head, out.pos, n,
                                                                       out.keys, out.first, out.start, out.count));
    QMBX_CUDA_TRY(cudaMemsetAsync(out.slots, 0xff, (out.slot_mask + 1) * sizeof(uint64_t), s));
    QMBX_KERNEL(kGroupKeys, s, hash_insert_kernel<W><<<grid_for(n, kThreads), kThreads, 0, s>>>(out.keys, out.count, out.slots, out.slot_mask));
    QMBX_LAUNCH_CHECK("build_rowset");
    return QMBX_OK;
}

// Sort out.n keys (W words, first n_bytes row bytes significant) and keep
// the distinct ones: out.keys[0 .. *out.count) in lexicographic order.  The
// keys are copied first, so `keys` may be any buffer; no hash set is built.
template <int W>
int sort_unique_keys(const uint64_t* keys, int n_bytes, RowSet& out, cudaStream_t s) {
    const int64_t n = out.n;
    if (n == 0) {
        QMBX_KERNEL(kGroupKeys, s, set_int_kernel<<<1, 1, 0, s>>>(out.count, 0));
        QMBX_LAUNCH_CHECK("set_int_kernel");
        return QMBX_OK;
    }
    int st;
    if ((st = sort_pairs<W>(keys, nullptr, out.sorted_keys, out.perm, n, n_bytes, out.sort, s)) != QMBX_OK) return st;
    QMBX_KERNEL(kGroupKeys, s, head_flags_kernel<W><<<grid_for(n, kThreads), kThreads, 0, s>>>(out.sorted_keys, n, out.head));
    if ((st = exclusive_scan(out.head, out.pos, n, nullptr, out.sort.scan, s)) != QMBX_OK) return st;
    QMBX_KERNEL(kGroupKeys, s, compact_heads_kernel<W><<<grid_for(n, kThreads), kThreads, 0, s>>>(out.sorted_keys, out.perm, out.head, out.pos, n,
                                                                       out.keys, out.first, out.start, out.count));
    QMBX_LAUNCH_CHECK("sort_unique_keys");
    return QMBX_OK;
}

// ---------------------------------------------------------------------------
// hash-based de-duplicated row sets
// ---------------------------------------------------------------------------

// Insert every row; a key already present keeps the lowest row.  A slot is
// claimed by a CAS on its row word and then given its fingerprint; a row
// that finds its key in a claimed slot (compared in full: the fingerprint
// may not be written yet) lowers that slot's row with atomicMin.  Every row
// of a key meets the same slot, the first claimed on the key's probe
// sequence.
template <int W>
__global__ void hashrows_insert_kernel(const uint64_t* __restrict__ keys, int64_t n, uint64_t* __restrict__ slots,
                                       uint64_t mask, uint32_t* __restrict__ bloom, uint32_t bloom_mask) {
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const Key<W> k = load_key<W>(keys, r);
    const uint64_t hv = key_hash<W>(k);
    if (bloom != nullptr) {
        const uint64_t f = bloom_mix(hv);
        atomicOr(bloom + bloom_word(f, bloom_mask), bloom_bits(f));
    }
    uint64_t i = hash_home(hv, hash_shift(mask + 1));
    uint32_t* w = reinterpret_cast<uint32_t*>(slots);
    for (uint64_t probe = 0; probe <= mask; ++probe) {
        uint32_t* row = w + slot_row_word(i);
        uint32_t cur = *(volatile uint32_t*)row;
        if (cur == kEmptyRow) {
            cur = atomicCAS(row, kEmptyRow, (uint32_t)r);
            if (cur == kEmptyRow) {
                w[slot_tag_word(i)] = hash_tag(hv);
                return;
            }
        }
        if (key_eq<W>(load_key<W>(keys, (int64_t)cur), k)) {
            atomicMin(row, (uint32_t)r);
            return;
        }
        i = (i + 1) & mask;
    }
}

// first[r] = lowest row with row r's key; every such first row is listed in
// unique[0 .. *count) (in no particular order: a warp reserves its places
// with one atomic).
template <int W>
__global__ void hashrows_resolve_kernel(const uint64_t* __restrict__ keys, int64_t n, HashView h,
                                        int32_t* __restrict__ first, int32_t* __restrict__ unique,
                                        int* __restrict__ count) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = r < n;
    int64_t f = -1;
    if (live) {
        f = hash_find<W>(h, load_key<W>(keys, r));
        first[r] = (int32_t)f;
    }
    const bool head = live && f == r;
    const unsigned m = __ballot_sync(0xffffffffu, head);
    const int lane = threadIdx.x & 31;
    int at = 0;
    if (lane == 0 && m) at = atomicAdd(count, __popc(m));
    at = __shfl_sync(0xffffffffu, at, 0);
    if (head) unique[at + __popc(m & ((1u << lane) - 1u))] = (int32_t)r;
}

template <int W>
HashRows take_hashrows(Arena& ws, int64_t n) {
    HashRows out;
    uint64_t cap = (uint64_t)(n > 0 ? n : 1);
    out.n = n;
    out.keys = ws.take<uint64_t>(cap * W);
    uint64_t slots = 64;
    while (slots < 4 * cap) slots <<= 1;
    out.slots = ws.take<uint64_t>(slots);
    out.slot_mask = slots - 1;
    out.first = ws.take<int32_t>(cap);
    out.unique = ws.take<int32_t>(cap);
    out.count = ws.take<int>(1);
    out.bloom_words = bloom_words_for(n);
    out.bloom = out.bloom_words ? ws.take<uint32_t>(out.bloom_words) : nullptr;
    return out;
}

template <int W>
int build_hashrows(const uint8_t* rows, int nq, HashRows& out, cudaStream_t s) {
    const int64_t n = out.n;
    QMBX_CUDA_TRY(cudaMemsetAsync(out.slots, 0xff, (out.slot_mask + 1) * sizeof(uint64_t), s));
    QMBX_CUDA_TRY(cudaMemsetAsync(out.count, 0, sizeof(int), s));
    if (n == 0) return QMBX_OK;
    int st;
    if ((st = pack_rows<W>(rows, n, nq, out.keys, s)) != QMBX_OK) return st;
    const unsigned grid = grid_for(n, kThreads);
    // the filter (when the set has one) is complete before the first lookup (the resolve pass)
    if (out.bloom_words) QMBX_CUDA_TRY(cudaMemsetAsync(out.bloom, 0, (size_t)out.bloom_words * sizeof(uint32_t), s));
    QMBX_KERNEL(kGroupKeys, s, hashrows_insert_kernel<W><<<grid, kThreads, 0, s>>>(out.keys, n, out.slots, out.slot_mask,
                                                                  out.bloom_words ? out.bloom : nullptr,
                                                                  out.bloom_words ? out.bloom_words - 1 : 0));
    QMBX_KERNEL(kGroupKeys, s, hashrows_resolve_kernel<W><<<grid, kThreads, 0, s>>>(out.keys, n, out.hash(), out.first, out.unique, out.count));
    QMBX_LAUNCH_CHECK("build_hashrows");
    return QMBX_OK;
}

#define QMBX_INSTANTIATE_KEYS(W)                                                                                \
    template int pack_rows<W>(const uint8_t*, int64_t, int, uint64_t*, cudaStream_t);                           \
    template int unpack_rows<W>(const uint64_t*, const int*, int64_t, int, uint8_t*, cudaStream_t);             \
    template SortScratch take_sort_scratch<W>(Arena&, int64_t);                                                 \
    template int sort_pairs<W>(const uint64_t*, const int32_t*, uint64_t*, int32_t*, int64_t, int,              \
                               const SortScratch&, cudaStream_t);                                               \
    template RowSet take_rowset<W>(Arena&, int64_t);                                                            \
    template int build_rowset<W>(const uint8_t*, int, RowSet&, cudaStream_t);                                   \
    template int sort_unique_keys<W>(const uint64_t*, int, RowSet&, cudaStream_t);                              \
    template HashRows take_hashrows<W>(Arena&, int64_t);                                                        \
    template int build_hashrows<W>(const uint8_t*, int, HashRows&, cudaStream_t);

QMBX_INSTANTIATE_KEYS(1)
QMBX_INSTANTIATE_KEYS(2)
QMBX_INSTANTIATE_KEYS(3)
QMBX_INSTANTIATE_KEYS(4)

}  // namespace qmbx

namespace qmbx {

static int sm_count() {
    static int sms[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = 0;
    if (sms[dev] == 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 132;
        sms[dev] = v;
    }
    return sms[dev];
}

int pivot_grid() { return sm_count() * 4; }

int row_split(int64_t n_rows) {
    const int64_t warps = (int64_t)sm_count() * 32 * 2;  // two waves of 32 resident warps per SM
    if (n_rows <= 0 || n_rows >= warps) return 1;
    const int64_t k = (warps + n_rows - 1) / n_rows;
    return (int)(k < 16 ? k : 16);
}

Walk choose_walk(const PartView& part, int64_t n_rows, bool pivot_ok) {
    const char* e = getenv("QMBX_WALK");
    const char f = e != nullptr ? e[0] : 0;
    if (part.n == 0 || f == 't') return Walk::kTiled;
    if (f == 'p') return pivot_ok ? Walk::kPivot : Walk::kGrouped;
    if (f == 'g') return Walk::kGrouped;
    if (part.n >= kGroupedMinTerms) {
        // groups holding hundreds of terms amortise staging them in shared memory
        const bool big_groups = part.n_nonempty > 0 && part.n >= (int64_t)kPivotMeanGroup * part.n_nonempty;
        if (pivot_ok && big_groups) return Walk::kPivot;
        // groups of a few terms (the diagonal part of an ab-initio table) over many rows: testing
        // every term of a shared-memory tile against each row, all lanes on the same term, costs
        // less than dealing the small groups to the lanes (C5's 1M-row diagonal: 12.9 -> ~3 ms)
        if (!part.wide && part.n <= kTiledMaxTerms && n_rows >= kFewWideRows) return Walk::kTiled;
        return Walk::kGrouped;
    }
    return n_rows < (part.wide ? kFewWideRows : kFewRows) ? Walk::kGrouped : Walk::kTiled;
}

bool deterministic_mode() {
    const char* e = getenv("QMBX_DETERMINISTIC");
    return e != nullptr && e[0] != 0 && e[0] != '0';
}

int grouped_grid(int64_t n_rows) {
    static int sms[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = 0;
    if (sms[dev] == 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 132;
        sms[dev] = v;
    }
    int64_t want = (n_rows + kWarpsPerBlock - 1) / kWarpsPerBlock;
    int64_t cap = (int64_t)sms[dev] * 16;
    if (want > cap) want = cap;
    return (int)(want > 0 ? want : 1);
}

}  // namespace qmbx
