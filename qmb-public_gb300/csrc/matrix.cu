// H restricted to one set of rows, materialised as a sparse matrix.
//
// The reference's Lanczos loops (qmb/rldiag.py:19-52, qmb/haar.py:107-183)
// call apply_within on the same rows once per iteration, so every iteration
// walks the whole term table again.  Here the walk runs twice in total (count
// the entries of every row, then fill them) and each iteration is a sparse
// matrix-vector product over the stored entries, which reads nnz x 20 bytes
// from HBM instead of walking T terms per row.
//
// Layout (CSR): row j holds, at [row_ptr[j], row_ptr[j + 1]), first the
// diagonal entry (column j, the sum of the diagonal terms, possibly zero),
// then one entry per (term, row i) pair that maps row i onto row j, with the
// sign-folded coefficient as value; pairs that reach the same (j, i) through
// different terms are separate entries.  Rows must be distinct.
#include <cuda_runtime.h>

#include "device.cuh"

namespace qmbx {
namespace {

// Grouped / tiled walks (warp or thread per walked row j, daggered terms):
// every hit is an entry (row j, column = the looked-up row).
template <int W, bool FILL>
struct MatrixRows : VisitorBase {
    HashView lookup;
    const double2* coef;     // adjoint part: stored coefficient, sign folded
    const int32_t* unique;   // walk index -> row
    int32_t* count;          // COUNT: off-diagonal entries per row
    int64_t* cursor;         // FILL: next free entry of each row
    int32_t* col;
    double2* val;
    struct Acc {
        int32_t row;
        int n;
    };
    static constexpr bool kBatched = true;
    __device__ __forceinline__ void init(Acc& a, int64_t u, const Key<W>&, int*) const {
        a.row = __ldg(unique + u);
        a.n = 0;
    }
    __device__ __forceinline__ bool probe(Acc&, const Key<W>&, const Key<W>& img, int parity, int64_t slot,
                                          int2& h) const {
        const int64_t pos = hash_find<W>(lookup, img);
        if (pos < 0) return false;
        h = make_int2((int)slot | (parity << 31), (int)pos);
        return true;
    }
    __device__ __forceinline__ void apply_hit(Acc& a, int2 h) const {
        if (!FILL) {
            ++a.n;
            return;
        }
        const double2 cf = __ldg(coef + (h.x & 0x7fffffff));
        const int64_t e = (int64_t)atomicAdd(reinterpret_cast<unsigned long long*>(cursor + a.row), 1ull);
        col[e] = h.y;
        val[e] = h.x < 0 ? make_double2(-cf.x, -cf.y) : cf;
    }
    __device__ __forceinline__ void visit(Acc& a, const Key<W>& c, const Key<W>& img, int parity, int64_t slot) const {
        int2 h;
        if (probe(a, c, img, parity, slot, h)) apply_hit(a, h);
    }
    __device__ __forceinline__ void visit_diag(Acc&, const Key<W>&, int, int64_t) const {}
    __device__ __forceinline__ void reduce(Acc& a) const {
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) a.n += __shfl_xor_sync(0xffffffffu, a.n, d);
    }
    __device__ __forceinline__ void finish(Acc& a, int64_t, const Key<W>&) const {
        if (!FILL) count[a.row] = a.n;
    }
};

// Pivot-major walk: hits carry their walked row; entries claimed with atomics.
template <int W, bool FILL>
struct MatrixPivot : VisitorBase {
    static constexpr bool kStateless = true;
    HashView lookup;
    const double2* coef;
    const int32_t* unique;
    int32_t* count;
    int64_t* cursor;
    int32_t* col;
    double2* val;
    struct Acc {};
    __device__ __forceinline__ bool probe_row(const Key<W>&, const Key<W>& img, int parity, int64_t slot, int64_t u,
                                              int4& h) const {
        const int64_t pos = hash_find<W>(lookup, img);
        if (pos < 0) return false;
        h = make_int4((int)slot | (parity << 31), (int)pos, (int)u, 0);
        return true;
    }
    __device__ __forceinline__ void apply_row_hit(int4 h) const {
        const int32_t row = __ldg(unique + h.z);
        if (!FILL) {
            atomicAdd(count + row, 1);
            return;
        }
        const double2 cf = __ldg(coef + (h.x & 0x7fffffff));
        const int64_t e = (int64_t)atomicAdd(reinterpret_cast<unsigned long long*>(cursor + row), 1ull);
        col[e] = h.y;
        val[e] = h.x < 0 ? make_double2(-cf.x, -cf.y) : cf;
    }
};

// The diagonal entry of every walked row (first entry of the row).
template <int W>
struct MatrixDiagonal : VisitorBase {
    const double2* dcoef;
    const int32_t* unique;
    const int64_t* row_ptr;
    int32_t* col;
    double2* val;
    struct Acc {
        double re, im;
    };
    __device__ __forceinline__ void init(Acc& a, int64_t, const Key<W>&, int*) const { a.re = a.im = 0.0; }
    __device__ __forceinline__ void visit(Acc&, const Key<W>&, const Key<W>&, int, int64_t) const {}
    __device__ __forceinline__ void visit_diag(Acc& a, const Key<W>&, int parity, int64_t slot) const {
        const double2 cf = __ldg(dcoef + slot);
        a.re += parity ? -cf.x : cf.x;
        a.im += parity ? -cf.y : cf.y;
    }
    __device__ __forceinline__ void reduce(Acc& a) const {
        a.re = warp_sum(a.re);
        a.im = warp_sum(a.im);
    }
    __device__ __forceinline__ void finish(Acc& a, int64_t u, const Key<W>&) const {
        const int32_t row = __ldg(unique + u);
        const int64_t e = row_ptr[row];
        col[e] = row;
        val[e] = make_double2(a.re, a.im);
    }
};

// count[i] += 1 (the diagonal entry); the 64-bit total of the counts goes to *total
__global__ void plus_one_kernel(int32_t* __restrict__ count, int64_t n, unsigned long long* __restrict__ total) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long v = 0;
    if (i < n) {
        count[i] += 1;
        v = (unsigned long long)(uint32_t)count[i];
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(total, v);
}

// row_ptr[i] = offsets[i] (exclusive scan of the per-row counts), row_ptr[n] = total
__global__ void row_ptr_kernel(const int32_t* __restrict__ offsets, const int* __restrict__ total, int64_t n,
                               int64_t* __restrict__ row_ptr) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) row_ptr[i] = (int64_t)(uint32_t)offsets[i];
    if (i == n) row_ptr[n] = (int64_t)(uint32_t)*total;
}

// cursor[i] = row_ptr[i] + 1: the diagonal entry keeps the first place
__global__ void cursor_kernel(const int64_t* __restrict__ row_ptr, int64_t n, int64_t* __restrict__ cursor) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) cursor[i] = row_ptr[i] + 1;
}

// y = A x, one warp per row, lanes over the row's entries in order, a fixed
// butterfly sum: the same bits on every call.
__global__ void __launch_bounds__(kThreads) spmv_kernel(int64_t n, const int64_t* __restrict__ row_ptr,
                                                        const int32_t* __restrict__ col,
                                                        const double2* __restrict__ val,
                                                        const double2* __restrict__ x, double2* __restrict__ y) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * kWarpsPerBlock;
    for (int64_t j = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5); j < n; j += warps) {
        const int64_t b = __ldg(row_ptr + j), e = __ldg(row_ptr + j + 1);
        double re = 0.0, im = 0.0;
        for (int64_t k = b + lane; k < e; k += 32) {
            const double2 v = __ldg(val + k);
            const double2 p = __ldg(x + __ldg(col + k));
            re += v.x * p.x - v.y * p.y;
            im += v.x * p.y + v.y * p.x;
        }
        re = warp_sum(re);
        im = warp_sum(im);
        if (lane == 0) y[j] = make_double2(re, im);
    }
}

// y = A x for rows with few entries (the mean below kFewEntries): one thread
// per row, entries summed in order.
__global__ void __launch_bounds__(kThreads) spmv_rows_kernel(int64_t n, const int64_t* __restrict__ row_ptr,
                                                             const int32_t* __restrict__ col,
                                                             const double2* __restrict__ val,
                                                             const double2* __restrict__ x, double2* __restrict__ y) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int64_t b = __ldg(row_ptr + j), e = __ldg(row_ptr + j + 1);
    double re = 0.0, im = 0.0;
    for (int64_t k = b; k < e; ++k) {
        const double2 v = __ldg(val + k);
        const double2 p = __ldg(x + __ldg(col + k));
        re += v.x * p.x - v.y * p.y;
        im += v.x * p.y + v.y * p.x;
    }
    y[j] = make_double2(re, im);
}
constexpr int64_t kFewEntries = 4;

// Y = A X for m vectors (X, Y row-major [n][m]): one warp per row, lane l
// owns vectors l, l + 32, ...; the row's entries are read once per 32
// vectors (the same address across lanes) and summed in order.
__global__ void __launch_bounds__(kThreads) spmm_kernel(int64_t n, int m, const int64_t* __restrict__ row_ptr,
                                                        const int32_t* __restrict__ col,
                                                        const double2* __restrict__ val,
                                                        const double2* __restrict__ x, double2* __restrict__ y) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * kWarpsPerBlock;
    for (int64_t j = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5); j < n; j += warps) {
        const int64_t b = __ldg(row_ptr + j), e = __ldg(row_ptr + j + 1);
        for (int c = lane; c < m; c += 32) {
            double re = 0.0, im = 0.0;
            for (int64_t k = b; k < e; ++k) {
                const double2 v = __ldg(val + k);
                const double2 p = __ldg(x + (int64_t)__ldg(col + k) * m + c);
                re += v.x * p.x - v.y * p.y;
                im += v.x * p.y + v.y * p.x;
            }
            y[j * m + c] = make_double2(re, im);
        }
    }
}

struct MatrixLayout {
    HashRows rows;
    int32_t* count;
    int32_t* scan;
    int* total;
    unsigned long long* total64;
    int64_t* cursor;
};

template <int W>
MatrixLayout take_matrix(Arena& ws, int64_t n) {
    MatrixLayout L;
    L.rows = take_hashrows<W>(ws, n);
    const uint64_t cap = (uint64_t)(n > 0 ? n : 1);
    L.count = ws.take<int32_t>(cap);
    L.scan = ws.take<int32_t>((uint64_t)scan_scratch(n));
    L.total = ws.take<int>(1);
    L.total64 = ws.take<unsigned long long>(1);
    L.cursor = ws.take<int64_t>(cap);
    return L;
}

// Walk the changing terms of every row (daggered terms, gather direction).
template <int W, bool FILL>
int matrix_walk(const void* table_host, const void* table_dev, const MatrixLayout& L, int64_t n, const int64_t* row_ptr,
                int32_t* col, double2* val, cudaStream_t s) {
    PartView adj = part_view(table_host, table_dev, QMBX_PART_ADJ);
    PartView diag = part_view(table_host, table_dev, QMBX_PART_DIAG);
    PartView none = adj;
    none.n = 0;
    const HashView look = L.rows.hash();
    UniqueRows<W> src{L.rows.keys, L.rows.unique};
    if (adj.n > 0) {
        const Walk kind = choose_walk(adj, n, true);
        if (kind == Walk::kPivot) {
            MatrixPivot<W, FILL> v{{}, look, adj.coef, L.rows.unique, L.count, L.cursor, col, val};
            QMBX_KERNEL(kGroupEnumerate, s, pivot_kernel<W><<<pivot_grid(), kThreads, 0, s>>>(v, src, L.rows.count, n, adj));
        } else {
            MatrixRows<W, FILL> v{{}, look, adj.coef, L.rows.unique, L.count, L.cursor, col, val};
            if (kind == Walk::kGrouped) {
                QMBX_KERNEL(kGroupEnumerate, s, grouped_kernel<W><<<grouped_grid(n), kThreads, 0, s>>>(v, src, L.rows.count, n, adj, none));
            } else {
                QMBX_KERNEL(kGroupEnumerate, s, enumerate_kernel<W><<<grid_for(n, kThreads), kThreads, 0, s>>>(v, src, L.rows.count, n, adj, none));
            }
        }
        QMBX_LAUNCH_CHECK("matrix walk");
    }
    if (FILL) {
        MatrixDiagonal<W> dv{{}, diag.coef, L.rows.unique, row_ptr, col, val};
        PartView nd = diag;
        if (choose_walk(diag, n, false) == Walk::kGrouped) {
            QMBX_KERNEL(kGroupDiagonal, s, grouped_kernel<W><<<grouped_grid(n), kThreads, 0, s>>>(dv, src, L.rows.count, n, none, nd));
        } else {
            QMBX_KERNEL(kGroupDiagonal, s, enumerate_kernel<W><<<grid_for(n, kThreads), kThreads, 0, s>>>(dv, src, L.rows.count, n, none, nd));
        }
        QMBX_LAUNCH_CHECK("matrix diagonal pass");
    }
    return QMBX_OK;
}

template <int W>
int matrix_count(const void* table_host, const void* table_dev, const uint8_t* configs, int64_t n, int64_t* row_ptr,
                 int64_t* nnz, Arena& ws, cudaStream_t s) {
    MatrixLayout L = take_matrix<W>(ws, n);
    if (ws.base == nullptr) return QMBX_OK;
    if (!ws.fits()) return fail(QMBX_ERR_WORKSPACE, "matrix needs %llu bytes of workspace", (unsigned long long)ws.used);
    const int nq = header_of(table_host)->n_qubytes;
    int st;
    if ((st = build_hashrows<W>(configs, nq, L.rows, s)) != QMBX_OK) return st;
    QMBX_CUDA_TRY(cudaMemsetAsync(L.count, 0, (size_t)n * sizeof(int32_t), s));
    if ((st = matrix_walk<W, false>(table_host, table_dev, L, n, nullptr, nullptr, nullptr, s)) != QMBX_OK) return st;
    QMBX_CUDA_TRY(cudaMemsetAsync(L.total64, 0, sizeof(unsigned long long), s));
    QMBX_KERNEL(kGroupOther, s, plus_one_kernel<<<grid_for(n, kThreads), kThreads, 0, s>>>(L.count, n, L.total64));
    if ((st = exclusive_scan(L.count, L.count, n, L.total, L.scan, s)) != QMBX_OK) return st;
    QMBX_KERNEL(kGroupOther, s, row_ptr_kernel<<<grid_for(n + 1, kThreads), kThreads, 0, s>>>(L.count, L.total, n, row_ptr));
    QMBX_LAUNCH_CHECK("matrix row pointers");
    int unique = 0;
    unsigned long long total = 0;
    QMBX_CUDA_TRY(cudaMemcpyAsync(&unique, L.rows.count, sizeof(int), cudaMemcpyDeviceToHost, s));
    QMBX_CUDA_TRY(cudaMemcpyAsync(&total, L.total64, sizeof(total), cudaMemcpyDeviceToHost, s));
    QMBX_CUDA_TRY(cudaStreamSynchronize(s));
    if (unique != n) return fail(QMBX_ERR_ARGUMENT, "matrix rows must be distinct (%d distinct of %lld)", unique, (long long)n);
    // the per-row offsets are scanned in 32 bits
    if (total >= (1ull << 31)) return fail(QMBX_ERR_ARGUMENT, "matrix has %llu entries, 2^31 or more", total);
    *nnz = (int64_t)total;
    return QMBX_OK;
}

template <int W>
int matrix_fill(const void* table_host, const void* table_dev, const uint8_t* configs, int64_t n, const int64_t* row_ptr,
                int32_t* col, double2* val, Arena& ws, cudaStream_t s) {
    MatrixLayout L = take_matrix<W>(ws, n);
    if (ws.base == nullptr) return QMBX_OK;
    if (!ws.fits()) return fail(QMBX_ERR_WORKSPACE, "matrix needs %llu bytes of workspace", (unsigned long long)ws.used);
    const int nq = header_of(table_host)->n_qubytes;
    int st;
    if ((st = build_hashrows<W>(configs, nq, L.rows, s)) != QMBX_OK) return st;
    QMBX_KERNEL(kGroupOther, s, cursor_kernel<<<grid_for(n, kThreads), kThreads, 0, s>>>(row_ptr, n, L.cursor));
    QMBX_LAUNCH_CHECK("matrix cursors");
    return matrix_walk<W, true>(table_host, table_dev, L, n, row_ptr, col, val, s);
}

int matrix_args(const void* table_host, const void* table_dev, const uint8_t* configs, int64_t n, void* workspace) {
    int st = check_table(table_host, table_dev);
    if (st != QMBX_OK) return st;
    if (n < 0 || n >= (int64_t(1) << 31)) return fail(QMBX_ERR_ARGUMENT, "row count out of range");
    if (n > 0 && configs == nullptr) return fail(QMBX_ERR_ARGUMENT, "configs must not be NULL");
    if (workspace != nullptr && reinterpret_cast<uintptr_t>(workspace) % QMBX_ALIGN != 0) {
        return fail(QMBX_ERR_ARGUMENT, "workspace must be %d-byte aligned", QMBX_ALIGN);
    }
    return QMBX_OK;
}

}  // namespace
}  // namespace qmbx

using namespace qmbx;

extern "C" int qmbx_matrix_workspace(const void* table_host, int64_t n, uint64_t* bytes) {
    clear_error();
    const qmbx_table_header* h = header_of(table_host);
    if (h == nullptr || h->magic != QMBX_MAGIC) return fail(QMBX_ERR_ARGUMENT, "not a compiled qmbx table");
    if (bytes == nullptr) return fail(QMBX_ERR_ARGUMENT, "bytes must not be NULL");
    Arena probe(nullptr, 0);
    switch (h->n_words) {
        case 1: take_matrix<1>(probe, n); break;
        case 2: take_matrix<2>(probe, n); break;
        case 3: take_matrix<3>(probe, n); break;
        case 4: take_matrix<4>(probe, n); break;
        default: return fail(QMBX_ERR_ARGUMENT, "unsupported word count");
    }
    *bytes = probe.used;
    return QMBX_OK;
}

extern "C" int qmbx_matrix_count(const void* table_host, const void* table_dev, const uint8_t* configs, int64_t n,
                                 int64_t* row_ptr, int64_t* nnz, void* workspace, uint64_t workspace_bytes,
                                 qmbx_stream_t stream) {
    clear_error();
    int st = matrix_args(table_host, table_dev, configs, n, workspace);
    if (st != QMBX_OK) return st;
    if (row_ptr == nullptr || nnz == nullptr) return fail(QMBX_ERR_ARGUMENT, "row_ptr and nnz must not be NULL");
    *nnz = 0;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (n == 0) {
        QMBX_CUDA_TRY(cudaMemsetAsync(row_ptr, 0, sizeof(int64_t), s));
        return QMBX_OK;
    }
    if (workspace == nullptr) return fail(QMBX_ERR_WORKSPACE, "matrix needs a workspace");
    Arena ws(workspace, workspace_bytes);
    switch (header_of(table_host)->n_words) {
        case 1: return matrix_count<1>(table_host, table_dev, configs, n, row_ptr, nnz, ws, s);
        case 2: return matrix_count<2>(table_host, table_dev, configs, n, row_ptr, nnz, ws, s);
        case 3: return matrix_count<3>(table_host, table_dev, configs, n, row_ptr, nnz, ws, s);
        case 4: return matrix_count<4>(table_host, table_dev, configs, n, row_ptr, nnz, ws, s);
        default: return fail(QMBX_ERR_ARGUMENT, "unsupported word count");
    }
}

extern "C" int qmbx_matrix_fill(const void* table_host, const void* table_dev, const uint8_t* configs, int64_t n,
                                const int64_t* row_ptr, int32_t* col, double* val, void* workspace,
                                uint64_t workspace_bytes, qmbx_stream_t stream) {
    clear_error();
    int st = matrix_args(table_host, table_dev, configs, n, workspace);
    if (st != QMBX_OK) return st;
    if (n == 0) return QMBX_OK;
    if (row_ptr == nullptr || col == nullptr || val == nullptr) return fail(QMBX_ERR_ARGUMENT, "pointers must not be NULL");
    if (workspace == nullptr) return fail(QMBX_ERR_WORKSPACE, "matrix needs a workspace");
    Arena ws(workspace, workspace_bytes);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    double2* v = reinterpret_cast<double2*>(val);
    switch (header_of(table_host)->n_words) {
        case 1: return matrix_fill<1>(table_host, table_dev, configs, n, row_ptr, col, v, ws, s);
        case 2: return matrix_fill<2>(table_host, table_dev, configs, n, row_ptr, col, v, ws, s);
        case 3: return matrix_fill<3>(table_host, table_dev, configs, n, row_ptr, col, v, ws, s);
        case 4: return matrix_fill<4>(table_host, table_dev, configs, n, row_ptr, col, v, ws, s);
        default: return fail(QMBX_ERR_ARGUMENT, "unsupported word count");
    }
}

extern "C" int qmbx_matrix_apply(int64_t n, const int64_t* row_ptr, const int32_t* col, const double* val,
                                 const double* x, double* y, qmbx_stream_t stream) {
    clear_error();
    if (n < 0 || n >= (int64_t(1) << 31)) return fail(QMBX_ERR_ARGUMENT, "row count out of range");
    if (n == 0) return QMBX_OK;
    if (row_ptr == nullptr || col == nullptr || val == nullptr || x == nullptr || y == nullptr) {
        return fail(QMBX_ERR_ARGUMENT, "pointers must not be NULL");
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    QMBX_KERNEL(kGroupSpmv, s, spmv_kernel<<<grouped_grid(n), kThreads, 0, s>>>(n, row_ptr, col, reinterpret_cast<const double2*>(val), reinterpret_cast<const double2*>(x), reinterpret_cast<double2*>(y)));
    QMBX_LAUNCH_CHECK("spmv_kernel");
    return QMBX_OK;
}

extern "C" int qmbx_matrix_apply_many(int64_t n, int64_t nnz, int32_t m, const int64_t* row_ptr, const int32_t* col,
                                      const double* val, const double* x, double* y, qmbx_stream_t stream) {
    clear_error();
    if (n < 0 || n >= (int64_t(1) << 31)) return fail(QMBX_ERR_ARGUMENT, "row count out of range");
    if (nnz < 0 || m < 1) return fail(QMBX_ERR_ARGUMENT, "entry count or vector count out of range");
    if (n == 0) return QMBX_OK;
    if (row_ptr == nullptr || col == nullptr || (nnz > 0 && val == nullptr) || x == nullptr || y == nullptr) {
        return fail(QMBX_ERR_ARGUMENT, "pointers must not be NULL");
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const double2* v = reinterpret_cast<const double2*>(val);
    const double2* xx = reinterpret_cast<const double2*>(x);
    double2* yy = reinterpret_cast<double2*>(y);
    if (m > 1) {
        QMBX_KERNEL(kGroupSpmv, s, spmm_kernel<<<grouped_grid(n), kThreads, 0, s>>>(n, m, row_ptr, col, v, xx, yy));
    } else if (nnz < kFewEntries * n) {
        QMBX_KERNEL(kGroupSpmv, s, spmv_rows_kernel<<<grid_for(n, kThreads), kThreads, 0, s>>>(n, row_ptr, col, v, xx, yy));
    } else {
        QMBX_KERNEL(kGroupSpmv, s, spmv_kernel<<<grouped_grid(n), kThreads, 0, s>>>(n, row_ptr, col, v, xx, yy));
    }
    QMBX_LAUNCH_CHECK("matrix product");
    return QMBX_OK;
}
