// apply_within (forward and adjoint, FP64 and compensated FP32) and
// diagonal_term.
//
// The reference scatters: one thread per (term, source) pair, a byte-wise
// binary search of the image among the sorted targets, and FP64 atomics
// (qmb/_hamiltonian_cuda.cu:86-274).  Here the work is gathered instead: one
// thread per distinct target row walks the daggered terms, finds the source
// row among the sorted, de-duplicated sources and accumulates in registers,
// so no atomics are needed and the summation order is fixed.  The adjoint
// runs the same walk with the forward terms over the sources.
#include <cuda_runtime.h>

#include "device.cuh"

namespace qmbx {

int check_table(const void* table_host, const void* table_dev) {
    const qmbx_table_header* h = header_of(table_host);
    if (h == nullptr || h->magic != QMBX_MAGIC || h->version != QMBX_TABLE_VERSION) {
        return fail(QMBX_ERR_ARGUMENT, "table_host is not a compiled qmbx table");
    }
    if (table_dev == nullptr || (reinterpret_cast<uintptr_t>(table_dev) % QMBX_ALIGN) != 0) {
        return fail(QMBX_ERR_ARGUMENT, "table_dev must be a %d-byte aligned device copy of the table", QMBX_ALIGN);
    }
    if (h->n_words < 1 || h->n_words > QMBX_MAX_WORDS) {
        return fail(QMBX_ERR_ARGUMENT, "table has an unsupported word count %d", h->n_words);
    }
    return QMBX_OK;
}

namespace {

// ---------------------------------------------------------------------------
// compensated FP32 arithmetic: TwoSum (Knuth) and the FMA two-product
// (Ogita, Rump and Oishi, "Accurate sum and dot product", SIAM J. Sci.
// Comput. 26(6), 2005).  The _rn intrinsics are never contracted or
// re-associated by the compiler.
// ---------------------------------------------------------------------------

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
    p = __fmul_rn(a, b);
    e = __fmaf_rn(a, b, -p);
}

struct CompSum {
    float s, c;
    __device__ __forceinline__ void zero() { s = c = 0.f; }
    __device__ __forceinline__ void add(float x) {
        float e;
        two_sum(s, x, s, e);
        c = __fadd_rn(c, e);
    }
    // a value split in a leading part and a tail (a coefficient's hi/lo pair)
    __device__ __forceinline__ void add2(float hi, float lo) {
        float e;
        two_sum(s, hi, s, e);
        c = __fadd_rn(c, __fadd_rn(e, lo));
    }
    __device__ __forceinline__ double value() const { return (double)s + (double)c; }
    // Combine the lanes' pairs: two-sum of the leading parts, plain sum of the tails.
    __device__ __forceinline__ void warp_reduce() { group_reduce<32>(); }
    // The same within aligned groups of L lanes (every lane of a group ends with its total).
    template <int L>
    __device__ __forceinline__ void group_reduce() {
#pragma unroll
        for (int d = L / 2; d > 0; d >>= 1) {
            float s2 = __shfl_xor_sync(0xffffffffu, s, d);
            float c2 = __shfl_xor_sync(0xffffffffu, c, d);
            float e;
            two_sum(s, s2, s, e);
            c = __fadd_rn(c, __fadd_rn(c2, e));
        }
    }
};

// A diagonal coefficient (hi/lo split) with sign (-1)^parity and optional
// conjugation, added to the compensated sums (dre, dim): FP32 work, so that
// the divergent per-term adds of a walk do not queue on the FP64 pipe.
template <bool CONJ>
__device__ __forceinline__ void comp_diag_add(CompSum& dre, CompSum& dim, float4 cf, int parity) {
    const float sg = parity ? -1.f : 1.f;
    const float ih = CONJ ? -cf.z : cf.z, il = CONJ ? -cf.w : cf.w;
    dre.add2(sg * cf.x, sg * cf.y);
    dim.add2(sg * ih, sg * il);
}

// coef (hi/lo split, sign already folded) times psi, added to (re, im) with
// sign (-1)^parity and optional conjugation of the coefficient.
template <bool CONJ>
__device__ __forceinline__ void comp_cmul_add(CompSum& re, CompSum& im, float4 cf, float2 p, int parity) {
    float chr = cf.x, clr = cf.y, chi = CONJ ? -cf.z : cf.z, cli = CONJ ? -cf.w : cf.w;
    if (parity) {
        chr = -chr;
        clr = -clr;
        chi = -chi;
        cli = -cli;
    }
    float a, ea, b, eb;
    // real part: chr*px - chi*py (+ low parts)
    two_prod(chr, p.x, a, ea);
    two_prod(chi, p.y, b, eb);
    re.add(a);
    re.add(-b);
    re.c = __fadd_rn(re.c, __fadd_rn(__fsub_rn(ea, eb), __fsub_rn(__fmul_rn(clr, p.x), __fmul_rn(cli, p.y))));
    // imaginary part: chr*py + chi*px (+ low parts)
    two_prod(chr, p.y, a, ea);
    two_prod(chi, p.x, b, eb);
    im.add(a);
    im.add(b);
    im.c = __fadd_rn(im.c, __fadd_rn(__fadd_rn(ea, eb), __fadd_rn(__fmul_rn(clr, p.y), __fmul_rn(cli, p.x))));
}

// ---------------------------------------------------------------------------
// visitors
// ---------------------------------------------------------------------------

// Forward (CONJ = false: targets walk the adjoint part, coef as stored) or
// adjoint (CONJ = true: sources walk the forward part, coef conjugated).
// Values of the looked-up rows sit in val[u] for unique key u of lookup.
template <int W, bool CONJ>
struct GatherF64 : VisitorBase {
    static constexpr bool kTiledDense = true;
    HashView lookup;         // hash set over the unique keys of the looked-up row set
    const double2* val;      // one amplitude per unique looked-up key
    const double2* coef;     // coefficients of the walked part
    const double2* dcoef;    // coefficients of the diagonal part
    const int32_t* unique;   // walk index -> first row of the walked key
    double2* res;            // result per first row of the walked side
    HitLog log;              // optional record of the hits (for the adjoint without a walk)
    struct Acc {
        double re, im, dre, dim;
        int row;
    };
    __device__ __forceinline__ void init(Acc& a, int64_t u, const Key<W>&, int*) const {
        a.re = a.im = a.dre = a.dim = 0.0;
        a.row = __ldg(unique + u);
    }
    __device__ __forceinline__ void record_hits(const Acc& a, const int2* q, int n, int lane) const {
        log_hits(log, a.row, q, n, lane);
    }
    __device__ __forceinline__ void record_hit(const Acc& a, int2 h) const { log_hit(log, a.row, h); }
    static constexpr bool kBatched = true;
    static constexpr bool kProbe = true;
    __device__ __forceinline__ bool take(Acc&, const Key<W>&, const Key<W>&, int parity, int64_t slot, int64_t pos,
                                         int2& h) const {
        if (pos < 0) return false;
        h = make_int2((int)slot | (parity << 31), (int)pos);
        return true;
    }
    __device__ __forceinline__ bool probe(Acc& a, const Key<W>& c, const Key<W>& img, int parity, int64_t slot,
                                          int2& h) const {
        return take(a, c, img, parity, slot, hash_find<W>(lookup, img), h);
    }
    __device__ __forceinline__ void apply_hit(Acc& a, int2 h) const {
        const int slot = h.x & 0x7fffffff;
        double2 cf = __ldg(coef + slot);
        double2 p = __ldg(val + h.y);
        double ci = CONJ ? -cf.y : cf.y;
        double re = cf.x * p.x - ci * p.y;
        double im = cf.x * p.y + ci * p.x;
        if (h.x < 0) {
            re = -re;
            im = -im;
        }
        a.re += re;
        a.im += im;
    }
    __device__ __forceinline__ void visit(Acc& a, const Key<W>& c, const Key<W>& img, int parity, int64_t slot) const {
        int2 h;
        if (probe(a, c, img, parity, slot, h)) {
            record_hit(a, h);
            apply_hit(a, h);
        }
    }
    __device__ __forceinline__ void visit_diag(Acc& a, const Key<W>&, int parity, int64_t slot) const {
        double2 cf = __ldg(dcoef + slot);
        double ci = CONJ ? -cf.y : cf.y;
        a.dre += parity ? -cf.x : cf.x;
        a.dim += parity ? -ci : ci;
    }
    __device__ __forceinline__ void reduce(Acc& a) const {
        a.re = warp_sum(a.re);
        a.im = warp_sum(a.im);
        a.dre = warp_sum(a.dre);
        a.dim = warp_sum(a.dim);
    }
    __device__ __forceinline__ void finish(Acc& a, int64_t u, const Key<W>& c) const {
        if (a.dre != 0.0 || a.dim != 0.0) {
            int64_t pos = hash_find<W>(lookup, c);
            if (pos >= 0) log_diag(log, u, a.row, pos, a.dre, CONJ ? -a.dim : a.dim);
            if (pos >= 0) {
                double2 p = __ldg(val + pos);
                a.re += a.dre * p.x - a.dim * p.y;
                a.im += a.dre * p.y + a.dim * p.x;
            }
        }
        res[__ldg(unique + u)] = make_double2(a.re, a.im);
    }
    // pivot-major walks: one (row, group) partial, added atomically; the
    // diagonal part is applied by a separate pass
    __device__ __forceinline__ void flush(Acc& a, int64_t u, const Key<W>&) const {
        double2* r = res + __ldg(unique + u);
        if (a.re != 0.0) atomicAdd(&r->x, a.re);
        if (a.im != 0.0) atomicAdd(&r->y, a.im);
    }
};

template <int W, bool CONJ>
struct GatherF32C : VisitorBase {
    static constexpr bool kTiledDense = true;
    HashView lookup;
    const float2* val;
    const float4* coef32;
    const float4* dcoef32;   // diagonal part, hi/lo FP32
    int include_diag;
    const int32_t* unique;
    double2* res;
    HitLog log;
    struct Acc {
        CompSum re, im, dre, dim;
        int row;
    };
    __device__ __forceinline__ void init(Acc& a, int64_t u, const Key<W>&, int*) const {
        a.re.zero();
        a.im.zero();
        a.dre.zero();
        a.dim.zero();
        a.row = __ldg(unique + u);
    }
    __device__ __forceinline__ void record_hits(const Acc& a, const int2* q, int n, int lane) const {
        log_hits(log, a.row, q, n, lane);
    }
    __device__ __forceinline__ void record_hit(const Acc& a, int2 h) const { log_hit(log, a.row, h); }
    static constexpr bool kBatched = true;
    static constexpr bool kProbe = true;
    __device__ __forceinline__ bool take(Acc&, const Key<W>&, const Key<W>&, int parity, int64_t slot, int64_t pos,
                                         int2& h) const {
        if (pos < 0) return false;
        h = make_int2((int)slot | (parity << 31), (int)pos);
        return true;
    }
    __device__ __forceinline__ bool probe(Acc& a, const Key<W>& c, const Key<W>& img, int parity, int64_t slot,
                                          int2& h) const {
        return take(a, c, img, parity, slot, hash_find<W>(lookup, img), h);
    }
    __device__ __forceinline__ void apply_hit(Acc& a, int2 h) const {
        comp_cmul_add<CONJ>(a.re, a.im, __ldg(coef32 + (h.x & 0x7fffffff)), __ldg(val + h.y), h.x < 0 ? 1 : 0);
    }
    __device__ __forceinline__ void visit(Acc& a, const Key<W>& c, const Key<W>& img, int parity, int64_t slot) const {
        int2 h;
        if (probe(a, c, img, parity, slot, h)) {
            record_hit(a, h);
            apply_hit(a, h);
        }
    }
    __device__ __forceinline__ void visit_diag(Acc& a, const Key<W>&, int parity, int64_t slot) const {
        comp_diag_add<CONJ>(a.dre, a.dim, __ldg(dcoef32 + slot), parity);
    }
    __device__ __forceinline__ void reduce(Acc& a) const {
        a.re.warp_reduce();
        a.im.warp_reduce();
        a.dre.warp_reduce();
        a.dim.warp_reduce();
    }
    __device__ __forceinline__ void finish(Acc& a, int64_t u, const Key<W>& c) const {
        double re = a.re.value(), im = a.im.value();
        const double dre = a.dre.value(), dim = a.dim.value();
        if (include_diag && (dre != 0.0 || dim != 0.0)) {
            int64_t pos = hash_find<W>(lookup, c);
            if (pos >= 0) log_diag(log, u, a.row, pos, dre, CONJ ? -dim : dim);
            if (pos >= 0) {
                float2 p = __ldg(val + pos);
                re += dre * (double)p.x - dim * (double)p.y;
                im += dre * (double)p.y + dim * (double)p.x;
            }
        }
        res[__ldg(unique + u)] = make_double2(re, im);
    }
    __device__ __forceinline__ void flush(Acc& a, int64_t u, const Key<W>&) const {
        const double re = a.re.value(), im = a.im.value();
        double2* r = res + __ldg(unique + u);
        if (re != 0.0) atomicAdd(&r->x, re);
        if (im != 0.0) atomicAdd(&r->y, im);
    }
};

template <int W>
struct DiagonalF64 : VisitorBase {
    const double2* dcoef;
    double2* out;
    struct Acc {
        double re, im;
    };
    __device__ __forceinline__ void init(Acc& a, int64_t, const Key<W>&, int*) const { a.re = a.im = 0.0; }
    __device__ __forceinline__ void visit(Acc&, const Key<W>&, const Key<W>&, int, int64_t) const {}
    __device__ __forceinline__ void visit_diag(Acc& a, const Key<W>&, int parity, int64_t slot) const {
        double2 cf = __ldg(dcoef + slot);
        a.re += parity ? -cf.x : cf.x;
        a.im += parity ? -cf.y : cf.y;
    }
    __device__ __forceinline__ void reduce(Acc& a) const {
        a.re = warp_sum(a.re);
        a.im = warp_sum(a.im);
    }
    __device__ __forceinline__ void finish(Acc& a, int64_t row, const Key<W>&) const {
        out[row] = make_double2(a.re, a.im);
    }
};

// Scatter: the input-side rows are walked and every image found among the
// output-side rows gets its contribution by an FP64 atomic add into acc[u].
// FP32C forms the products in FP32 (exact two-products), FP64 otherwise.
template <int W, bool CONJ, bool F32>
struct Scatter : VisitorBase {
    static constexpr bool kTiledDense = true;
    HashView lookup;        // output-side row set
    const void* val;        // amplitude per first row of the walked side (double2, or float2 for F32)
    const int32_t* unique;  // walk index -> first row of the walked key
    const double2* coef;    // walked part, FP64
    const float4* coef32;   // walked part, hi/lo FP32
    const double2* dcoef;   // diagonal part (FP64 path)
    const float4* dcoef32;  // diagonal part, hi/lo FP32 (F32 path)
    int include_diag;
    double2* acc;           // per unique output-side key
    HitLog log;
    struct Acc {
        double2 p;
        double dre, dim;    // FP64 path
        CompSum fre, fim;   // F32 path
        int row;
    };
    __device__ __forceinline__ void record_hits(const Acc& a, const int2* q, int n, int lane) const {
        log_hits(log, a.row, q, n, lane);
    }
    __device__ __forceinline__ void record_hit(const Acc& a, int2 h) const { log_hit(log, a.row, h); }
    __device__ __forceinline__ void init(Acc& a, int64_t u, const Key<W>&, int*) const {
        const int64_t row = __ldg(unique + u);
        a.row = (int)row;
        if (F32) {
            float2 q = __ldg(static_cast<const float2*>(val) + row);
            a.p = make_double2((double)q.x, (double)q.y);
        } else {
            a.p = __ldg(static_cast<const double2*>(val) + row);
        }
        a.dre = a.dim = 0.0;
        a.fre.zero();
        a.fim.zero();
    }
    static constexpr bool kBatched = true;
    static constexpr bool kProbe = true;
    __device__ __forceinline__ bool take(Acc&, const Key<W>&, const Key<W>&, int parity, int64_t slot, int64_t u,
                                         int2& h) const {
        if (u < 0) return false;
        h = make_int2((int)slot | (parity << 31), (int)u);
        return true;
    }
    __device__ __forceinline__ bool probe(Acc& a, const Key<W>& c, const Key<W>& img, int parity, int64_t slot,
                                          int2& h) const {
        return take(a, c, img, parity, slot, hash_find<W>(lookup, img), h);
    }
    __device__ __forceinline__ void apply_hit(Acc& a, int2 h) const {
        const int64_t slot = h.x & 0x7fffffff;
        const int64_t u = h.y;
        const int parity = h.x < 0 ? 1 : 0;
        double re, im;
        if (F32) {
            float4 cf = __ldg(coef32 + slot);
            float2 p = make_float2((float)a.p.x, (float)a.p.y);
            float chi = CONJ ? -cf.z : cf.z, cli = CONJ ? -cf.w : cf.w;
            float x1, e1, x2, e2;
            two_prod(cf.x, p.x, x1, e1);
            two_prod(chi, p.y, x2, e2);
            float lo = __fadd_rn(__fsub_rn(e1, e2), __fsub_rn(__fmul_rn(cf.y, p.x), __fmul_rn(cli, p.y)));
            re = ((double)x1 - (double)x2) + (double)lo;
            two_prod(cf.x, p.y, x1, e1);
            two_prod(chi, p.x, x2, e2);
            lo = __fadd_rn(__fadd_rn(e1, e2), __fadd_rn(__fmul_rn(cf.y, p.y), __fmul_rn(cli, p.x)));
            im = ((double)x1 + (double)x2) + (double)lo;
        } else {
            double2 cf = __ldg(coef + slot);
            double ci = CONJ ? -cf.y : cf.y;
            re = cf.x * a.p.x - ci * a.p.y;
            im = cf.x * a.p.y + ci * a.p.x;
        }
        if (parity) {
            re = -re;
            im = -im;
        }
        atomicAdd(&acc[u].x, re);
        atomicAdd(&acc[u].y, im);
    }
    __device__ __forceinline__ void visit(Acc& a, const Key<W>& c, const Key<W>& img, int parity, int64_t slot) const {
        int2 h;
        if (probe(a, c, img, parity, slot, h)) {
            record_hit(a, h);
            apply_hit(a, h);
        }
    }
    __device__ __forceinline__ void visit_diag(Acc& a, const Key<W>&, int parity, int64_t slot) const {
        if (F32) {
            comp_diag_add<CONJ>(a.fre, a.fim, __ldg(dcoef32 + slot), parity);
        } else {
            double2 cf = __ldg(dcoef + slot);
            double ci = CONJ ? -cf.y : cf.y;
            a.dre += parity ? -cf.x : cf.x;
            a.dim += parity ? -ci : ci;
        }
    }
    __device__ __forceinline__ void reduce(Acc& a) const {
        if (F32) {
            a.fre.warp_reduce();
            a.fim.warp_reduce();
        } else {
            a.dre = warp_sum(a.dre);
            a.dim = warp_sum(a.dim);
        }
    }
    __device__ __forceinline__ void finish(Acc& a, int64_t w, const Key<W>& c) const {
        const double dre = F32 ? a.fre.value() : a.dre, dim = F32 ? a.fim.value() : a.dim;
        if (!include_diag || (dre == 0.0 && dim == 0.0)) return;
        int64_t u = hash_find<W>(lookup, c);
        if (u < 0) return;
        log_diag(log, w, a.row, u, dre, dim);
        atomicAdd(&acc[u].x, dre * a.p.x - dim * a.p.y);
        atomicAdd(&acc[u].y, dre * a.p.y + dim * a.p.x);
    }
};

// Hits of a pivot-major walk: each carries its walked row, and its product
// is added at once to the output row with FP64 atomics (gather: the walked
// row, amplitude of the looked-up row; scatter: the looked-up row,
// amplitude of the walked row).  FP32 forms the products exactly in FP32
// (two-products) and converts them to FP64 for the add.
template <int W, bool CONJ, bool F32, bool SCATTER>
struct PivotHits : VisitorBase {
    static constexpr bool kStateless = true;
    HashView lookup;
    const void* val;        // amplitude per first row of the input side
    const int32_t* unique;  // walked index -> first row
    const double2* coef;
    const float4* coef32;
    double2* res;
    HitLog log;
    struct Acc {};
    __device__ __forceinline__ void record_row_hits(const int4* q, int n, int lane) const {
        if (log.hits == nullptr || n <= 0) return;
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(log.count, (unsigned long long)n);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (lane < n && base + lane < (unsigned long long)log.cap) {
            const int4 h = q[lane];
            log.hits[base + lane] = make_int4(__ldg(unique + h.z), h.y, h.x, 0);
        }
    }
    __device__ __forceinline__ bool probe_row(const Key<W>&, const Key<W>& img, int parity, int64_t slot, int64_t u,
                                              int4& h) const {
        const int64_t pos = hash_find<W>(lookup, img);
        if (pos < 0) return false;
        h = make_int4((int)slot | (parity << 31), (int)pos, (int)u, 0);
        return true;
    }
    __device__ __forceinline__ void apply_row_hit(int4 h) const {
        const int64_t slot = h.x & 0x7fffffff;
        const int64_t walked = __ldg(unique + h.z);
        const int64_t from = SCATTER ? walked : (int64_t)h.y;
        const int64_t to = SCATTER ? (int64_t)h.y : walked;
        double re, im;
        if (F32) {
            const float4 cf = __ldg(coef32 + slot);
            const float2 p = __ldg(static_cast<const float2*>(val) + from);
            const float chi = CONJ ? -cf.z : cf.z, cli = CONJ ? -cf.w : cf.w;
            float x1, e1, x2, e2;
            two_prod(cf.x, p.x, x1, e1);
            two_prod(chi, p.y, x2, e2);
            float lo = __fadd_rn(__fsub_rn(e1, e2), __fsub_rn(__fmul_rn(cf.y, p.x), __fmul_rn(cli, p.y)));
            re = ((double)x1 - (double)x2) + (double)lo;
            two_prod(cf.x, p.y, x1, e1);
            two_prod(chi, p.x, x2, e2);
            lo = __fadd_rn(__fadd_rn(e1, e2), __fadd_rn(__fmul_rn(cf.y, p.y), __fmul_rn(cli, p.x)));
            im = ((double)x1 + (double)x2) + (double)lo;
        } else {
            const double2 cf = __ldg(coef + slot);
            const double2 p = __ldg(static_cast<const double2*>(val) + from);
            const double ci = CONJ ? -cf.y : cf.y;
            re = cf.x * p.x - ci * p.y;
            im = cf.x * p.y + ci * p.x;
        }
        if (h.x < 0) {
            re = -re;
            im = -im;
        }
        atomicAdd(&res[to].x, re);
        atomicAdd(&res[to].y, im);
    }
};

// Diagonal terms of a pivot-major walk: per walked row, the sum of its
// diagonal coefficients times the amplitude of the row itself, added to the
// row's result (gather: amplitude from the input side; scatter: the walked
// amplitude, result at the output side's copy of the row).
template <int W, bool CONJ, bool F32, bool SCATTER>
struct DiagAdd : VisitorBase {
    HashView lookup;
    const void* val;
    const int32_t* unique;
    const double2* dcoef;    // FP64 path
    const float4* dcoef32;   // F32 path (hi/lo)
    double2* res;
    HitLog log;
    struct Acc {
        double dre, dim;     // FP64 path
        CompSum fre, fim;    // F32 path
    };
    __device__ __forceinline__ void init(Acc& a, int64_t, const Key<W>&, int*) const {
        a.dre = a.dim = 0.0;
        a.fre.zero();
        a.fim.zero();
    }
    __device__ __forceinline__ void visit(Acc&, const Key<W>&, const Key<W>&, int, int64_t) const {}
    __device__ __forceinline__ void visit_diag(Acc& a, const Key<W>&, int parity, int64_t slot) const {
        if (F32) {
            comp_diag_add<CONJ>(a.fre, a.fim, __ldg(dcoef32 + slot), parity);
        } else {
            const double2 cf = __ldg(dcoef + slot);
            const double ci = CONJ ? -cf.y : cf.y;
            a.dre += parity ? -cf.x : cf.x;
            a.dim += parity ? -ci : ci;
        }
    }
    __device__ __forceinline__ void reduce(Acc& a) const {
        if (F32) {
            a.fre.warp_reduce();
            a.fim.warp_reduce();
        } else {
            a.dre = warp_sum(a.dre);
            a.dim = warp_sum(a.dim);
        }
    }
    template <int L>
    __device__ __forceinline__ void reduce_lanes(Acc& a) const {
        if (F32) {
            a.fre.template group_reduce<L>();
            a.fim.template group_reduce<L>();
        } else {
#pragma unroll
            for (int d = L / 2; d > 0; d >>= 1) {
                a.dre += __shfl_xor_sync(0xffffffffu, a.dre, d);
                a.dim += __shfl_xor_sync(0xffffffffu, a.dim, d);
            }
        }
    }
    __device__ __forceinline__ void finish(Acc& a, int64_t u, const Key<W>& c) const {
        if (F32) {
            a.dre = a.fre.value();
            a.dim = a.fim.value();
        }
        if (a.dre == 0.0 && a.dim == 0.0) return;
        const int64_t pos = hash_find<W>(lookup, c);
        if (pos < 0) return;
        log_diag(log, u, __ldg(unique + u), pos, a.dre, a.dim);
        const int64_t from = SCATTER ? (int64_t)__ldg(unique + u) : pos;
        const int64_t to = SCATTER ? pos : (int64_t)__ldg(unique + u);
        double px, py;
        if (F32) {
            const float2 q = __ldg(static_cast<const float2*>(val) + from);
            px = q.x;
            py = q.y;
        } else {
            const double2 q = __ldg(static_cast<const double2*>(val) + from);
            px = q.x;
            py = q.y;
        }
        atomicAdd(&res[to].x, a.dre * px - a.dim * py);
        atomicAdd(&res[to].y, a.dre * py + a.dim * px);
    }
};

// The first 32 bytes of a hit log: written by the forward call, checked by
// the replay before it reads anything else.
struct LogHead {
    unsigned long long count;  // hits found (more than the capacity: the log is incomplete)
    int32_t dir;               // 0: walked the input side, 1: the output side, 2: nothing walked
    int32_t magic;
    int64_t n_i, n_j;          // the forward call's row counts (n_j = n_i for same_configs)
    int64_t cap;               // and its capacity in hits
};
constexpr int32_t kLogMagic = 0x51484c47;

__global__ void log_head_kernel(LogHead* h, int dir, int64_t n_i, int64_t n_j, int64_t cap) {
    h->dir = dir;
    h->magic = kLogMagic;
    h->n_i = n_i;
    h->n_j = n_j;
    h->cap = cap;
}

// Write the user's output rows from the per-first-row results: the forward
// map gives each key's value to its first row only (repeated rows get zero),
// the adjoint gives it to every row holding the key.
__global__ void apply_finalize_kernel(const double2* __restrict__ res, const int32_t* __restrict__ first, int64_t n,
                                      int every_row, double2* __restrict__ out64, float2* __restrict__ out32) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t f = __ldg(first + i);
    double2 r = make_double2(0.0, 0.0);
    if (f >= 0 && (every_row || f == i)) r = res[f];
    if (out64) out64[i] = r;
    if (out32) out32[i] = make_float2((float)r.x, (float)r.y);
}

// ---------------------------------------------------------------------------
// per-unique-key amplitudes
// ---------------------------------------------------------------------------

// Sum of the amplitudes of every row holding a key, stored at its first row
// (one exact add per row without repeats).
template <class T>
__global__ void sum_repeats_kernel(const T* __restrict__ psi, const int32_t* __restrict__ first, int64_t n,
                                   T* __restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t f = __ldg(first + i);
    if (f < 0) return;
    const T p = psi[i];
    T* o = out + f;
    atomicAdd(&o->x, p.x);
    atomicAdd(&o->y, p.y);
}

// ---------------------------------------------------------------------------
// host side: workspace layout and kernel launches
// ---------------------------------------------------------------------------

enum class Prec { F64, F32C };

struct ApplyArgs {
    const void* table_host;
    const void* table_dev;
    const uint8_t* configs_i;
    int64_t n_i;
    const uint8_t* configs_j;
    int64_t n_j;
    bool same;
    bool adjoint;
    Prec prec;
    const void* in;   // forward: psi_i (n_i); adjoint: g_j (n_j)
    double2* out64;   // forward: n_j rows; adjoint: n_i rows
    float2* out32;
    int include_diag;
    HitLog log;       // forward calls: record the hits here (hits == NULL: no record)
    LogHead* log_head;   // and the walk's direction and row counts
    int64_t log_rows;    // diagonal records the replay reads: max(n_i, n_j)
};

// Launch one enumeration over the unique rows of `walk`: the grouped kernel
// (warp per row) or the tiled kernel (thread per row), as choose_walk says.
template <int W, class V>
int launch_walk(const V& v, const HashRows& walk, const PartView& part, const PartView& diag, cudaStream_t s,
                int group = kGroupEnumerate) {
    UniqueRows<W> src{walk.keys, walk.unique};
    if (choose_walk(part, walk.n, false) == Walk::kGrouped) {
        QMBX_KERNEL(group, s, grouped_kernel<W><<<grouped_grid(walk.n), kThreads, 0, s>>>(v, src, walk.count, walk.n, part, diag));
    } else {
        if constexpr (V::kTiledDense && W <= 2) {
            QMBX_KERNEL(group, s, enumerate_dense_kernel<W><<<grid_for(walk.n, kThreads), kThreads, 0, s>>>(v, src, walk.count, walk.n, part, diag));
        } else {
            QMBX_KERNEL(group, s, enumerate_kernel<W><<<grid_for(walk.n, kThreads), kThreads, 0, s>>>(v, src, walk.count, walk.n, part, diag));
        }
    }
    QMBX_LAUNCH_CHECK("apply_within enumeration");
    return QMBX_OK;
}

// Pass over the diagonal terms of every walked row (adds into res): grouped
// or tiled, as choose_walk says.
template <int W, class D>
int launch_diag(const D& dv, const HashRows& walk, const PartView& part, const PartView& diag, cudaStream_t s,
                int group = kGroupDiagonal) {
    if (diag.n == 0) return QMBX_OK;
    UniqueRows<W> src{walk.keys, walk.unique};
    PartView none = part;
    none.n = 0;
    if (choose_walk(diag, walk.n, false) == Walk::kGrouped) {
        QMBX_KERNEL(group, s, grouped_kernel<W><<<grouped_grid(walk.n), kThreads, 0, s>>>(dv, src, walk.count, walk.n, none, diag));
    } else {
        if (diag_lanes(walk.n) == 8) {
            QMBX_KERNEL(group, s, diag_split_kernel<W, 8><<<grid_for(walk.n * 8, kThreads), kThreads, 0, s>>>(dv, src, walk.count, walk.n, diag));
        } else {
            QMBX_KERNEL(group, s, enumerate_kernel<W><<<grid_for(walk.n, kThreads), kThreads, 0, s>>>(dv, src, walk.count, walk.n, none, diag));
        }
    }
    QMBX_LAUNCH_CHECK("apply_within diagonal pass");
    return QMBX_OK;
}

// Pivot-major walk of the changing terms (results added into res by the
// visitor's flush or hits) followed by a tiled pass over the diagonal terms.
template <int W, class V, class D>
int launch_pivot(const V& v, const D& dv, const HashRows& walk, const PartView& part, const PartView& diag,
                 cudaStream_t s, int group = kGroupEnumerate, int diag_group = kGroupDiagonal) {
    UniqueRows<W> src{walk.keys, walk.unique};
    QMBX_KERNEL(group, s, pivot_kernel<W><<<pivot_grid(), kThreads, 0, s>>>(v, src, walk.count, walk.n, part));
    QMBX_LAUNCH_CHECK("apply_within pivot walk");
    return launch_diag<W>(dv, walk, part, diag, s, diag_group);
}

// Whether apply_within walks its input side (scatter) or its output side:
// the side with fewer rows, unless the sets are the same or QMBX_DETERMINISTIC
// asks for fixed-order sums.
bool apply_scatter(const ApplyArgs& a, int64_t n_in, int64_t n_out) {
    return !deterministic_mode() && !a.same && 2 * n_in < n_out;
}

// The term part a walk in direction `scatter` reads.
PartView walk_part_of(const ApplyArgs& a, bool scatter) {
    return part_view(a.table_host, a.table_dev,
                     scatter ? (a.adjoint ? QMBX_PART_ADJ : QMBX_PART_FWD) : (a.adjoint ? QMBX_PART_FWD : QMBX_PART_ADJ));
}

// The walks of apply_within over built row sets: amplitudes `val` per first
// row of the input side, results into res per first row of the output side
// (gather walks assign their rows' sums; scatter and pivot walks add, so the
// caller clears res for them).  rows_gate (device int, or NULL): the walked
// rows are the first *rows_gate of the walked set, so a launch can be made
// conditional on device state without a host round trip.
template <int W>
int walk_apply(const ApplyArgs& a, const HashRows& in_set, const HashRows& out_set, const void* val, double2* res,
               const int* rows_gate, cudaStream_t s, int group = kGroupEnumerate, int diag_group = kGroupDiagonal) {
    const int64_t n_in = a.adjoint ? a.n_j : a.n_i;
    const int64_t n_out = a.adjoint ? a.n_i : a.n_j;
    int st = QMBX_OK;
    PartView fwd = part_view(a.table_host, a.table_dev, QMBX_PART_FWD);
    PartView adj = part_view(a.table_host, a.table_dev, QMBX_PART_ADJ);
    PartView diag = part_view(a.table_host, a.table_dev, QMBX_PART_DIAG);
    const bool include_diag = a.prec == Prec::F64 || a.include_diag;
    if (!include_diag) diag.n = 0;
    const bool exact_order = deterministic_mode();
    const bool scatter = apply_scatter(a, n_in, n_out);
    // walk the input side (scatter) with forward terms for the forward map
    // or daggered terms (conjugated) for the adjoint; walk the output side
    // (gather) with daggered terms for the forward map or forward terms
    // (conjugated) for the adjoint
    const PartView& part = scatter ? (a.adjoint ? adj : fwd) : (a.adjoint ? fwd : adj);
    HashRows walk = scatter ? in_set : out_set;
    const Walk kind = choose_walk(part, walk.n, !exact_order);
    const bool pivot = kind == Walk::kPivot;
    // a gated walk takes its row count from *rows_gate (0: nothing to walk)
    if (rows_gate != nullptr) walk.count = const_cast<int*>(rows_gate);
    const HashView look = scatter ? out_set.hash() : in_set.hash();
    // the grouped kernel walks the changing terms and a tiled pass adds the
    // diagonal ones
    const bool grouped = kind == Walk::kGrouped;
    PartView walk_diag = diag;
    if (grouped) walk_diag.n = 0;
    if (pivot) {
#define QMBX_PIVOT_CASE(CONJ, F32, SCATTER)                                                                      \
    {                                                                                                            \
        PivotHits<W, CONJ, F32, SCATTER> v{{}, look, val, walk.unique, part.coef, part.coef32, res}; v.log = a.log;             \
        DiagAdd<W, CONJ, F32, SCATTER> dv{{}, look, val, walk.unique, diag.coef, diag.coef32, res}; dv.log = a.log;                           \
        st = launch_pivot<W>(v, dv, walk, part, diag, s, group, diag_group);                                                        \
    }
        const bool f32 = a.prec == Prec::F32C;
        if (scatter) {
            if (a.adjoint) {
                if (f32) QMBX_PIVOT_CASE(true, true, true) else QMBX_PIVOT_CASE(true, false, true)
            } else {
                if (f32) QMBX_PIVOT_CASE(false, true, true) else QMBX_PIVOT_CASE(false, false, true)
            }
        } else {
            if (a.adjoint) {
                if (f32) QMBX_PIVOT_CASE(true, true, false) else QMBX_PIVOT_CASE(true, false, false)
            } else {
                if (f32) QMBX_PIVOT_CASE(false, true, false) else QMBX_PIVOT_CASE(false, false, false)
            }
        }
#undef QMBX_PIVOT_CASE
    } else if (scatter) {
        if (a.prec == Prec::F64) {
            if (a.adjoint) {
                Scatter<W, true, false> v{{}, look, val, walk.unique, part.coef, part.coef32, diag.coef, diag.coef32, 1, res}; v.log = a.log;
                st = launch_walk<W>(v, walk, part, walk_diag, s, group);
            } else {
                Scatter<W, false, false> v{{}, look, val, walk.unique, part.coef, part.coef32, diag.coef, diag.coef32, 1, res}; v.log = a.log;
                st = launch_walk<W>(v, walk, part, walk_diag, s, group);
            }
        } else {
            if (a.adjoint) {
                Scatter<W, true, true> v{{}, look, val, walk.unique, part.coef, part.coef32, diag.coef, diag.coef32, include_diag, res}; v.log = a.log;
                st = launch_walk<W>(v, walk, part, walk_diag, s, group);
            } else {
                Scatter<W, false, true> v{{}, look, val, walk.unique, part.coef, part.coef32, diag.coef, diag.coef32, include_diag, res}; v.log = a.log;
                st = launch_walk<W>(v, walk, part, walk_diag, s, group);
            }
        }
    } else {
        if (a.prec == Prec::F64) {
            if (a.adjoint) {
                GatherF64<W, true> v{{}, look, (const double2*)val, part.coef, diag.coef, walk.unique, res}; v.log = a.log;
                st = launch_walk<W>(v, walk, part, walk_diag, s, group);
            } else {
                GatherF64<W, false> v{{}, look, (const double2*)val, part.coef, diag.coef, walk.unique, res}; v.log = a.log;
                st = launch_walk<W>(v, walk, part, walk_diag, s, group);
            }
        } else {
            if (a.adjoint) {
                GatherF32C<W, true> v{{}, look, (const float2*)val, part.coef32, diag.coef32, a.include_diag, walk.unique, res}; v.log = a.log;
                st = launch_walk<W>(v, walk, part, walk_diag, s, group);
            } else {
                GatherF32C<W, false> v{{}, look, (const float2*)val, part.coef32, diag.coef32, a.include_diag, walk.unique, res}; v.log = a.log;
                st = launch_walk<W>(v, walk, part, walk_diag, s, group);
            }
        }
    }
    if (st != QMBX_OK) return st;
    if (grouped && diag.n > 0) {
        const bool f32 = a.prec == Prec::F32C;
#define QMBX_DIAG_CASE(CONJ, F32, SCATTER)                                              \
    {                                                                                   \
        DiagAdd<W, CONJ, F32, SCATTER> dv{{}, look, val, walk.unique, diag.coef, diag.coef32, res}; dv.log = a.log;  \
        st = launch_diag<W>(dv, walk, part, diag, s, diag_group);                                   \
    }
        if (scatter) {
            if (a.adjoint) {
                if (f32) QMBX_DIAG_CASE(true, true, true) else QMBX_DIAG_CASE(true, false, true)
            } else {
                if (f32) QMBX_DIAG_CASE(false, true, true) else QMBX_DIAG_CASE(false, false, true)
            }
        } else {
            if (a.adjoint) {
                if (f32) QMBX_DIAG_CASE(true, true, false) else QMBX_DIAG_CASE(true, false, false)
            } else {
                if (f32) QMBX_DIAG_CASE(false, true, false) else QMBX_DIAG_CASE(false, false, false)
            }
        }
#undef QMBX_DIAG_CASE
        if (st != QMBX_OK) return st;
    }
    return QMBX_OK;
}

// Forward maps amplitudes on configs_i (input side) to configs_j (output
// side); the adjoint maps configs_j to configs_i.  Gather walks the output
// side's distinct rows (daggered terms for the forward map) and sums in
// registers; scatter walks the input side's distinct rows (forward terms
// for the forward map) and adds into the output side with FP64 atomics; the
// walk over fewer rows is taken.  Both leave one result per distinct output
// row, which apply_finalize_kernel spreads to the user's rows.
template <int W>
int apply_impl(const ApplyArgs& a, Arena& ws, cudaStream_t s) {
    const qmbx_table_header* h = header_of(a.table_host);
    const int nq = h->n_qubytes;
    HashRows rs_i = take_hashrows<W>(ws, a.n_i);
    HashRows rs_j = a.same ? rs_i : take_hashrows<W>(ws, a.n_j);
    const int64_t n_in = a.adjoint ? a.n_j : a.n_i;
    const int64_t n_out = a.adjoint ? a.n_i : a.n_j;
    const size_t val_size = a.prec == Prec::F64 ? sizeof(double2) : sizeof(float2);
    void* summed = ws.take<unsigned char>((uint64_t)(n_in > 0 ? n_in : 1) * val_size);
    double2* res = ws.take<double2>((uint64_t)(n_out > 0 ? n_out : 1));
    if (ws.base == nullptr) return QMBX_OK;
    if (!ws.fits()) {
        return fail(QMBX_ERR_WORKSPACE, "workspace of %llu bytes is smaller than the %llu needed",
                    (unsigned long long)ws.cap, (unsigned long long)ws.used);
    }
    if (a.log.hits != nullptr) {
        // an empty record until the walk below fills it (direction 2: nothing walked)
        QMBX_CUDA_TRY(cudaMemsetAsync(a.log.count, 0, sizeof(unsigned long long), s));
        QMBX_KERNEL(kGroupOther, s, log_head_kernel<<<1, 1, 0, s>>>(a.log_head, 2, a.n_i, a.n_j, a.log.cap));
    }
    if (n_out == 0) return QMBX_OK;
    int st;
    if (n_in == 0) {
        if (a.out64) QMBX_CUDA_TRY(cudaMemsetAsync(a.out64, 0, (size_t)n_out * sizeof(double2), s));
        if (a.out32) QMBX_CUDA_TRY(cudaMemsetAsync(a.out32, 0, (size_t)n_out * sizeof(float2), s));
        return QMBX_OK;
    }
    if ((st = build_hashrows<W>(a.configs_i, nq, rs_i, s)) != QMBX_OK) return st;
    if (!a.same && (st = build_hashrows<W>(a.configs_j, nq, rs_j, s)) != QMBX_OK) return st;
    const HashRows& in_set = a.adjoint ? rs_j : rs_i;
    const HashRows& out_set = a.adjoint ? rs_i : rs_j;

    // amplitude per first row of the input side: the forward map sums
    // repeated source rows; the adjoint reads the first occurrence as given
    const void* val = a.in;
    if (!a.adjoint) {
        QMBX_CUDA_TRY(cudaMemsetAsync(summed, 0, (size_t)n_in * val_size, s));
        if (a.prec == Prec::F64) {
            QMBX_KERNEL(kGroupOther, s, sum_repeats_kernel<double2><<<grid_for(n_in, kThreads), kThreads, 0, s>>>(static_cast<const double2*>(a.in), in_set.first, n_in, static_cast<double2*>(summed)));
        } else {
            QMBX_KERNEL(kGroupOther, s, sum_repeats_kernel<float2><<<grid_for(n_in, kThreads), kThreads, 0, s>>>(static_cast<const float2*>(a.in), in_set.first, n_in, static_cast<float2*>(summed)));
        }
        QMBX_LAUNCH_CHECK("sum_repeats_kernel");
        val = summed;
    }

    const bool scatter = apply_scatter(a, n_in, n_out);
    const HashRows& walked = scatter ? in_set : out_set;
    if (scatter || choose_walk(walk_part_of(a, scatter), walked.n, !deterministic_mode()) == Walk::kPivot) {
        QMBX_CUDA_TRY(cudaMemsetAsync(res, 0, (size_t)n_out * sizeof(double2), s));
    }
    if (a.log.hits != nullptr) {
        // the record of this forward call: no diagonal records yet, the walk's
        // direction (every record the replay reads, not only the walked
        // side's: the replay runs over max(n_i, n_j) of them)
        QMBX_CUDA_TRY(cudaMemsetAsync(a.log.diag_rows, 0xff, (size_t)a.log_rows * sizeof(int2), s));
        QMBX_KERNEL(kGroupOther, s, log_head_kernel<<<1, 1, 0, s>>>(a.log_head, scatter ? 0 : 1, a.n_i, a.n_j, a.log.cap));
    }
    if ((st = walk_apply<W>(a, in_set, out_set, val, res, nullptr, s)) != QMBX_OK) return st;
    QMBX_KERNEL(kGroupOther, s, apply_finalize_kernel<<<grid_for(n_out, kThreads), kThreads, 0, s>>>(res, out_set.first, n_out, a.adjoint ? 1 : 0, a.out64, a.out32));
    QMBX_LAUNCH_CHECK("apply_finalize_kernel");
    return QMBX_OK;
}

int dispatch_apply(const ApplyArgs& a, Arena& ws, cudaStream_t s) {
    switch (header_of(a.table_host)->n_words) {
        case 1: return apply_impl<1>(a, ws, s);
        case 2: return apply_impl<2>(a, ws, s);
        case 3: return apply_impl<3>(a, ws, s);
        case 4: return apply_impl<4>(a, ws, s);
        default: return fail(QMBX_ERR_ARGUMENT, "unsupported word count");
    }
}

int check_rows(const char* name, const void* p, int64_t n) {
    if (n < 0 || n >= (int64_t(1) << 31)) return fail(QMBX_ERR_ARGUMENT, "%s: row count %lld out of range", name, (long long)n);
    if (n > 0 && p == nullptr) return fail(QMBX_ERR_ARGUMENT, "%s must not be NULL", name);
    return QMBX_OK;
}

int run_apply(ApplyArgs a, void* workspace, uint64_t workspace_bytes, cudaStream_t s) {
    clear_error();
    int st = check_table(a.table_host, a.table_dev);
    if (st != QMBX_OK) return st;
    if (a.same) {
        a.configs_j = a.configs_i;
        a.n_j = a.n_i;
    }
    if ((st = check_rows("configs_i", a.configs_i, a.n_i)) != QMBX_OK) return st;
    if ((st = check_rows("configs_j", a.configs_j, a.n_j)) != QMBX_OK) return st;
    const int64_t n_in = a.adjoint ? a.n_j : a.n_i;
    const int64_t n_out = a.adjoint ? a.n_i : a.n_j;
    if ((st = check_rows("input amplitudes", a.in, n_in)) != QMBX_OK) return st;
    if (n_out > 0 && a.out64 == nullptr && a.out32 == nullptr) return fail(QMBX_ERR_ARGUMENT, "no output given");
    if (workspace == nullptr && workspace_bytes > 0) return fail(QMBX_ERR_ARGUMENT, "workspace is NULL");
    if (workspace != nullptr && reinterpret_cast<uintptr_t>(workspace) % QMBX_ALIGN != 0) {
        return fail(QMBX_ERR_ARGUMENT, "workspace must be %d-byte aligned", QMBX_ALIGN);
    }
    if (workspace == nullptr) {
        // a call with no workspace is valid only when nothing needs one
        Arena probe(nullptr, 0);
        dispatch_apply(a, probe, s);
        return fail(QMBX_ERR_WORKSPACE, "workspace of %llu bytes required", (unsigned long long)probe.used);
    }
    Arena ws(workspace, workspace_bytes);
    return dispatch_apply(a, ws, s);
}

template <int W>
int diagonal_impl(const void* table_host, const void* table_dev, const uint8_t* configs, int64_t n, double2* out,
                  cudaStream_t s) {
    const qmbx_table_header* h = header_of(table_host);
    PartView none = part_view(table_host, table_dev, QMBX_PART_DIAG);
    none.n = 0;
    PartView diag = part_view(table_host, table_dev, QMBX_PART_DIAG);
    DiagonalF64<W> v{{}, diag.coef, out};
    ByteRows<W> src{configs, h->n_qubytes};
    if (choose_walk(diag, n, false) == Walk::kGrouped) {
        QMBX_KERNEL(kGroupEnumerate, s, grouped_kernel<W><<<grouped_grid(n), kThreads, 0, s>>>(v, src, nullptr, n, none, diag));
    } else {
        QMBX_KERNEL(kGroupEnumerate, s, enumerate_kernel<W><<<grid_for(n, kThreads), kThreads, 0, s>>>(v, src, nullptr, n, none, diag));
    }
    QMBX_LAUNCH_CHECK("diagonal_term enumeration");
    return QMBX_OK;
}

}  // namespace
}  // namespace qmbx

using namespace qmbx;

namespace qmbx {

// Workspace of an apply_within call on n_i x n_j rows, for one value of
// same_configs (one row set instead of two when it is set): the largest of
// the forward / adjoint, FP64 / FP32 layouts (they differ by one value array).
int apply_within_workspace_for(const void* table_host, int64_t n_i, int64_t n_j, bool same, uint64_t* bytes) {
    const qmbx_table_header* h = header_of(table_host);
    if (h == nullptr || h->magic != QMBX_MAGIC) return fail(QMBX_ERR_ARGUMENT, "not a compiled qmbx table");
    ApplyArgs a{};
    a.table_host = table_host;
    a.n_i = n_i;
    a.n_j = same ? n_i : n_j;
    a.same = same;
    a.prec = Prec::F64;
    uint64_t most = 0;
    for (int adj = 0; adj < 2; ++adj) {
        a.adjoint = adj != 0;
        Arena probe(nullptr, 0);
        int st = dispatch_apply(a, probe, nullptr);
        if (st != QMBX_OK) return st;
        if (probe.used > most) most = probe.used;
    }
    *bytes = most;
    return QMBX_OK;
}

}  // namespace qmbx

extern "C" int qmbx_apply_within_workspace(const void* table_host, int64_t n_i, int64_t n_j, uint64_t* bytes) {
    clear_error();
    if (bytes == nullptr) return fail(QMBX_ERR_ARGUMENT, "bytes must not be NULL");
    // sized for two row sets, which also covers same_configs calls
    return apply_within_workspace_for(table_host, n_i, n_j, false, bytes);
}

extern "C" int qmbx_apply_within(const void* table_host, const void* table_dev, const uint8_t* configs_i,
                                 const double* psi_i, int64_t n_i, const uint8_t* configs_j, int64_t n_j,
                                 int32_t same_configs, double* psi_j, void* workspace, uint64_t workspace_bytes,
                                 qmbx_stream_t stream) {
    ApplyArgs a{table_host, table_dev, configs_i, n_i, configs_j, n_j, same_configs != 0, false, Prec::F64,
                psi_i, reinterpret_cast<double2*>(psi_j), nullptr, 1};
    return run_apply(a, workspace, workspace_bytes, reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int qmbx_apply_within_adjoint(const void* table_host, const void* table_dev, const uint8_t* configs_i,
                                         int64_t n_i, const uint8_t* configs_j, const double* g_j, int64_t n_j,
                                         int32_t same_configs, double* out_i, void* workspace,
                                         uint64_t workspace_bytes, qmbx_stream_t stream) {
    ApplyArgs a{table_host, table_dev, configs_i, n_i, configs_j, n_j, same_configs != 0, true, Prec::F64,
                g_j, reinterpret_cast<double2*>(out_i), nullptr, 1};
    return run_apply(a, workspace, workspace_bytes, reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int qmbx_apply_within_f32c(const void* table_host, const void* table_dev, const uint8_t* configs_i,
                                      const float* psi_i, int64_t n_i, const uint8_t* configs_j, int64_t n_j,
                                      int32_t same_configs, int32_t include_diagonal, double* out_f64, float* out_f32,
                                      void* workspace, uint64_t workspace_bytes, qmbx_stream_t stream) {
    ApplyArgs a{table_host, table_dev, configs_i, n_i, configs_j, n_j, same_configs != 0, false, Prec::F32C,
                psi_i, reinterpret_cast<double2*>(out_f64), reinterpret_cast<float2*>(out_f32), include_diagonal};
    return run_apply(a, workspace, workspace_bytes, reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int qmbx_apply_within_adjoint_f32c(const void* table_host, const void* table_dev, const uint8_t* configs_i,
                                              int64_t n_i, const uint8_t* configs_j, const float* g_j, int64_t n_j,
                                              int32_t same_configs, int32_t include_diagonal, double* out_f64,
                                              float* out_f32, void* workspace, uint64_t workspace_bytes,
                                              qmbx_stream_t stream) {
    ApplyArgs a{table_host, table_dev, configs_i, n_i, configs_j, n_j, same_configs != 0, true, Prec::F32C,
                g_j, reinterpret_cast<double2*>(out_f64), reinterpret_cast<float2*>(out_f32), include_diagonal};
    return run_apply(a, workspace, workspace_bytes, reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int qmbx_diagonal_term(const void* table_host, const void* table_dev, const uint8_t* configs, int64_t n,
                                  double* out, qmbx_stream_t stream) {
    clear_error();
    int st = check_table(table_host, table_dev);
    if (st != QMBX_OK) return st;
    if ((st = check_rows("configs", configs, n)) != QMBX_OK) return st;
    if (n > 0 && out == nullptr) return fail(QMBX_ERR_ARGUMENT, "out must not be NULL");
    if (n == 0) return QMBX_OK;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    double2* o = reinterpret_cast<double2*>(out);
    switch (header_of(table_host)->n_words) {
        case 1: return diagonal_impl<1>(table_host, table_dev, configs, n, o, s);
        case 2: return diagonal_impl<2>(table_host, table_dev, configs, n, o, s);
        case 3: return diagonal_impl<3>(table_host, table_dev, configs, n, o, s);
        case 4: return diagonal_impl<4>(table_host, table_dev, configs, n, o, s);
        default: return fail(QMBX_ERR_ARGUMENT, "unsupported word count");
    }
}

// ---------------------------------------------------------------------------
// Hit logs: a forward apply_within that records what its walk found, and the
// adjoint product computed from that record instead of a second walk.  In an
// energy-gradient step the adjoint follows the forward on the same rows (the
// backward of apply_within), and every (term, row) pair it needs is one the
// forward walk already found; replaying the record reads ~16 bytes per hit
// instead of testing every term of every walked row again.
//
// Log layout (one caller buffer, 256-byte aligned): a 256-byte header
// (LogHead: hit count, walk direction, the forward's row counts and
// capacity), configs_i's first rows (n_i int32), the
// per-walk-index diagonal records (max(n_i, n_j) int2 + double2), the
// adjoint's per-first-row sums (n_i double2), then cap hit records (int4).
// ---------------------------------------------------------------------------

namespace qmbx {
namespace {

struct LogLayout {
    uint64_t gate, diag_rows, diag_val, res, hits, ws, ws_bytes, total;
};

// Device flags of one adjoint replay, written by log_gate_kernel.
struct LogGate {
    int valid;   // the header is a logged forward's with these row counts and capacity
    int replay;  // valid and the record holds every hit: replay it
    int rows;    // valid and the record is incomplete: rows the adjoint walk takes (else 0)
    int pad;
};

// The log buffer: header, gate, diagonal records, the adjoint's per-row
// sums, cap hit records, then the forward's own workspace (its row sets,
// which the adjoint reuses).
int log_layout(const void* table_host, int64_t n_i, int64_t n_j, bool same, int64_t cap, LogLayout& L) {
    uint64_t ws_bytes = 0;
    int st = apply_within_workspace_for(table_host, n_i, same ? n_i : n_j, same, &ws_bytes);
    if (st != QMBX_OK) return st;
    if (same) n_j = n_i;
    Arena a(nullptr, 0);
    a.take<LogHead>(1);
    L.gate = a.used;
    a.take<LogGate>(1);
    const uint64_t nw = (uint64_t)(n_i > n_j ? n_i : n_j);
    L.diag_rows = a.used;
    a.take<int2>(nw > 0 ? nw : 1);
    L.diag_val = a.used;
    a.take<double2>(nw > 0 ? nw : 1);
    L.res = a.used;
    a.take<double2>((uint64_t)(n_i > 0 ? n_i : 1));
    L.hits = a.used;
    a.take<int4>((uint64_t)(cap > 0 ? cap : 1));
    L.ws = a.used;
    L.ws_bytes = ws_bytes;
    a.take<unsigned char>(ws_bytes > 0 ? ws_bytes : 1);
    L.total = a.used;
    return QMBX_OK;
}

// Point the forward's log fields into the caller's log buffer; the forward
// then runs on the workspace inside the buffer (ws, ws_bytes).
int attach_log(ApplyArgs& a, void* log, uint64_t log_bytes, int64_t cap, void** ws, uint64_t* ws_bytes) {
    if (log == nullptr || reinterpret_cast<uintptr_t>(log) % QMBX_ALIGN != 0) {
        return fail(QMBX_ERR_ARGUMENT, "log must be a %d-byte aligned device buffer", QMBX_ALIGN);
    }
    if (cap < 0) return fail(QMBX_ERR_ARGUMENT, "log capacity must not be negative");
    const int64_t n_j = a.same ? a.n_i : a.n_j;
    LogLayout L;
    int st = log_layout(a.table_host, a.n_i, n_j, a.same, cap, L);
    if (st != QMBX_OK) return st;
    if (log_bytes < L.total) {
        return fail(QMBX_ERR_WORKSPACE, "a log of %lld hits on %lld x %lld rows needs %llu bytes", (long long)cap,
                    (long long)a.n_i, (long long)n_j, (unsigned long long)L.total);
    }
    char* b = static_cast<char*>(log);
    a.log_head = reinterpret_cast<LogHead*>(b);
    a.log.count = &a.log_head->count;
    a.log.hits = reinterpret_cast<int4*>(b + L.hits);
    a.log.cap = cap;
    a.log.diag_rows = reinterpret_cast<int2*>(b + L.diag_rows);
    a.log.diag_val = reinterpret_cast<double2*>(b + L.diag_val);
    a.log_rows = a.n_i > n_j ? a.n_i : n_j;
    *ws = b + L.ws;
    *ws_bytes = L.ws_bytes;
    return QMBX_OK;
}

// Decide, on the device, how the adjoint is formed from the log: replayed
// when the header matches and the record is complete, walked (rows = the
// walked set's distinct rows) when it is incomplete, neither when the buffer
// holds no matching log (the output is then NaN).
__global__ void log_gate_kernel(const LogHead* __restrict__ h, int64_t n_i, int64_t n_j, int64_t cap,
                                const int* __restrict__ walk_rows, LogGate* __restrict__ g) {
    const bool valid = h->magic == kLogMagic && h->dir >= 0 && h->dir <= 2 && h->n_i == n_i && h->n_j == n_j &&
                       h->cap == cap;
    const bool complete = valid && h->count <= (unsigned long long)cap;
    g->valid = valid ? 1 : 0;
    g->replay = complete && h->dir != 2 ? 1 : 0;
    g->rows = valid && !complete ? *walk_rows : 0;
}

__global__ void log_poison_kernel(const LogGate* __restrict__ g, int64_t n, double2* out64, float2* out32) {
    if (g->valid) return;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (out64) out64[i] = make_double2(nan(""), nan(""));
    if (out32) out32[i] = make_float2(nanf(""), nanf(""));
}

// res[out] += conj(s * coef) * g[in] for every recorded hit: out and in are
// the walked and the looked-up rows (direction 0: the forward walked the
// input side) or the reverse (direction 1); the coefficient is read from the
// part the forward walked.  A drain of the forward writes up to 32
// consecutive records of one walked row, so when the walked rows are the
// outputs (direction 0) neighbouring lanes add into the same row: each warp
// first sums its runs of equal output rows (a segmented shuffle scan) and
// the last lane of a run adds the run's sum, one atomic pair per run instead
// of one per record.  Lanes past n take part in the scan with nothing to add.
//
// The FP32 path keeps every product and the run sums in compensated FP32
// (exact two-products, TwoSum combination of (leading, tail) pairs) and
// converts to FP64 once per run: GB300 issues FP64 arithmetic at a small
// fraction of the FP32 rate, and per-record FP64 adds and shuffles made the
// FP64 pipe this kernel's bound.
// The IEEE 754 double equal to x, formed with integer operations: a
// conversion instruction would run on the FP64 pipe, which GB300 issues at a
// small fraction of the FP32 rate and holds for tens of cycles a warp
// instruction whatever its active mask.
__device__ __forceinline__ double widen(float x) {
    const uint32_t u = __float_as_uint(x);
    const uint64_t sign = (uint64_t)(u >> 31) << 63;
    const uint32_t ex = (u >> 23) & 0xffu;
    const uint64_t mant = u & 0x7fffffu;
    uint64_t bits;
    if (ex == 0xffu) {
        bits = sign | (0x7ffull << 52) | (mant << 29);  // infinity, NaN (payload kept)
    } else if (ex != 0) {
        bits = sign | ((uint64_t)(ex + 896u) << 52) | (mant << 29);  // normal: exponent bias 127 -> 1023
    } else if (mant == 0) {
        bits = sign;  // signed zero
    } else {
        // subnormal mant * 2^-149 with leading bit p: 2^(p - 149) (1 + f), normal as a double
        const int p = 31 - __clz((unsigned)mant);
        bits = sign | ((uint64_t)(p + 874) << 52) | ((mant << (52 - p)) & ((1ull << 52) - 1));
    }
    return __longlong_as_double((long long)bits);
}

// Add a compensated FP32 sum to an FP64 value in memory: head and tail go as
// two FP64 atomics (executed in L2), so no FP64 arithmetic runs on the SM.
__device__ __forceinline__ void atomic_add_comp(double* p, const CompSum& a) {
    if (a.s != 0.f) atomicAdd(p, widen(a.s));
    if (a.c != 0.f) atomicAdd(p, widen(a.c));
}

__device__ __forceinline__ void run_add_f32(CompSum& a, float s2, float c2) {
    float e;
    two_sum(a.s, s2, a.s, e);
    a.c = __fadd_rn(a.c, __fadd_rn(c2, e));
}

template <bool F32>
__global__ void log_adjoint_kernel(const int4* __restrict__ hits, const LogHead* __restrict__ head,
                                   const LogGate* __restrict__ gate, PartView fwd, PartView adj,
                                   const void* __restrict__ g, double2* __restrict__ res) {
    if (!gate->replay) return;
    const int64_t n = (int64_t)head->count;  // <= the capacity the grid covers (gate->replay)
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if ((int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u) >= n) return;  // whole warps past n
    const int lane = threadIdx.x & 31;
    const bool live = i < n;
    const int dir = head->dir;
    const int4 h = live ? __ldg(hits + i) : make_int4(-1, -1, 0, 0);
    const int64_t slot = h.z & 0x7fffffff;
    const int out = dir == 0 ? h.x : h.y;
    const int in = dir == 0 ? h.y : h.x;
    // runs of equal `out` in lane order: run index = number of run heads up to this lane
    const unsigned full = 0xffffffffu;
    const int prev = __shfl_up_sync(full, out, 1);
    const unsigned heads = __ballot_sync(full, lane == 0 || prev != out);
    const int run = __popc(heads & (full >> (31 - lane)));
    const int next = __shfl_down_sync(full, run, 1);
    const bool last = live && (lane == 31 || next != run);
    if (F32) {
        CompSum re, im;
        re.zero();
        im.zero();
        if (live) {
            const float4 cf = __ldg((dir == 0 ? fwd.coef32 : adj.coef32) + slot);
            const float2 p = __ldg(static_cast<const float2*>(g) + in);
            // conj(c) p with c = (cf.x + cf.y) + i (cf.z + cf.w), sign (-1)^parity
            const float sg = h.z < 0 ? -1.f : 1.f;
            float x1, e1, x2, e2;
            two_prod(sg * cf.x, p.x, x1, e1);
            two_prod(sg * cf.z, p.y, x2, e2);
            float lo = __fadd_rn(__fadd_rn(e1, e2), __fadd_rn(__fmul_rn(sg * cf.y, p.x), __fmul_rn(sg * cf.w, p.y)));
            re.add2(x1, lo);
            re.add(x2);
            two_prod(sg * cf.x, p.y, x1, e1);
            two_prod(sg * cf.z, p.x, x2, e2);
            lo = __fadd_rn(__fsub_rn(e1, e2), __fsub_rn(__fmul_rn(sg * cf.y, p.y), __fmul_rn(sg * cf.w, p.x)));
            im.add2(x1, lo);
            im.add(-x2);
        }
        if (dir != 0) {
            // the walked rows were the inputs: neighbouring records add into different rows
            if (live) {
                atomic_add_comp(&res[out].x, re);
                atomic_add_comp(&res[out].y, im);
            }
            return;
        }
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const float rs = __shfl_up_sync(full, re.s, off), rc = __shfl_up_sync(full, re.c, off);
            const float is = __shfl_up_sync(full, im.s, off), ic = __shfl_up_sync(full, im.c, off);
            const int k = __shfl_up_sync(full, run, off);
            if (lane >= off && k == run) {
                run_add_f32(re, rs, rc);
                run_add_f32(im, is, ic);
            }
        }
        if (last) {
            atomic_add_comp(&res[out].x, re);
            atomic_add_comp(&res[out].y, im);
        }
    } else {
        double re = 0.0, im = 0.0;
        if (live) {
            const double2 cf = __ldg((dir == 0 ? fwd.coef : adj.coef) + slot);
            const double2 p = __ldg(static_cast<const double2*>(g) + in);
            re = cf.x * p.x + cf.y * p.y;
            im = cf.x * p.y - cf.y * p.x;
            if (h.z < 0) {
                re = -re;
                im = -im;
            }
        }
        if (dir != 0) {
            if (live) {
                atomicAdd(&res[out].x, re);
                atomicAdd(&res[out].y, im);
            }
            return;
        }
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const double r = __shfl_up_sync(full, re, off);
            const double m = __shfl_up_sync(full, im, off);
            const int k = __shfl_up_sync(full, run, off);
            if (lane >= off && k == run) {
                re += r;
                im += m;
            }
        }
        if (last) {
            atomicAdd(&res[out].x, re);
            atomicAdd(&res[out].y, im);
        }
    }
}

template <bool F32>
__global__ void log_diag_adjoint_kernel(const int2* __restrict__ rows, const double2* __restrict__ vals, int64_t n,
                                        const LogHead* __restrict__ head, const LogGate* __restrict__ gate,
                                        const void* __restrict__ g, double2* __restrict__ res) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !gate->replay) return;
    const int2 d = rows[i];
    if (d.y < 0) return;
    const int dir = head->dir;
    const int out = dir == 0 ? d.x : d.y;
    const int in = dir == 0 ? d.y : d.x;
    const double2 v = vals[i];
    double px, py;
    if (F32) {
        const float2 q = __ldg(static_cast<const float2*>(g) + in);
        px = q.x;
        py = q.y;
    } else {
        const double2 q = __ldg(static_cast<const double2*>(g) + in);
        px = q.x;
        py = q.y;
    }
    atomicAdd(&res[out].x, v.x * px + v.y * py);
    atomicAdd(&res[out].y, v.x * py - v.y * px);
}

// The adjoint product g_j -> configs_i from a logged forward's buffer, with
// no host round trip: a gate kernel reads the log's header on the device;
// a complete record is replayed, an incomplete one (more hits than its
// capacity) is replaced by the adjoint walk over the row sets the forward
// left in the buffer; a buffer that holds no matching log gives NaN.
template <int W>
int adjoint_from_log_impl(const void* table_host, const void* table_dev, char* b, const LogLayout& L, int64_t cap,
                          int64_t n_i, int64_t n_j, bool same, bool f32, int include_diag, const void* g,
                          double2* out64, float2* out32, cudaStream_t s) {
    Arena ws(b + L.ws, L.ws_bytes);
    HashRows rs_i = take_hashrows<W>(ws, n_i);
    HashRows rs_j = same ? rs_i : take_hashrows<W>(ws, n_j);
    if (!ws.fits()) return fail(QMBX_ERR_ARGUMENT, "log buffer smaller than its layout");
    const LogHead* head = reinterpret_cast<const LogHead*>(b);
    LogGate* gate = reinterpret_cast<LogGate*>(b + L.gate);
    double2* res = reinterpret_cast<double2*>(b + L.res);
    // the adjoint walk the record stands in for: its walked set's distinct rows gate it
    ApplyArgs a{table_host, table_dev, nullptr, n_i, nullptr, n_j, same, true, f32 ? Prec::F32C : Prec::F64,
                g, out64, out32, include_diag, {}, nullptr, 0};
    const bool scatter = apply_scatter(a, n_j, n_i);
    const HashRows& walked = scatter ? rs_j : rs_i;
    QMBX_CUDA_TRY(cudaMemsetAsync(res, 0, (size_t)n_i * sizeof(double2), s));
    QMBX_KERNEL(kGroupOther, s, log_gate_kernel<<<1, 1, 0, s>>>(head, n_i, n_j, cap, walked.count, gate));
    const PartView fwd = part_view(table_host, table_dev, QMBX_PART_FWD);
    const PartView adj = part_view(table_host, table_dev, QMBX_PART_ADJ);
    const int64_t nw = n_i > n_j ? n_i : n_j;
    const int4* hits = reinterpret_cast<const int4*>(b + L.hits);
    const int2* drows = reinterpret_cast<const int2*>(b + L.diag_rows);
    const double2* dvals = reinterpret_cast<const double2*>(b + L.diag_val);
    const int64_t ncap = cap > 0 ? cap : 1;
    if (f32) {
        QMBX_KERNEL(kGroupSpmv, s, log_adjoint_kernel<true><<<grid_for(ncap, kThreads), kThreads, 0, s>>>(hits, head, gate, fwd, adj, g, res));
        QMBX_KERNEL(kGroupSpmv, s, log_diag_adjoint_kernel<true><<<grid_for(nw, kThreads), kThreads, 0, s>>>(drows, dvals, nw, head, gate, g, res));
    } else {
        QMBX_KERNEL(kGroupSpmv, s, log_adjoint_kernel<false><<<grid_for(ncap, kThreads), kThreads, 0, s>>>(hits, head, gate, fwd, adj, g, res));
        QMBX_KERNEL(kGroupSpmv, s, log_diag_adjoint_kernel<false><<<grid_for(nw, kThreads), kThreads, 0, s>>>(drows, dvals, nw, head, gate, g, res));
    }
    QMBX_LAUNCH_CHECK("adjoint from log");
    // an incomplete record: the adjoint walk (its walked rows gated by the device count; 0 otherwise)
    int st = walk_apply<W>(a, rs_j, rs_i, g, res, &gate->rows, s, kGroupSpmv, kGroupSpmv);
    if (st != QMBX_OK) return st;
    QMBX_KERNEL(kGroupOther, s, apply_finalize_kernel<<<grid_for(n_i, kThreads), kThreads, 0, s>>>(res, rs_i.first, n_i, 1, out64, out32));
    QMBX_KERNEL(kGroupOther, s, log_poison_kernel<<<grid_for(n_i, kThreads), kThreads, 0, s>>>(gate, n_i, out64, out32));
    QMBX_LAUNCH_CHECK("adjoint from log");
    return QMBX_OK;
}

int adjoint_from_log(const void* table_host, const void* table_dev, const void* log, uint64_t log_bytes, int64_t cap,
                     int64_t n_i, int64_t n_j, bool same, bool f32, int include_diag, const void* g, double2* out64,
                     float2* out32, cudaStream_t s) {
    clear_error();
    int st = check_table(table_host, table_dev);
    if (st != QMBX_OK) return st;
    if (same) n_j = n_i;
    if (n_i < 0 || n_j < 0 || n_i >= (int64_t(1) << 31) || n_j >= (int64_t(1) << 31) || cap < 0) {
        return fail(QMBX_ERR_ARGUMENT, "row counts or capacity out of range");
    }
    if (log == nullptr || reinterpret_cast<uintptr_t>(log) % QMBX_ALIGN != 0) {
        return fail(QMBX_ERR_ARGUMENT, "log must be a %d-byte aligned device buffer", QMBX_ALIGN);
    }
    LogLayout L;
    if ((st = log_layout(table_host, n_i, n_j, same, cap, L)) != QMBX_OK) return st;
    if (log_bytes < L.total) return fail(QMBX_ERR_ARGUMENT, "log buffer smaller than its layout");
    if (n_i > 0 && out64 == nullptr && out32 == nullptr) return fail(QMBX_ERR_ARGUMENT, "no output given");
    if (n_j > 0 && g == nullptr) return fail(QMBX_ERR_ARGUMENT, "g_j must not be NULL");
    if (n_i == 0) return QMBX_OK;
    if (n_j == 0) {
        if (out64) QMBX_CUDA_TRY(cudaMemsetAsync(out64, 0, (size_t)n_i * sizeof(double2), s));
        if (out32) QMBX_CUDA_TRY(cudaMemsetAsync(out32, 0, (size_t)n_i * sizeof(float2), s));
        return QMBX_OK;
    }
    char* b = static_cast<char*>(const_cast<void*>(log));
    switch (header_of(table_host)->n_words) {
        case 1: return adjoint_from_log_impl<1>(table_host, table_dev, b, L, cap, n_i, n_j, same, f32, include_diag, g, out64, out32, s);
        case 2: return adjoint_from_log_impl<2>(table_host, table_dev, b, L, cap, n_i, n_j, same, f32, include_diag, g, out64, out32, s);
        case 3: return adjoint_from_log_impl<3>(table_host, table_dev, b, L, cap, n_i, n_j, same, f32, include_diag, g, out64, out32, s);
        case 4: return adjoint_from_log_impl<4>(table_host, table_dev, b, L, cap, n_i, n_j, same, f32, include_diag, g, out64, out32, s);
        default: return fail(QMBX_ERR_ARGUMENT, "unsupported word count");
    }
}

}  // namespace
}  // namespace qmbx

extern "C" int qmbx_hitlog_bytes(const void* table_host, int64_t n_i, int64_t n_j, int32_t same_configs, int64_t cap,
                                 uint64_t* bytes) {
    clear_error();
    if (bytes == nullptr) return fail(QMBX_ERR_ARGUMENT, "bytes must not be NULL");
    if (n_i < 0 || n_j < 0 || cap < 0) return fail(QMBX_ERR_ARGUMENT, "sizes must not be negative");
    const qmbx_table_header* h = header_of(table_host);
    if (h == nullptr || h->magic != QMBX_MAGIC) return fail(QMBX_ERR_ARGUMENT, "not a compiled qmbx table");
    LogLayout L;
    int st = log_layout(table_host, n_i, n_j, same_configs != 0, cap, L);
    if (st != QMBX_OK) return st;
    *bytes = L.total;
    return QMBX_OK;
}

extern "C" int qmbx_hitlog_count(const void* log, unsigned long long* count, qmbx_stream_t stream) {
    clear_error();
    if (log == nullptr || count == nullptr) return fail(QMBX_ERR_ARGUMENT, "pointers must not be NULL");
    QMBX_CUDA_TRY(cudaMemcpyAsync(count, &static_cast<const LogHead*>(log)->count, sizeof(unsigned long long),
                                  cudaMemcpyDefault, reinterpret_cast<cudaStream_t>(stream)));
    return QMBX_OK;
}

extern "C" int qmbx_apply_within_logged(const void* table_host, const void* table_dev, const uint8_t* configs_i,
                                        const double* psi_i, int64_t n_i, const uint8_t* configs_j, int64_t n_j,
                                        int32_t same_configs, double* psi_j, void* log, uint64_t log_bytes,
                                        int64_t log_cap, qmbx_stream_t stream) {
    clear_error();
    int st = check_table(table_host, table_dev);
    if (st != QMBX_OK) return st;
    ApplyArgs a{table_host, table_dev, configs_i, n_i, configs_j, n_j, same_configs != 0, false, Prec::F64,
                psi_i, reinterpret_cast<double2*>(psi_j), nullptr, 1, {}, nullptr, 0};
    void* ws = nullptr;
    uint64_t ws_bytes = 0;
    if ((st = attach_log(a, log, log_bytes, log_cap, &ws, &ws_bytes)) != QMBX_OK) return st;
    return run_apply(a, ws, ws_bytes, reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int qmbx_apply_within_f32c_logged(const void* table_host, const void* table_dev, const uint8_t* configs_i,
                                             const float* psi_i, int64_t n_i, const uint8_t* configs_j, int64_t n_j,
                                             int32_t same_configs, int32_t include_diagonal, double* out_f64,
                                             float* out_f32, void* log, uint64_t log_bytes, int64_t log_cap,
                                             qmbx_stream_t stream) {
    clear_error();
    int st = check_table(table_host, table_dev);
    if (st != QMBX_OK) return st;
    ApplyArgs a{table_host, table_dev, configs_i, n_i, configs_j, n_j, same_configs != 0, false, Prec::F32C,
                psi_i, reinterpret_cast<double2*>(out_f64), reinterpret_cast<float2*>(out_f32), include_diagonal,
                {}, nullptr, 0};
    void* ws = nullptr;
    uint64_t ws_bytes = 0;
    if ((st = attach_log(a, log, log_bytes, log_cap, &ws, &ws_bytes)) != QMBX_OK) return st;
    return run_apply(a, ws, ws_bytes, reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int qmbx_apply_within_adjoint_logged(const void* table_host, const void* table_dev, const void* log,
                                                uint64_t log_bytes, int64_t log_cap, int64_t n_i, int64_t n_j,
                                                int32_t same_configs, const double* g_j, double* out_i,
                                                qmbx_stream_t stream) {
    return adjoint_from_log(table_host, table_dev, log, log_bytes, log_cap, n_i, n_j, same_configs != 0, false, 1,
                            g_j, reinterpret_cast<double2*>(out_i), nullptr, reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int qmbx_apply_within_adjoint_f32c_logged(const void* table_host, const void* table_dev, const void* log,
                                                     uint64_t log_bytes, int64_t log_cap, int64_t n_i, int64_t n_j,
                                                     int32_t same_configs, int32_t include_diagonal,
                                                     const float* g_j, double* out_f64, float* out_f32,
                                                     qmbx_stream_t stream) {
    return adjoint_from_log(table_host, table_dev, log, log_bytes, log_cap, n_i, n_j, same_configs != 0, true,
                            include_diagonal, g_j, reinterpret_cast<double2*>(out_f64),
                            reinterpret_cast<float2*>(out_f32), reinterpret_cast<cudaStream_t>(stream));
}
