/*
 * CPU oracle for the second-quantized Hamiltonian engine.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C, the algorithms of
 * the reference engine (qmb/_hamiltonian_cpu.cpp and qmb/_hamiltonian_cuda.cu)
 * so that the CUDA path can be checked against it.  Nothing in the product
 * path may call it: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg load this library.
 *
 * Data layout (qmb/bitspack.py:8-94, qmb/_hamiltonian_cpu.cpp:36-46): a
 * configuration is a row of n_qubytes bytes; site s lives in byte s/8, bit
 * s%8 (LSB first).  Rows are ordered lexicographically by unsigned byte value,
 * byte 0 most significant (array_less, qmb/_hamiltonian_cpu.cpp:7-20).
 *
 * A term is four (site, kind) slots with kind 0 = annihilate, 1 = create,
 * 2 = empty, plus a complex coefficient (qmb/_hamiltonian.cpp:29-64).
 *
 * Parity is pinned by tests/golden fixtures produced by the reference itself.
 * Floating point: compiled with -ffp-contract=off so that every product and
 * sum is rounded once, in the order written here.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define MAX_OPS 4

static int get_bit(const uint8_t* cfg, int s) { return (cfg[s >> 3] >> (s & 7)) & 1; }

static void put_bit(uint8_t* cfg, int s, int v) {
    if (v) {
        cfg[s >> 3] = (uint8_t)(cfg[s >> 3] | (1u << (s & 7)));
    } else {
        cfg[s >> 3] = (uint8_t)(cfg[s >> 3] & ~(1u << (s & 7)));
    }
}

/*
 * Apply one term to cfg in place (qmb/_hamiltonian_cpu.cpp:48-78).  Slots are
 * applied from the last to the first; an operator fails when the bit already
 * holds the value it would write.  For fermions (particle_cut 1) the parity
 * accumulates the occupation of every site below the operator's site, read in
 * the configuration *after* the operator has acted.  Returns 1 on success.
 */
int oracle_apply_term(int n_qubytes, int particle_cut, const int16_t* site, const uint8_t* kind, uint8_t* cfg,
                      int* parity_out) {
    (void)n_qubytes;
    int parity = 0;
    for (int op = MAX_OPS - 1; op >= 0; --op) {
        int k = kind[op];
        if (k == 2) {
            continue;
        }
        int s = site[op];
        if (get_bit(cfg, s) == k) {
            *parity_out = parity;
            return 0;
        }
        put_bit(cfg, s, k);
        if (particle_cut == 1) {
            for (int b = 0; b < s; ++b) {
                parity ^= get_bit(cfg, b);
            }
        }
    }
    *parity_out = parity;
    return 1;
}

/* Lexicographic row comparison, unsigned bytes (array_less). */
static int row_cmp(const uint8_t* a, const uint8_t* b, int nq) { return memcmp(a, b, (size_t)nq); }

/* ---- stable index sort of rows (merge sort) ------------------------------ */

static void merge_sort_idx(int64_t* idx, int64_t* tmp, int64_t n, const uint8_t* rows, int nq) {
    if (n < 2) {
        return;
    }
    int64_t h = n / 2;
    merge_sort_idx(idx, tmp, h, rows, nq);
    merge_sort_idx(idx + h, tmp, n - h, rows, nq);
    int64_t a = 0, b = h, o = 0;
    while (a < h && b < n) {
        if (row_cmp(rows + idx[b] * nq, rows + idx[a] * nq, nq) < 0) {
            tmp[o++] = idx[b++];
        } else {
            tmp[o++] = idx[a++];
        }
    }
    while (a < h) {
        tmp[o++] = idx[a++];
    }
    while (b < n) {
        tmp[o++] = idx[b++];
    }
    memcpy(idx, tmp, (size_t)n * sizeof(int64_t));
}

/* Returns a malloc'ed array: stable lexicographic order of the rows. */
static int64_t* sorted_index(const uint8_t* rows, int64_t n, int nq) {
    int64_t* idx = (int64_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
    int64_t* tmp = (int64_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
    for (int64_t i = 0; i < n; ++i) {
        idx[i] = i;
    }
    merge_sort_idx(idx, tmp, n, rows, nq);
    free(tmp);
    return idx;
}

/* Leftmost position of key among sorted rows (via idx), or -1 when absent. */
static int64_t find_row(const uint8_t* rows, const int64_t* idx, int64_t n, const uint8_t* key, int nq) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t mid = lo + (hi - lo) / 2;
        if (row_cmp(rows + idx[mid] * nq, key, nq) < 0) {
            lo = mid + 1;
        } else {
            hi = mid;
        }
    }
    if (lo < n && row_cmp(rows + idx[lo] * nq, key, nq) == 0) {
        return lo;
    }
    return -1;
}

/* Stable lexicographic order of n rows into idx (the reference's sort of configs_j). */
void oracle_sort_rows(const uint8_t* rows, int64_t n, int n_qubytes, int64_t* idx) {
    int64_t* sorted = sorted_index(rows, n, n_qubytes);
    memcpy(idx, sorted, (size_t)(n > 0 ? n : 0) * sizeof(int64_t));
    free(sorted);
}

/*
 * The loop of apply_within over sources [row_begin, row_end) with configs_j
 * already sorted (idx from oracle_sort_rows): acc[pos] (complex, by sorted
 * position) accumulates sign*coef*psi for every (term, source) whose image is
 * the configs_j row at sorted position pos.  Split out so that timing runs can
 * sort once and walk slices of the sources.
 */
void oracle_apply_within_sorted(int n_qubytes, int particle_cut, int64_t n_terms, const int16_t* site,
                                const uint8_t* kind, const double* coef, int64_t row_begin, int64_t row_end,
                                const uint8_t* configs_i, const double* psi_i, int64_t n_j, const uint8_t* configs_j,
                                const int64_t* idx, double* acc) {
    int nq = n_qubytes;
    uint8_t* cur = (uint8_t*)malloc((size_t)nq);
    for (int64_t t = 0; t < n_terms; ++t) {
        for (int64_t i = row_begin; i < row_end; ++i) {
            memcpy(cur, configs_i + i * nq, (size_t)nq);
            int parity;
            if (!oracle_apply_term(nq, particle_cut, site + t * MAX_OPS, kind + t * MAX_OPS, cur, &parity)) {
                continue;
            }
            int64_t pos = find_row(configs_j, idx, n_j, cur, nq);
            if (pos < 0) {
                continue;
            }
            double sign = parity ? -1.0 : 1.0;
            const double* c = coef + 2 * t;
            const double* p = psi_i + 2 * i;
            acc[2 * pos + 0] += sign * (c[0] * p[0] - c[1] * p[1]);
            acc[2 * pos + 1] += sign * (c[0] * p[1] + c[1] * p[0]);
        }
    }
    free(cur);
}

/*
 * apply_within (qmb/_hamiltonian_cpu.cpp:80-257): term-major double loop; for
 * every (term, source) whose image lies in configs_j, out[j] += sign*coef*psi.
 * The complex product is written exactly as in :127-128.  Where configs_j holds
 * duplicate rows, the whole amplitude goes to the first of them (lowest row
 * index); the reference gives it to one of them, chosen by its unstable sort.
 */
void oracle_apply_within(int n_qubytes, int particle_cut, int64_t n_terms, const int16_t* site, const uint8_t* kind,
                         const double* coef, int64_t n_i, const uint8_t* configs_i, const double* psi_i, int64_t n_j,
                         const uint8_t* configs_j, double* psi_j) {
    int nq = n_qubytes;
    int64_t* idx = sorted_index(configs_j, n_j, nq);
    double* acc = (double*)calloc((size_t)(n_j > 0 ? n_j : 1) * 2, sizeof(double));
    oracle_apply_within_sorted(nq, particle_cut, n_terms, site, kind, coef, 0, n_i, configs_i, psi_i, n_j, configs_j,
                               idx, acc);
    memset(psi_j, 0, (size_t)n_j * 2 * sizeof(double));
    for (int64_t k = 0; k < n_j; ++k) {
        psi_j[2 * idx[k] + 0] = acc[2 * k + 0];
        psi_j[2 * idx[k] + 1] = acc[2 * k + 1];
    }
    free(acc);
    free(idx);
}

/*
 * The adjoint of apply_within (no counterpart in the reference, whose
 * vmc.py:108-110 detaches H psi): out_i[i] = sum over terms t with
 * t|i> = sign|j>, j in configs_j, of conj(sign * coef_t) * g_j[j].  The walk
 * is the forward one (qmb/_hamiltonian_cpu.cpp:80-257) read backwards: every
 * (term, row i) pair is visited once and the found target's value is pulled
 * instead of pushed.  Where configs_j repeats a row, its first occurrence
 * (lowest index) supplies the value, matching the forward map.  Rows
 * [row_begin, row_end) of configs_i are computed (out_i holds those rows), so
 * callers can split the rows across processes.
 */
void oracle_apply_within_adjoint(int n_qubytes, int particle_cut, int64_t n_terms, const int16_t* site,
                                 const uint8_t* kind, const double* coef, int64_t row_begin, int64_t row_end,
                                 const uint8_t* configs_i, int64_t n_j, const uint8_t* configs_j, const double* g_j,
                                 double* out_i) {
    int nq = n_qubytes;
    int64_t* idx = sorted_index(configs_j, n_j, nq);
    uint8_t* cur = (uint8_t*)malloc((size_t)nq);
    int64_t n = row_end - row_begin;
    memset(out_i, 0, (size_t)(n > 0 ? n : 0) * 2 * sizeof(double));
    for (int64_t t = 0; t < n_terms; ++t) {
        for (int64_t i = row_begin; i < row_end; ++i) {
            memcpy(cur, configs_i + i * nq, (size_t)nq);
            int parity;
            if (!oracle_apply_term(nq, particle_cut, site + t * MAX_OPS, kind + t * MAX_OPS, cur, &parity)) {
                continue;
            }
            int64_t pos = find_row(configs_j, idx, n_j, cur, nq);
            if (pos < 0) {
                continue;
            }
            double sign = parity ? -1.0 : 1.0;
            const double* c = coef + 2 * t;
            const double* g = g_j + 2 * idx[pos];
            /* conj(sign * c) * g */
            out_i[2 * (i - row_begin) + 0] += sign * (c[0] * g[0] + c[1] * g[1]);
            out_i[2 * (i - row_begin) + 1] += sign * (c[0] * g[1] - c[1] * g[0]);
        }
    }
    free(cur);
    free(idx);
}

/*
 * diagonal_term (qmb/_hamiltonian_cuda.cu:677-803; the reference has no CPU
 * version): sum of sign*coef over the terms that map a configuration onto
 * itself, identity terms included.
 */
void oracle_diagonal_term(int n_qubytes, int particle_cut, int64_t n_terms, const int16_t* site, const uint8_t* kind,
                          const double* coef, int64_t n, const uint8_t* configs, double* out) {
    int nq = n_qubytes;
    uint8_t* cur = (uint8_t*)malloc((size_t)nq);
    for (int64_t b = 0; b < n; ++b) {
        double re = 0.0, im = 0.0;
        for (int64_t t = 0; t < n_terms; ++t) {
            memcpy(cur, configs + b * nq, (size_t)nq);
            int parity;
            if (!oracle_apply_term(nq, particle_cut, site + t * MAX_OPS, kind + t * MAX_OPS, cur, &parity)) {
                continue;
            }
            if (row_cmp(cur, configs + b * nq, nq) != 0) {
                continue;
            }
            double sign = parity ? -1.0 : 1.0;
            re += sign * coef[2 * t + 0];
            im += sign * coef[2 * t + 1];
        }
        out[2 * b + 0] = re;
        out[2 * b + 1] = im;
    }
    free(cur);
}

/* ---- find_relative -------------------------------------------------------- */

typedef struct {
    double weight;
    uint64_t order; /* term * n_i + source: the reference's visiting order */
    uint8_t row[64];
} record_t;

/*
 * Offer one record to a size-n min-heap keyed by weight
 * (add_into_heap, qmb/_hamiltonian_cpu.cpp:259-324): a record lighter than the
 * root is dropped; otherwise it replaces the root and sinks.  The sink moves
 * toward a child that is not heavier than the record; when both qualify it
 * takes the strictly lighter one, and the right one on equal weights.
 */
static void heap_offer(record_t* heap, int64_t n, const record_t* v) {
    if (v->weight < heap[0].weight) {
        return;
    }
    int64_t pos = 0;
    for (;;) {
        int64_t l = 2 * pos + 1, r = 2 * pos + 2, next;
        if (r < n) {
            int lighter_l = v->weight < heap[l].weight;
            int lighter_r = v->weight < heap[r].weight;
            if (lighter_l && lighter_r) {
                break;
            }
            if (lighter_l) {
                next = r;
            } else if (lighter_r) {
                next = l;
            } else {
                next = heap[l].weight < heap[r].weight ? l : r;
            }
        } else if (l < n) {
            if (v->weight < heap[l].weight) {
                break;
            }
            next = l;
        } else {
            break;
        }
        heap[pos] = heap[next];
        pos = next;
    }
    heap[pos] = *v;
}

static int cmp_rows_global_nq;
static int cmp_rows_qsort(const void* a, const void* b) {
    return memcmp(a, b, (size_t)cmp_rows_global_nq);
}

/* Sort rows lexicographically and drop duplicates; returns the new count. */
static int64_t unique_rows(uint8_t* rows, int64_t n, int nq) {
    if (n == 0) {
        return 0;
    }
    cmp_rows_global_nq = nq;
    qsort(rows, (size_t)n, (size_t)nq, cmp_rows_qsort);
    int64_t u = 1;
    for (int64_t k = 1; k < n; ++k) {
        if (memcmp(rows + k * nq, rows + (u - 1) * nq, (size_t)nq) != 0) {
            memmove(rows + u * nq, rows + k * nq, (size_t)nq);
            ++u;
        }
    }
    return u;
}

/*
 * Enumerate every candidate record of find_relative in the reference's order
 * (term-major, qmb/_hamiltonian_cpu.cpp:407-440): the image of source i under
 * term t, kept when it is not an excluded row, with weight |sign*coef*psi|^2
 * computed as in :388-392.  Sources [row_begin, row_end) of configs_i are
 * walked; a record's visiting order is t * n_i + i with i its index in the
 * whole configs_i (n_i rows), so that records of row ranges walked
 * separately rank as one walk would.  Each record goes to the sink: the
 * reference's heap, a list of every record, a bounded top-K under the ranked
 * order, or a list of the records of one exact weight.
 */
typedef struct {
    record_t* list;
    int64_t count;
    int64_t cap;
} record_list_t;

typedef struct {
    record_t* heap;       /* the reference's size-heap_n min-heap (heap_offer) */
    int64_t heap_n;
    record_list_t* list;  /* every record (or, with filter, the records of weight == filter_weight) */
    int filter;
    double filter_weight;
    record_t* top;        /* bounded min-heap of the top_cap heaviest records under cmp_rank's order */
    int64_t top_cap;
    int64_t top_n;
} record_sink_t;

static void list_push(record_list_t* list, const record_t* rec) {
    if (list->count == list->cap) {
        list->cap = list->cap ? list->cap * 2 : 1024;
        list->list = (record_t*)realloc(list->list, (size_t)list->cap * sizeof(record_t));
    }
    list->list[list->count++] = *rec;
}

/* a ranks below b: lighter, or equally heavy and visited earlier */
static int rank_below(const record_t* a, const record_t* b) {
    if (a->weight != b->weight) {
        return a->weight < b->weight;
    }
    return a->order < b->order;
}

/* Keep the top_cap records that rank highest; the root is the lowest kept. */
static void top_offer(record_sink_t* s, const record_t* v) {
    if (v->weight == 0.0) {
        return; /* the reference drops records of zero weight */
    }
    record_t* h = s->top;
    int64_t pos;
    if (s->top_n < s->top_cap) {
        pos = s->top_n++;
        while (pos > 0) {
            int64_t up = (pos - 1) / 2;
            if (!rank_below(v, &h[up])) {
                break;
            }
            h[pos] = h[up];
            pos = up;
        }
        h[pos] = *v;
        return;
    }
    if (!rank_below(&h[0], v)) {
        return;
    }
    int64_t n = s->top_n;
    pos = 0;
    for (;;) {
        int64_t l = 2 * pos + 1, r = l + 1, m = pos;
        const record_t* low = v;
        if (l < n && rank_below(&h[l], low)) {
            m = l;
            low = &h[l];
        }
        if (r < n && rank_below(&h[r], low)) {
            m = r;
        }
        if (m == pos) {
            break;
        }
        h[pos] = h[m];
        pos = m;
    }
    h[pos] = *v;
}

static void enumerate_candidates(int nq, int particle_cut, int64_t n_terms, const int16_t* site, const uint8_t* kind,
                                 const double* coef, int64_t n_i, int64_t row_begin, int64_t row_end,
                                 const uint8_t* configs_i, const double* psi_i, int64_t n_ex,
                                 const uint8_t* configs_ex, record_sink_t* sink) {
    int64_t* idx = sorted_index(configs_ex, n_ex, nq);
    record_t rec;
    memset(&rec, 0, sizeof(rec));
    for (int64_t t = 0; t < n_terms; ++t) {
        for (int64_t i = row_begin; i < row_end; ++i) {
            memcpy(rec.row, configs_i + i * nq, (size_t)nq);
            int parity;
            if (!oracle_apply_term(nq, particle_cut, site + t * MAX_OPS, kind + t * MAX_OPS, rec.row, &parity)) {
                continue;
            }
            if (find_row(configs_ex, idx, n_ex, rec.row, nq) >= 0) {
                continue;
            }
            double sign = parity ? -1.0 : 1.0;
            const double* c = coef + 2 * t;
            const double* p = psi_i + 2 * i;
            double re = sign * (c[0] * p[0] - c[1] * p[1]);
            double im = sign * (c[0] * p[1] + c[1] * p[0]);
            rec.weight = re * re + im * im;
            rec.order = (uint64_t)t * (uint64_t)n_i + (uint64_t)i;
            if (sink->heap) {
                heap_offer(sink->heap, sink->heap_n, &rec);
            }
            if (sink->top) {
                top_offer(sink, &rec);
            }
            if (sink->list && (!sink->filter || rec.weight == sink->filter_weight)) {
                list_push(sink->list, &rec);
            }
        }
    }
    free(idx);
}

/*
 * find_relative with the reference's own selection (qmb/_hamiltonian_cpu.cpp
 * :442-546): a size-K heap initialised to zero records, then records of zero
 * weight are dropped and the rows are sorted and de-duplicated.  Writes at
 * most K rows to out and returns their count.  K must be positive.
 */
int64_t oracle_find_relative_heap(int n_qubytes, int particle_cut, int64_t n_terms, const int16_t* site,
                                  const uint8_t* kind, const double* coef, int64_t n_i, const uint8_t* configs_i,
                                  const double* psi_i, int64_t count_selected, int64_t n_ex, const uint8_t* configs_ex,
                                  uint8_t* out) {
    int nq = n_qubytes;
    if (count_selected <= 0) {
        return 0;
    }
    record_t* heap = (record_t*)calloc((size_t)count_selected, sizeof(record_t));
    record_sink_t sink = {heap, count_selected, NULL, 0, 0.0, NULL, 0, 0};
    enumerate_candidates(nq, particle_cut, n_terms, site, kind, coef, n_i, 0, n_i, configs_i, psi_i, n_ex, configs_ex,
                         &sink);
    int64_t m = 0;
    for (int64_t k = 0; k < count_selected; ++k) {
        if (heap[k].weight != 0.0) {
            memcpy(out + m * nq, heap[k].row, (size_t)nq);
            ++m;
        }
    }
    free(heap);
    return unique_rows(out, m, nq);
}

/* Heavier first; among equal weights the later record (larger order) first. */
static int cmp_rank(const void* a, const void* b) {
    const record_t* x = (const record_t*)a;
    const record_t* y = (const record_t*)b;
    if (x->weight != y->weight) {
        return x->weight > y->weight ? -1 : 1;
    }
    if (x->order != y->order) {
        return x->order > y->order ? -1 : 1;
    }
    return 0;
}

/*
 * find_relative with a total order in place of the heap: records of non-zero
 * weight ranked by (weight descending, visiting order descending), the first
 * K kept, rows sorted and de-duplicated.  This is the selection rule of the
 * CUDA path.  It differs from the heap only in which records of weight equal
 * to the K-th weight survive.  info (may be NULL) receives
 * [K-th weight, records heavier than it, records equal to it, all records].
 */
int64_t oracle_find_relative_ranked(int n_qubytes, int particle_cut, int64_t n_terms, const int16_t* site,
                                    const uint8_t* kind, const double* coef, int64_t n_i, const uint8_t* configs_i,
                                    const double* psi_i, int64_t count_selected, int64_t n_ex,
                                    const uint8_t* configs_ex, uint8_t* out, double* info) {
    int nq = n_qubytes;
    record_list_t list = {NULL, 0, 0};
    record_sink_t sink = {NULL, 0, &list, 0, 0.0, NULL, 0, 0};
    enumerate_candidates(nq, particle_cut, n_terms, site, kind, coef, n_i, 0, n_i, configs_i, psi_i, n_ex, configs_ex,
                         &sink);
    int64_t nz = 0;
    for (int64_t k = 0; k < list.count; ++k) {
        if (list.list[k].weight != 0.0) {
            list.list[nz++] = list.list[k];
        }
    }
    if (nz > 0) {
        qsort(list.list, (size_t)nz, sizeof(record_t), cmp_rank);
    }
    int64_t keep = count_selected < nz ? count_selected : nz;
    if (keep < 0) {
        keep = 0;
    }
    if (info) {
        double wk = keep > 0 ? list.list[keep - 1].weight : 0.0;
        int64_t above = 0, equal = 0;
        for (int64_t k = 0; k < nz; ++k) {
            if (list.list[k].weight > wk) {
                ++above;
            } else if (list.list[k].weight == wk) {
                ++equal;
            }
        }
        info[0] = wk;
        info[1] = (double)above;
        info[2] = (double)equal;
        info[3] = (double)nz;
    }
    for (int64_t k = 0; k < keep; ++k) {
        memcpy(out + k * nq, list.list[k].row, (size_t)nq);
    }
    free(list.list);
    return unique_rows(out, keep, nq);
}

/*
 * The top_cap records of sources [row_begin, row_end) under the ranked order
 * of oracle_find_relative_ranked (weight descending, visiting order
 * descending, zero weights dropped), with visiting orders of the whole
 * configs_i (n_i rows).  Because the order is total, the top K of a union of
 * row ranges is the top K of the union of their top-K lists: callers split
 * the rows across processes and merge.  Writes weights, orders and rows (in
 * no particular order) and returns the count.
 */
int64_t oracle_relative_top_records(int n_qubytes, int particle_cut, int64_t n_terms, const int16_t* site,
                                    const uint8_t* kind, const double* coef, int64_t n_i, int64_t row_begin,
                                    int64_t row_end, const uint8_t* configs_i, const double* psi_i, int64_t top_cap,
                                    int64_t n_ex, const uint8_t* configs_ex, double* weights, uint64_t* orders,
                                    uint8_t* rows) {
    int nq = n_qubytes;
    if (top_cap <= 0) {
        return 0;
    }
    record_t* top = (record_t*)malloc((size_t)top_cap * sizeof(record_t));
    record_sink_t sink = {NULL, 0, NULL, 0, 0.0, top, top_cap, 0};
    enumerate_candidates(nq, particle_cut, n_terms, site, kind, coef, n_i, row_begin, row_end, configs_i, psi_i, n_ex,
                         configs_ex, &sink);
    for (int64_t k = 0; k < sink.top_n; ++k) {
        weights[k] = top[k].weight;
        orders[k] = top[k].order;
        memcpy(rows + k * nq, top[k].row, (size_t)nq);
    }
    free(top);
    return sink.top_n;
}

/*
 * Rows of every candidate whose weight is exactly w (used by the tests to
 * name the boundary-tie class).  Writes up to cap rows, returns the count of
 * distinct rows found.
 */
int64_t oracle_rows_with_weight(int n_qubytes, int particle_cut, int64_t n_terms, const int16_t* site,
                                const uint8_t* kind, const double* coef, int64_t n_i, const uint8_t* configs_i,
                                const double* psi_i, int64_t n_ex, const uint8_t* configs_ex, double w, int64_t cap,
                                uint8_t* out) {
    int nq = n_qubytes;
    record_list_t list = {NULL, 0, 0};
    record_sink_t sink = {NULL, 0, &list, 1, w, NULL, 0, 0};
    enumerate_candidates(nq, particle_cut, n_terms, site, kind, coef, n_i, 0, n_i, configs_i, psi_i, n_ex, configs_ex,
                         &sink);
    uint8_t* rows = (uint8_t*)malloc((size_t)(list.count > 0 ? list.count : 1) * (size_t)nq);
    int64_t m = 0;
    for (int64_t k = 0; k < list.count; ++k) {
        memcpy(rows + m * nq, list.list[k].row, (size_t)nq);
        ++m;
    }
    int64_t u = unique_rows(rows, m, nq);
    memcpy(out, rows, (size_t)(u < cap ? u : cap) * (size_t)nq);
    free(rows);
    free(list.list);
    return u;
}

/* ---- single_relative ---------------------------------------------------- */

/* SplitMix64 finaliser (Steele, Lea and Flood, OOPSLA 2014). */
static uint64_t splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* The per-term uniform variate in (0, 1] that the CUDA path draws. */
double oracle_term_uniform(uint64_t seed, int64_t term) {
    uint64_t bits = splitmix64(seed ^ splitmix64((uint64_t)term));
    return (double)((bits >> 11) + 1) * (1.0 / 9007199254740992.0);
}

/*
 * single_relative (qmb/_hamiltonian_cuda.cu:805-996): for every configuration,
 * among the terms that map it to a row outside the input set, pick one by
 * Efraimidis-Spirakis sampling with weight |coef|: maximise log(u_t)/|coef_t|
 * (the logarithm of the reference's u^(1/w) key), u_t shared by all rows as
 * in :857.  Ties go to the lowest term index; rows with no candidate are all
 * zero (:966).  keys (may be NULL) receives the winning key, -inf when none.
 */
void oracle_single_relative(int n_qubytes, int particle_cut, int64_t n_terms, const int16_t* site,
                            const uint8_t* kind, const double* coef, int64_t n, const uint8_t* configs, uint64_t seed,
                            uint8_t* out, double* keys, int64_t* terms) {
    int nq = n_qubytes;
    int64_t* idx = sorted_index(configs, n, nq);
    uint8_t* cur = (uint8_t*)malloc((size_t)nq);
    double* kf = (double*)malloc((size_t)(n_terms > 0 ? n_terms : 1) * sizeof(double));
    for (int64_t t = 0; t < n_terms; ++t) {
        double w = sqrt(coef[2 * t] * coef[2 * t] + coef[2 * t + 1] * coef[2 * t + 1]);
        kf[t] = w > 0.0 ? log(oracle_term_uniform(seed, t)) / w : -INFINITY;
    }
    for (int64_t b = 0; b < n; ++b) {
        int64_t best = -1;
        double best_key = -INFINITY;
        memset(out + b * nq, 0, (size_t)nq);
        for (int64_t t = 0; t < n_terms; ++t) {
            memcpy(cur, configs + b * nq, (size_t)nq);
            int parity;
            if (!oracle_apply_term(nq, particle_cut, site + t * MAX_OPS, kind + t * MAX_OPS, cur, &parity)) {
                continue;
            }
            if (find_row(configs, idx, n, cur, nq) >= 0) {
                continue;
            }
            if (best < 0 || kf[t] > best_key) {
                best = t;
                best_key = kf[t];
                memcpy(out + b * nq, cur, (size_t)nq);
            }
        }
        if (keys) {
            keys[b] = best_key;
        }
        if (terms) {
            terms[b] = best;
        }
    }
    free(kf);
    free(cur);
    free(idx);
}

/*
 * Columns [col_begin, col_end) of the dense matrix below: mat[j][i - col_begin]
 * = <j|H|i> for every row j of configs, n x (col_end - col_begin) complex,
 * row-major.  Callers split the columns across processes.
 */
void oracle_dense_columns(int n_qubytes, int particle_cut, int64_t n_terms, const int16_t* site, const uint8_t* kind,
                          const double* coef, int64_t n, const uint8_t* configs, int64_t col_begin, int64_t col_end,
                          double* mat) {
    int nq = n_qubytes;
    int64_t w = col_end - col_begin;
    int64_t* idx = sorted_index(configs, n, nq);
    uint8_t* cur = (uint8_t*)malloc((size_t)nq);
    memset(mat, 0, (size_t)n * (size_t)(w > 0 ? w : 0) * 2 * sizeof(double));
    for (int64_t t = 0; t < n_terms; ++t) {
        for (int64_t i = col_begin; i < col_end; ++i) {
            memcpy(cur, configs + i * nq, (size_t)nq);
            int parity;
            if (!oracle_apply_term(nq, particle_cut, site + t * MAX_OPS, kind + t * MAX_OPS, cur, &parity)) {
                continue;
            }
            int64_t pos = find_row(configs, idx, n, cur, nq);
            if (pos < 0) {
                continue;
            }
            int64_t j = idx[pos];
            double sign = parity ? -1.0 : 1.0;
            mat[2 * (j * w + (i - col_begin)) + 0] += sign * coef[2 * t + 0];
            mat[2 * (j * w + (i - col_begin)) + 1] += sign * coef[2 * t + 1];
        }
    }
    free(cur);
    free(idx);
}

/*
 * Dense matrix H[j][i] = <j|H|i> over one list of configurations (for the
 * gradient checks).  mat is n*n complex, row-major.
 */
void oracle_dense_matrix(int n_qubytes, int particle_cut, int64_t n_terms, const int16_t* site, const uint8_t* kind,
                         const double* coef, int64_t n, const uint8_t* configs, double* mat) {
    int nq = n_qubytes;
    int64_t* idx = sorted_index(configs, n, nq);
    uint8_t* cur = (uint8_t*)malloc((size_t)nq);
    memset(mat, 0, (size_t)n * (size_t)n * 2 * sizeof(double));
    for (int64_t t = 0; t < n_terms; ++t) {
        for (int64_t i = 0; i < n; ++i) {
            memcpy(cur, configs + i * nq, (size_t)nq);
            int parity;
            if (!oracle_apply_term(nq, particle_cut, site + t * MAX_OPS, kind + t * MAX_OPS, cur, &parity)) {
                continue;
            }
            int64_t pos = find_row(configs, idx, n, cur, nq);
            if (pos < 0) {
                continue;
            }
            int64_t j = idx[pos];
            double sign = parity ? -1.0 : 1.0;
            mat[2 * (j * n + i) + 0] += sign * coef[2 * t + 0];
            mat[2 * (j * n + i) + 1] += sign * coef[2 * t + 1];
        }
    }
    free(cur);
    free(idx);
}
