// Host-side term compiler and error plumbing of the qmbx C ABI.
//
// qmbx_table_build replaces the per-call, per-thread decoding of
// (site, kind) slots that the reference performs inside every kernel thread
// (qmb/_hamiltonian_cuda.cu:54-84) with a one-off compilation into bit masks
// (see format.h for the closed form).
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "../../include/qmbx.h"
#include "common.h"
#include "format.h"

namespace qmbx {

static thread_local std::string g_last_error;

int fail(int status, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

void clear_error() { g_last_error.clear(); }

namespace {

struct Compiled {
    bool live = true;
    uint64_t mask[QMBX_MAX_WORDS] = {0, 0, 0, 0};
    uint64_t val[QMBX_MAX_WORDS] = {0, 0, 0, 0};
    uint64_t flip[QMBX_MAX_WORDS] = {0, 0, 0, 0};
    uint64_t par[QMBX_MAX_WORDS] = {0, 0, 0, 0};
    int pconst = 0;
    bool diagonal() const { return (flip[0] | flip[1] | flip[2] | flip[3]) == 0; }
};

struct Below {
    // below[s] = key-space mask of every site < s
    std::vector<uint64_t> m;
    int words;
    Below(int n_sites, int w) : m((size_t)(n_sites + 1) * QMBX_MAX_WORDS, 0), words(w) {
        for (int s = 1; s <= n_sites; ++s) {
            uint64_t* row = &m[(size_t)s * QMBX_MAX_WORDS];
            const uint64_t* prev = &m[(size_t)(s - 1) * QMBX_MAX_WORDS];
            for (int k = 0; k < QMBX_MAX_WORDS; ++k) row[k] = prev[k];
            row[qmbx_keyword(s - 1)] |= 1ull << qmbx_keybit(s - 1);
        }
    }
    const uint64_t* of(int s) const { return &m[(size_t)s * QMBX_MAX_WORDS]; }
};

int parity64(uint64_t x) { return __builtin_popcountll(x) & 1; }

// Replay the slots from the last to the first (qmb/_hamiltonian_cpu.cpp:59-76)
// symbolically.  adjoint = true compiles the daggered term: slots in reverse
// order with create and annihilate exchanged.
Compiled compile_term(const int16_t* site, const uint8_t* kind, bool fermi, bool adjoint, const Below& below) {
    Compiled c;
    uint64_t known[QMBX_MAX_WORDS] = {0, 0, 0, 0};
    uint64_t now[QMBX_MAX_WORDS] = {0, 0, 0, 0};  // current value of known sites
    for (int step = 0; step < 4; ++step) {
        int slot = adjoint ? step : 3 - step;
        int k = kind[slot];
        if (k == 2) continue;
        if (adjoint) k = 1 - k;
        int s = site[slot];
        int w = qmbx_keyword(s);
        uint64_t bit = 1ull << qmbx_keybit(s);
        if (!(known[w] & bit)) {
            known[w] |= bit;
            c.mask[w] |= bit;
            if (k == 0) {  // annihilation needs the site occupied
                c.val[w] |= bit;
                now[w] |= bit;
            }
        }
        int current = (now[w] & bit) ? 1 : 0;
        if (current == k) {
            c.live = false;
            return c;
        }
        now[w] ^= bit;
        c.flip[w] ^= bit;
        if (fermi) {
            const uint64_t* b = below.of(s);
            for (int q = 0; q < QMBX_MAX_WORDS; ++q) {
                c.par[q] ^= b[q];
                c.pconst ^= parity64(c.flip[q] & b[q]);
            }
        }
    }
    return c;
}

uint64_t align_up(uint64_t x) { return (x + QMBX_ALIGN - 1) / QMBX_ALIGN * QMBX_ALIGN; }

int validate(const int16_t* site, const uint8_t* kind, int64_t n_terms, int32_t n_qubytes, int32_t particle_cut) {
    if (n_qubytes < 1 || n_qubytes > 8 * QMBX_MAX_WORDS) {
        return fail(QMBX_ERR_ARGUMENT, "n_qubytes must be in [1, %d], got %d", 8 * QMBX_MAX_WORDS, n_qubytes);
    }
    if (particle_cut != 1 && particle_cut != 2) {
        return fail(QMBX_ERR_ARGUMENT, "particle_cut must be 1 (fermi) or 2 (bose2), got %d", particle_cut);
    }
    if (n_terms < 0 || n_terms >= (int64_t(1) << 31)) {
        return fail(QMBX_ERR_ARGUMENT, "term count out of range: %lld", (long long)n_terms);
    }
    if (n_terms > 0 && (site == nullptr || kind == nullptr)) {
        return fail(QMBX_ERR_ARGUMENT, "site and kind must not be NULL");
    }
    int n_sites = 8 * n_qubytes;
    for (int64_t t = 0; t < n_terms; ++t) {
        for (int k = 0; k < 4; ++k) {
            int kd = kind[t * 4 + k];
            if (kd > 2) {
                return fail(QMBX_ERR_ARGUMENT, "term %lld slot %d: kind must be 0, 1 or 2, got %d", (long long)t, k, kd);
            }
            if (kd != 2) {
                int s = site[t * 4 + k];
                if (s < 0 || s >= n_sites) {
                    return fail(QMBX_ERR_ARGUMENT, "term %lld slot %d: site %d outside [0, %d)", (long long)t, k, s,
                                n_sites);
                }
            }
        }
    }
    return QMBX_OK;
}

struct Layout {
    qmbx_table_header h;
};

void layout_part(qmbx_table_part& p, int64_t n, int words, bool narrow, uint64_t& cursor) {
    p.n = n;
    p.n_groups = qmbx_group_count(words);
    uint64_t un = (uint64_t)n;
    p.off_test = cursor;
    cursor = align_up(cursor + un * 2 * words * 8);
    p.off_apply = cursor;
    cursor = align_up(cursor + un * 2 * words * 8);
    p.off_coef = cursor;
    cursor = align_up(cursor + un * 16);
    p.off_coef32 = cursor;
    cursor = align_up(cursor + un * 16);
    p.off_orig = cursor;
    cursor = align_up(cursor + un * 4);
    p.off_norm = cursor;
    cursor = align_up(cursor + un * 4);
    p.off_groups = cursor;
    cursor = align_up(cursor + (uint64_t)p.n_groups * 8);
    p.off_single_ne = cursor;
    cursor = align_up(cursor + (uint64_t)words * 8);
    p.off_pair_ne = cursor;
    cursor = align_up(cursor + (uint64_t)64 * words * words * 8);
    p.off_nonempty = cursor;
    cursor = align_up(cursor + (uint64_t)p.n_groups * 16);
    p.off_narrow = 0;
    if (narrow) {
        p.off_narrow = cursor;
        cursor = align_up(cursor + un * 16);
    }
}

// Pivot group of a compiled term (see format.h).
int64_t group_of(const Compiled& c, int words) {
    int first = -1, second = -1;
    for (int w = 0; w < words && second < 0; ++w) {
        uint64_t req = c.mask[w] & c.val[w];
        while (req && second < 0) {
            int b = __builtin_ctzll(req);
            req &= req - 1;
            int kp = 64 * w + b;
            if (first < 0) {
                first = kp;
            } else {
                second = kp;
            }
        }
    }
    if (second >= 0) return qmbx_pair_group(words, first, second);
    if (first >= 0) return qmbx_single_group(first);
    return 0;
}

// Counting sort of one part's terms by group: fills groups[g] = [start, end),
// the non-empty masks and the per-term destination slot.
void group_part(char* blob, qmbx_table_part& p, int words, const std::vector<int64_t>& gid,
                std::vector<int64_t>& dest) {
    const int64_t G = p.n_groups;
    std::vector<int64_t> count((size_t)G + 1, 0);
    for (int64_t g : gid) ++count[(size_t)g + 1];
    for (int64_t g = 0; g < G; ++g) count[(size_t)g + 1] += count[(size_t)g];
    int32_t* groups = reinterpret_cast<int32_t*>(blob + p.off_groups);
    uint64_t* single_ne = reinterpret_cast<uint64_t*>(blob + p.off_single_ne);
    uint64_t* pair_ne = reinterpret_cast<uint64_t*>(blob + p.off_pair_ne);
    int32_t* listed = reinterpret_cast<int32_t*>(blob + p.off_nonempty);
    int64_t nonempty = 0;
    const int P = 64 * words;
    for (int64_t g = 0; g < G; ++g) {
        groups[2 * g + 0] = (int32_t)count[(size_t)g];
        groups[2 * g + 1] = (int32_t)count[(size_t)g + 1];
        if (count[(size_t)g + 1] == count[(size_t)g]) continue;
        int pivot_p = -1, pivot_q = -1;
        if (g >= 1 && g <= P) {
            int kp = (int)(g - 1);
            single_ne[kp >> 6] |= 1ull << (kp & 63);
            pivot_p = kp;
        } else if (g > P) {
            int64_t r = g - 1 - P;  // q(q-1)/2 + p
            int q = 1;
            while ((int64_t)(q + 1) * q / 2 <= r) ++q;
            int pp = (int)(r - (int64_t)q * (q - 1) / 2);
            pair_ne[(size_t)pp * words + (q >> 6)] |= 1ull << (q & 63);
            pivot_p = pp;
            pivot_q = q;
        }
        int32_t* row = listed + 4 * nonempty;
        row[0] = (int32_t)count[(size_t)g];
        row[1] = (int32_t)count[(size_t)g + 1];
        row[2] = pivot_p;
        row[3] = pivot_q;
        ++nonempty;
    }
    p.n_nonempty = nonempty;
    p.wide_groups = (nonempty > 0 && p.n >= 8 * nonempty) ? 1 : 0;
    dest.resize(gid.size());
    std::vector<int64_t> cursor(count.begin(), count.end() - 1);
    for (size_t k = 0; k < gid.size(); ++k) dest[k] = cursor[(size_t)gid[k]]++;
}

qmbx_table_header make_header(int64_t n_terms, int32_t n_qubytes, int32_t particle_cut, int64_t n_off, int64_t n_diag) {
    qmbx_table_header h;
    std::memset(&h, 0, sizeof(h));
    h.magic = QMBX_MAGIC;
    h.version = QMBX_TABLE_VERSION;
    h.n_qubytes = n_qubytes;
    h.particle_cut = particle_cut;
    h.n_words = (n_qubytes + 7) / 8;
    h.n_sites = 8 * n_qubytes;
    h.n_terms = n_terms;
    h.n_live = n_off + n_diag;
    uint64_t cursor = align_up(sizeof(qmbx_table_header));
    const bool narrow = h.n_sites <= 32;  // every mask in the high half of key word 0
    layout_part(h.part[QMBX_PART_FWD], n_off, h.n_words, narrow, cursor);
    layout_part(h.part[QMBX_PART_ADJ], n_off, h.n_words, narrow, cursor);
    layout_part(h.part[QMBX_PART_DIAG], n_diag, h.n_words, narrow, cursor);
    h.total_bytes = cursor;
    return h;
}

void count_terms(const int16_t* site, const uint8_t* kind, int64_t n_terms, int32_t n_qubytes, int32_t particle_cut,
                 int64_t& n_off, int64_t& n_diag) {
    Below below(8 * n_qubytes, (n_qubytes + 7) / 8);
    n_off = n_diag = 0;
    for (int64_t t = 0; t < n_terms; ++t) {
        Compiled c = compile_term(site + 4 * t, kind + 4 * t, particle_cut == 1, false, below);
        if (!c.live) continue;
        if (c.diagonal()) {
            ++n_diag;
        } else {
            ++n_off;
        }
    }
}

void write_term(char* blob, const qmbx_table_part& p, int words, int64_t slot, const Compiled& c, const double* coef,
                int64_t orig) {
    uint64_t* test = reinterpret_cast<uint64_t*>(blob + p.off_test);
    uint64_t* apply = reinterpret_cast<uint64_t*>(blob + p.off_apply);
    for (int w = 0; w < words; ++w) {
        const uint64_t at = ((uint64_t)w * (uint64_t)p.n + (uint64_t)slot) * 2;
        test[at] = c.mask[w];
        test[at + 1] = c.val[w];
        apply[at] = c.flip[w];
        apply[at + 1] = c.par[w];
    }
    double re = coef[0], im = coef[1];
    if (c.pconst) {
        re = -re;
        im = -im;
    }
    double* cf = reinterpret_cast<double*>(blob + p.off_coef) + slot * 2;
    cf[0] = re;
    cf[1] = im;
    float* c32 = reinterpret_cast<float*>(blob + p.off_coef32) + slot * 4;
    float re_hi = (float)re, im_hi = (float)im;
    c32[0] = re_hi;
    c32[1] = (float)(re - (double)re_hi);
    c32[2] = im_hi;
    c32[3] = (float)(im - (double)im_hi);
    reinterpret_cast<int32_t*>(blob + p.off_orig)[slot] = (int32_t)orig;
    reinterpret_cast<float*>(blob + p.off_norm)[slot] = (float)(re * re + im * im);
    if (p.off_narrow != 0) {
        uint32_t* nr = reinterpret_cast<uint32_t*>(blob + p.off_narrow) + slot * 4;
        nr[0] = (uint32_t)(c.mask[0] >> 32);
        nr[1] = (uint32_t)(c.val[0] >> 32);
        nr[2] = (uint32_t)(c.flip[0] >> 32);
        nr[3] = (uint32_t)(c.par[0] >> 32);
    }
}

}  // namespace
}  // namespace qmbx

using namespace qmbx;

extern "C" int qmbx_version(void) { return 10001; }

extern "C" const char* qmbx_last_error(void) { return g_last_error.c_str(); }

extern "C" int qmbx_table_bytes(const int16_t* site, const uint8_t* kind, int64_t n_terms, int32_t n_qubytes,
                                int32_t particle_cut, uint64_t* bytes) {
    clear_error();
    if (bytes == nullptr) return fail(QMBX_ERR_ARGUMENT, "bytes must not be NULL");
    int st = validate(site, kind, n_terms, n_qubytes, particle_cut);
    if (st != QMBX_OK) return st;
    int64_t n_off, n_diag;
    count_terms(site, kind, n_terms, n_qubytes, particle_cut, n_off, n_diag);
    *bytes = make_header(n_terms, n_qubytes, particle_cut, n_off, n_diag).total_bytes;
    return QMBX_OK;
}

extern "C" int qmbx_table_build(const int16_t* site, const uint8_t* kind, const double* coef, int64_t n_terms,
                                int32_t n_qubytes, int32_t particle_cut, void* blob, uint64_t blob_bytes) {
    clear_error();
    int st = validate(site, kind, n_terms, n_qubytes, particle_cut);
    if (st != QMBX_OK) return st;
    if (n_terms > 0 && coef == nullptr) return fail(QMBX_ERR_ARGUMENT, "coef must not be NULL");
    if (blob == nullptr) return fail(QMBX_ERR_ARGUMENT, "blob must not be NULL");
    int64_t n_off, n_diag;
    count_terms(site, kind, n_terms, n_qubytes, particle_cut, n_off, n_diag);
    qmbx_table_header h = make_header(n_terms, n_qubytes, particle_cut, n_off, n_diag);
    if (blob_bytes < h.total_bytes) {
        return fail(QMBX_ERR_ARGUMENT, "table blob holds %llu bytes, needs %llu", (unsigned long long)blob_bytes,
                    (unsigned long long)h.total_bytes);
    }
    char* out = static_cast<char*>(blob);
    std::memset(out, 0, h.total_bytes);
    Below below(h.n_sites, h.n_words);
    bool fermi = particle_cut == 1;
    const int words = h.n_words;
    // pass 1: group of every live term in each part
    std::vector<int64_t> gid[QMBX_PARTS];
    for (int64_t t = 0; t < n_terms; ++t) {
        Compiled c = compile_term(site + 4 * t, kind + 4 * t, fermi, false, below);
        if (!c.live) continue;
        if (c.diagonal()) {
            gid[QMBX_PART_DIAG].push_back(group_of(c, words));
        } else {
            gid[QMBX_PART_FWD].push_back(group_of(c, words));
            Compiled a = compile_term(site + 4 * t, kind + 4 * t, fermi, true, below);
            gid[QMBX_PART_ADJ].push_back(group_of(a, words));
        }
    }
    std::vector<int64_t> dest[QMBX_PARTS];
    for (int part = 0; part < QMBX_PARTS; ++part) group_part(out, h.part[part], words, gid[part], dest[part]);
    // pass 2: write every term at its grouped position
    int64_t k_off = 0, k_diag = 0;
    for (int64_t t = 0; t < n_terms; ++t) {
        Compiled c = compile_term(site + 4 * t, kind + 4 * t, fermi, false, below);
        if (!c.live) continue;
        if (c.diagonal()) {
            write_term(out, h.part[QMBX_PART_DIAG], words, dest[QMBX_PART_DIAG][(size_t)k_diag++], c, coef + 2 * t, t);
        } else {
            write_term(out, h.part[QMBX_PART_FWD], words, dest[QMBX_PART_FWD][(size_t)k_off], c, coef + 2 * t, t);
            Compiled a = compile_term(site + 4 * t, kind + 4 * t, fermi, true, below);
            write_term(out, h.part[QMBX_PART_ADJ], words, dest[QMBX_PART_ADJ][(size_t)k_off], a, coef + 2 * t, t);
            ++k_off;
        }
    }
    std::memcpy(out, &h, sizeof(h));
    return QMBX_OK;
}

extern "C" int qmbx_table_check(const void* blob, uint64_t blob_bytes) {
    clear_error();
    const qmbx_table_header* h = static_cast<const qmbx_table_header*>(blob);
    if (h == nullptr || blob_bytes < sizeof(qmbx_table_header)) return fail(QMBX_ERR_ARGUMENT, "blob too short for a table");
    if (h->magic != QMBX_MAGIC) return fail(QMBX_ERR_ARGUMENT, "not a compiled qmbx table");
    if (h->version != QMBX_TABLE_VERSION) {
        return fail(QMBX_ERR_ARGUMENT, "table format %u, this library reads %u", h->version, QMBX_TABLE_VERSION);
    }
    if (h->total_bytes != blob_bytes) {
        return fail(QMBX_ERR_ARGUMENT, "table of %llu bytes in a blob of %llu", (unsigned long long)h->total_bytes,
                    (unsigned long long)blob_bytes);
    }
    return QMBX_OK;
}

extern "C" int qmbx_table_counts(const void* table_host, int64_t counts[6]) {
    clear_error();
    const qmbx_table_header* h = static_cast<const qmbx_table_header*>(table_host);
    if (h == nullptr || h->magic != QMBX_MAGIC || h->version != QMBX_TABLE_VERSION) {
        return fail(QMBX_ERR_ARGUMENT, "not a compiled qmbx table");
    }
    counts[0] = h->n_terms;
    counts[1] = h->n_live;
    counts[2] = h->part[QMBX_PART_DIAG].n;
    counts[3] = h->n_qubytes;
    counts[4] = h->particle_cut;
    counts[5] = h->n_words;
    return QMBX_OK;
}

namespace qmbx {
namespace {

// 128-bit fingerprint of a canonical closed form (two independent 64-bit
// mixes of its words): distinct forms collide with probability ~n^2 / 2^129.
struct FormKey {
    uint64_t a, b;
    bool operator==(const FormKey& o) const { return a == o.a && b == o.b; }
};
struct FormKeyHash {
    size_t operator()(const FormKey& k) const { return (size_t)(k.a ^ (k.b * 0x9E3779B97F4A7C15ull)); }
};

uint64_t mix64(uint64_t x) {
    x ^= x >> 30;
    x *= 0xBF58476D1CE4E5B9ull;
    x ^= x >> 27;
    x *= 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// Accumulate sign * coef of every term of a part under its canonical closed
// form: the parity bits inside the mask are fixed by val on every row the
// term applies to, so they move into the sign and leave the mask.
void accumulate(const char* blob, const qmbx_table_part& p, int words, bool conj, double sign,
                std::unordered_map<FormKey, std::pair<double, double>, FormKeyHash>& acc, double& scale) {
    const uint64_t* test = reinterpret_cast<const uint64_t*>(blob + p.off_test);
    const uint64_t* apply = reinterpret_cast<const uint64_t*>(blob + p.off_apply);
    const double* coef = reinterpret_cast<const double*>(blob + p.off_coef);
    for (int64_t t = 0; t < p.n; ++t) {
        uint64_t ka = 0x243F6A8885A308D3ull, kb = 0x13198A2E03707344ull;
        int parity = 0;
        for (int q = 0; q < words; ++q) {
            const uint64_t at = ((uint64_t)q * (uint64_t)p.n + (uint64_t)t) * 2;
            const uint64_t mask = test[at], val = test[at + 1] & mask, flip = apply[at], par = apply[at + 1];
            parity ^= __builtin_popcountll(val & par & mask) & 1;
            const uint64_t form[4] = {mask, val, flip, par & ~mask};
            for (int k = 0; k < 4; ++k) {
                ka = mix64(ka ^ form[k]);
                kb = mix64(kb + form[k] * 0xD6E8FEB86659FD93ull);
            }
        }
        const double s = parity ? -sign : sign;
        const double re = coef[2 * t], im = conj ? -coef[2 * t + 1] : coef[2 * t + 1];
        std::pair<double, double>& v = acc[FormKey{ka, kb}];
        v.first += s * re;
        v.second += s * im;
        scale = std::fmax(scale, std::fabs(re) + std::fabs(im));
    }
}

}  // namespace
}  // namespace qmbx

extern "C" int qmbx_table_hermitian(const void* table_host, int32_t* hermitian) {
    clear_error();
    const qmbx_table_header* h = static_cast<const qmbx_table_header*>(table_host);
    if (h == nullptr || h->magic != QMBX_MAGIC || h->version != QMBX_TABLE_VERSION) {
        return fail(QMBX_ERR_ARGUMENT, "not a compiled qmbx table");
    }
    if (hermitian == nullptr) return fail(QMBX_ERR_ARGUMENT, "hermitian must not be NULL");
    const char* blob = static_cast<const char*>(table_host);
    // H = sum of forward terms; H^dagger = sum of the daggered terms with
    // conjugated coefficients.  H is Hermitian when both sums agree form by
    // form, and the diagonal terms sum to a real coefficient per form.
    std::unordered_map<FormKey, std::pair<double, double>, FormKeyHash> off, diag;
    double scale = 0.0;
    accumulate(blob, h->part[QMBX_PART_FWD], h->n_words, false, 1.0, off, scale);
    accumulate(blob, h->part[QMBX_PART_ADJ], h->n_words, true, -1.0, off, scale);
    accumulate(blob, h->part[QMBX_PART_DIAG], h->n_words, false, 1.0, diag, scale);
    const double tol = 1e-12 * (scale > 0.0 ? scale : 1.0);
    int32_t ok = 1;
    for (const auto& kv : off) {
        if (std::fabs(kv.second.first) > tol || std::fabs(kv.second.second) > tol) ok = 0;
    }
    for (const auto& kv : diag) {
        if (std::fabs(kv.second.second) > tol) ok = 0;
    }
    *hermitian = ok;
    return QMBX_OK;
}
