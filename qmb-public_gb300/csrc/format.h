// Layout of a compiled term table (shared by the host compiler and the kernels).
//
// A configuration is held as n_words 64-bit "key words" in big-endian byte
// order: row byte b sits in word b / 8 at bits (7 - b % 8) * 8 .. +7, so that
// comparing key words as unsigned integers, word 0 first, is the reference's
// lexicographic row order (array_less, qmb/_hamiltonian_cuda.cu:13-26) and
// site s sits at key bit keybit(s) of word s / 64.
//
// Every live term t is compiled, for the configuration c it acts on, into
//   applicable  <=>  ((c ^ val) & mask) == 0           (per word)
//   image        =   c ^ flip
//   sign         =   (-1)^(popcount(c & par))          (par == 0 for hard-core bosons)
// with the constant part of the sign folded into the stored coefficient.
// This is the closed form of the reference's operator-by-operator walk
// (qmb/_hamiltonian_cpu.cpp:48-78): the walk's bit tests fix the initial value
// of every touched site, its writes toggle each touched site once per
// operator, and its parity is a GF(2)-linear function of the initial
// configuration.
//
// Three parts are stored: the forward part (terms that change the
// configuration, applied to sources), the adjoint part (the same terms
// daggered: slots reversed, create <-> annihilate, applied to targets) and
// the diagonal part (terms whose flip mask is empty).  Terms that can never
// apply (an operator writing the value a previous operator of the same term
// left) are dropped.
//
// Within each part the terms are grouped by a pivot taken from the sites
// they require occupied (bits of mask & val), numbered by key position
// kp = word * 64 + bit: the two lowest such positions (p < q) give the pair
// group 1 + 64W + q(q-1)/2 + p, a single one gives the single group 1 + p,
// none gives group 0.  A row can only be acted on by terms whose pivot sites
// it occupies, so a walk over a row visits group 0, the single groups of its
// occupied positions and the pair groups of its occupied pairs, nothing else.
// Terms are stored sorted by group (stable in input order); groups[g] holds
// [start, end); single_ne marks non-empty single groups and pair_ne[p] the
// positions q > p whose pair group is non-empty.
//
// The per-word masks are stored word-major in two arrays, the test pair
// (mask, val) and the apply pair (flip, par): lanes that read consecutive
// terms of one word read consecutive 16-byte pairs (fully coalesced loads),
// and a walk that tests terms one at a time reads the apply pair only for
// terms whose test passed.  Tables of at most 32 sites (n_qubytes <= 4) also
// hold every term's four masks narrowed to their high 32 bits in one 16-byte
// record, which the grouped walks read instead: half the bytes a term, one
// load, and 32-bit tests.
#pragma once

#include <stdint.h>

#define QMBX_MAGIC 0x58424D51u  // "QMBX"
#define QMBX_TABLE_VERSION 7u
#define QMBX_MAX_WORDS 4
#define QMBX_ALIGN 256

enum { QMBX_PART_FWD = 0, QMBX_PART_ADJ = 1, QMBX_PART_DIAG = 2, QMBX_PARTS = 3 };

struct qmbx_table_part {
    int64_t n;            // terms in this part
    uint64_t off_test;    // uint64[W][n][2]: (mask, val) of word q of term t at (q * n + t) * 2
    uint64_t off_apply;   // uint64[W][n][2]: (flip, par), same order
    uint64_t off_coef;    // double[n][2]   sign-folded coefficient
    uint64_t off_coef32;  // float[n][4]    (re_hi, re_lo, im_hi, im_lo)
    uint64_t off_orig;    // int32[n]       index of the term in the input table
    uint64_t off_norm;    // float[n]       |coef|^2 rounded to FP32
    uint64_t off_groups;  // int32[n_groups][2]  [start, end) of each group
    uint64_t off_single_ne;  // uint64[W]       non-empty single groups by key position
    uint64_t off_pair_ne;    // uint64[64W][W]  for position p: positions q > p with a non-empty pair group
    uint64_t off_nonempty;   // int32[n_groups][4]: (start, end, p, q) of each non-empty group in id order
                             // (p, q the pivot key positions, -1 when absent; first n_nonempty rows valid)
    uint64_t off_narrow;     // uint32[n][4]: (mask, val, flip, par) >> 32 of every term, present (non-zero)
                             // when n_sites <= 32: one key word whose low half is always zero
    int64_t n_groups;        // 1 + 64W + 64W(64W-1)/2
    int64_t n_nonempty;      // groups holding at least one term
    int32_t wide_groups;     // 1 when non-empty groups hold 8 or more terms on average
    int32_t reserved;
};

struct qmbx_table_header {
    uint32_t magic;
    uint32_t version;
    int32_t n_qubytes;
    int32_t particle_cut;
    int32_t n_words;
    int32_t n_sites;
    int64_t n_terms;      // rows of the input table
    int64_t n_live;       // terms that can apply
    qmbx_table_part part[QMBX_PARTS];
    uint64_t total_bytes;
};

#ifdef __cplusplus
static inline int qmbx_keyword(int s) { return s >> 6; }
static inline int qmbx_keybit(int s) { return (7 - ((s >> 3) & 7)) * 8 + (s & 7); }
static inline int64_t qmbx_group_count(int words) {
    int64_t p = 64 * (int64_t)words;
    return 1 + p + p * (p - 1) / 2;
}
#endif

#ifdef __CUDACC__
#define QMBX_HD __host__ __device__
#else
#define QMBX_HD
#endif

#ifdef __cplusplus
static inline QMBX_HD int64_t qmbx_single_group(int kp) { return 1 + kp; }
static inline QMBX_HD int64_t qmbx_pair_group(int words, int p, int q) {
    return 1 + 64 * (int64_t)words + (int64_t)q * (q - 1) / 2 + p;
}
#endif
