/*
 * qmbx — C ABI of the GB300 (sm_103a) second-quantized Hamiltonian engine.
 *
 * Drop-in boundary for the four torch operators that the reference declares in
 * qmb/_hamiltonian.cpp:83-89 and implements in qmb/_hamiltonian_cuda.cu:
 *
 *   apply_within(configs_i, psi_i, configs_j, site, kind, coef) -> psi_j
 *   find_relative(configs_i, psi_i, count_selected, site, kind, coef, configs_exclude) -> configs
 *   diagonal_term(configs, site, kind, coef) -> psi
 *   single_relative(configs, site, kind, coef) -> configs
 *
 * Conventions (qmb/_hamiltonian_cuda.cu:184-232):
 *   - configurations are rows of n_qubytes bytes, site s in byte s/8 bit s%8
 *     (qmb/bitspack.py:8-94); rows need no alignment;
 *   - amplitudes are complex numbers stored as (real, imaginary) pairs:
 *     double[n][2] for complex128, float[n][2] for complex64;
 *   - the term table (site int16[T][4], kind uint8[T][4] with 0 = annihilate,
 *     1 = create, 2 = empty slot, coef double[T][2]) is compiled once on the
 *     host by qmbx_table_build into a blob that the caller copies to device
 *     memory (256-byte aligned) and passes to every device call together with
 *     its host copy, from which only the header is read;
 *   - device calls take device pointers, a caller-owned workspace of at least
 *     the size the matching *_workspace query returns (256-byte aligned), and
 *     a CUDA stream; they enqueue work on that stream and return without
 *     synchronising, except where noted;
 *   - no call allocates device memory;
 *   - every call returns QMBX_OK or an error status and never traps; the
 *     message of the last error of the calling thread is qmbx_last_error().
 *
 * Limits: 1 <= n_qubytes <= 32 (at most 256 sites); particle_cut 1 (fermions)
 * or 2 (hard-core bosons); row counts below 2^31.
 */
#ifndef QMBX_H
#define QMBX_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* qmbx_stream_t; /* a cudaStream_t; NULL is the legacy default stream */

enum {
    QMBX_OK = 0,
    QMBX_ERR_ARGUMENT = 1,  /* invalid argument (sizes, kinds, sites, alignment) */
    QMBX_ERR_CUDA = 2,      /* a CUDA runtime call failed */
    QMBX_ERR_WORKSPACE = 3, /* workspace smaller than the query asked for */
    QMBX_ERR_DEVICE = 4,    /* a kernel reported an error status (bounded wait expired, capacity exceeded) */
};

/* Version of this ABI (major * 10000 + minor * 100 + patch). */
int qmbx_version(void);

/* Message of the last failed call made by this thread ("" when none). */
const char* qmbx_last_error(void);

/* ---------------------------------------------------------------------------
 * Term table (host only, no GPU needed).
 * Replaces the term-table handling of qmb/hamiltonian.py:71-102 and the
 * per-thread term decoding of qmb/_hamiltonian_cuda.cu:54-84.
 * ------------------------------------------------------------------------- */

/* Bytes of the compiled table for these terms. */
int qmbx_table_bytes(const int16_t* site, const uint8_t* kind, int64_t n_terms, int32_t n_qubytes,
                     int32_t particle_cut, uint64_t* bytes);

/* Compile the terms into blob (blob_bytes >= qmbx_table_bytes). */
int qmbx_table_build(const int16_t* site, const uint8_t* kind, const double* coef, int64_t n_terms, int32_t n_qubytes,
                     int32_t particle_cut, void* blob, uint64_t blob_bytes);

/* QMBX_OK when blob (blob_bytes long) holds a whole table of the format this
 * library reads, e.g. one written to a cache file by an earlier process. */
int qmbx_table_check(const void* blob, uint64_t blob_bytes);

/* Counts read from a compiled table: [n_terms, live terms, diagonal terms, n_qubytes, particle_cut, n_words]. */
int qmbx_table_counts(const void* table_host, int64_t counts[6]);

/* *hermitian = 1 when the compiled operator equals its adjoint, else 0 (no
 * counterpart in the reference).  The check compares the forward terms with
 * the daggered, conjugated terms closed form by closed form (1e-12 relative
 * to the largest coefficient) and requires the diagonal terms to sum to real
 * coefficients; an operator written so that equal matrices have different
 * closed forms can be reported 0 although Hermitian.  The tolerance is the
 * bound the other way: an operator whose closed forms differ from their
 * adjoints' by at most 1e-12 of the largest |coefficient| is reported 1, and
 * a gradient taken from H psi alone then misses that anti-Hermitian part
 * (its size is at most 1e-12 max|c| times the number of such terms).
 * Callers use it to get the gradient of <psi|H|psi> from H psi alone; the
 * Python energy function takes hermitian_shortcut=False to always walk the
 * adjoint instead. */
int qmbx_table_hermitian(const void* table_host, int32_t* hermitian);

/* ---------------------------------------------------------------------------
 * apply_within: psi_j[j] = sum over terms t and rows i with t|i> = s|j> of
 * s * coef_t * psi_i[i].  Replaces apply_within_interface
 * (qmb/_hamiltonian_cuda.cu:171-274).  Where configs_j repeats a row, the
 * first occurrence receives the amplitude and the others zero.
 * same_configs != 0 declares configs_i and configs_j to be the same rows
 * (configs_j is then ignored), which saves one sort.
 *
 * Determinism (this entry point, its adjoint and their FP32 variants): the
 * walk over the output side's rows sums each row in a fixed order and
 * repeats bit for bit; it is taken when the rows are the same or the output
 * side is not much larger than the input side.  Otherwise the input side is
 * walked and contributions are added with FP64 atomics (as is every
 * pivot-major walk, taken for tables whose pivot groups hold hundreds of
 * terms), whose order varies from run to run in the last bits.
 * QMBX_DETERMINISTIC=1 in the environment (read at every call) keeps every
 * call on the fixed-order walk.  Repeated rows of an input are summed with
 * atomics before the walk in any case.
 * ------------------------------------------------------------------------- */

int qmbx_apply_within_workspace(const void* table_host, int64_t n_i, int64_t n_j, uint64_t* bytes);

int qmbx_apply_within(const void* table_host, const void* table_dev, const uint8_t* configs_i, const double* psi_i,
                      int64_t n_i, const uint8_t* configs_j, int64_t n_j, int32_t same_configs, double* psi_j,
                      void* workspace, uint64_t workspace_bytes, qmbx_stream_t stream);

/*
 * Allocation-free qmbx_apply_within (no counterpart in the reference).
 *
 * For callers that cannot allocate device memory themselves or through this
 * library: a host program that has given all device memory to its own pool
 * and forbids further allocation, a latency-critical loop that cannot afford
 * the implicit synchronisation of cudaMalloc/cudaFree, or a plain C caller
 * without an allocator that does not want to size and keep a workspace.
 * Same arguments and results as qmbx_apply_within minus the workspace: the
 * scratch is a fixed device array of QMBX_STATIC_SCRATCH_BYTES inside this
 * library, which every GPU that loads the library holds until the process
 * exits.  Inputs needing more scratch than that (qmbx_apply_within_workspace)
 * are rejected with QMBX_ERR_ARGUMENT; a same_configs call is sized for its
 * one row set.  The array's device address is looked up with the calling
 * device current, on every call made on a stream that is not capturing (so a
 * device reset leaves no stale address); a call on a capturing stream uses
 * the address of the last call on that device, so make the first call on
 * each device before any stream capture.  All calls share the one array:
 * calls whose work overlaps on the GPU race and must be serialised by the
 * caller.  Calls no allocation routine.
 */
#define QMBX_STATIC_SCRATCH_BYTES (32ull << 20)

int qmbx_apply_within_static(const void* table_host, const void* table_dev, const uint8_t* configs_i,
                             const double* psi_i, int64_t n_i, const uint8_t* configs_j, int64_t n_j,
                             int32_t same_configs, double* psi_j, qmbx_stream_t stream);

/*
 * Adjoint of qmbx_apply_within (no counterpart in the reference): with the
 * same rows, out_i[i] = sum over t and j of conj(s * coef_t) * g_j[j], i.e.
 * H^dagger applied with the roles of the two row sets swapped.  Every row of
 * configs_i receives its value; repeated rows of configs_j contribute through
 * their first occurrence only, matching the forward operator.
 */
int qmbx_apply_within_adjoint(const void* table_host, const void* table_dev, const uint8_t* configs_i, int64_t n_i,
                              const uint8_t* configs_j, const double* g_j, int64_t n_j, int32_t same_configs,
                              double* out_i, void* workspace, uint64_t workspace_bytes, qmbx_stream_t stream);

/*
 * FP32 variants (no counterpart in the reference): complex64 inputs, products
 * formed with an exact FP32 two-product and accumulated per target with
 * two-sum compensation.  The result is written as complex128 (the compensated
 * pair, summed exactly) to out_f64 when it is non-NULL and as complex64 to
 * out_f32 when that is non-NULL.  include_diagonal = 0 leaves out the terms
 * that map a row onto itself (their contribution is then added in FP64 by
 * the caller from qmbx_diagonal_term).
 */
int qmbx_apply_within_f32c(const void* table_host, const void* table_dev, const uint8_t* configs_i, const float* psi_i,
                           int64_t n_i, const uint8_t* configs_j, int64_t n_j, int32_t same_configs,
                           int32_t include_diagonal, double* out_f64, float* out_f32, void* workspace,
                           uint64_t workspace_bytes, qmbx_stream_t stream);

int qmbx_apply_within_adjoint_f32c(const void* table_host, const void* table_dev, const uint8_t* configs_i,
                                   int64_t n_i, const uint8_t* configs_j, const float* g_j, int64_t n_j,
                                   int32_t same_configs, int32_t include_diagonal, double* out_f64, float* out_f32,
                                   void* workspace, uint64_t workspace_bytes, qmbx_stream_t stream);

/* ---------------------------------------------------------------------------
 * H restricted to one set of n distinct rows as a sparse matrix (no
 * counterpart in the reference, whose Lanczos loops, qmb/rldiag.py:19-52 and
 * qmb/haar.py:107-183, call apply_within on the same rows every iteration).
 * CSR layout: row j holds entries [row_ptr[j], row_ptr[j + 1]): first the
 * diagonal (column j, possibly zero), then one entry (column i, value = the
 * term's signed coefficient) per (term, row i) mapping row i onto row j.
 * qmbx_matrix_count writes row_ptr (n + 1 device int64) and stores the entry
 * count in *nnz (host); it synchronises the stream.  qmbx_matrix_fill then
 * writes col (nnz int32) and val (nnz complex128) for the same rows and
 * table.  qmbx_matrix_apply computes y = A x (complex128) with a fixed
 * summation order.  Limits: distinct rows, nnz below 2^31.
 * ------------------------------------------------------------------------- */

int qmbx_matrix_workspace(const void* table_host, int64_t n, uint64_t* bytes);

int qmbx_matrix_count(const void* table_host, const void* table_dev, const uint8_t* configs, int64_t n,
                      int64_t* row_ptr, int64_t* nnz, void* workspace, uint64_t workspace_bytes, qmbx_stream_t stream);

int qmbx_matrix_fill(const void* table_host, const void* table_dev, const uint8_t* configs, int64_t n,
                     const int64_t* row_ptr, int32_t* col, double* val, void* workspace, uint64_t workspace_bytes,
                     qmbx_stream_t stream);

int qmbx_matrix_apply(int64_t n, const int64_t* row_ptr, const int32_t* col, const double* val, const double* x,
                      double* y, qmbx_stream_t stream);

/* Y = A X for m complex128 vectors at once (X, Y row-major [n][m]; m = 1 is a
 * plain product), given the matrix's entry count nnz (row_ptr[n]).  Every
 * call with the same arguments gives the same bits: each output is summed
 * over its row's entries in order (rows averaging fewer than 4 entries and
 * m = 1: a thread per row; otherwise a warp per row). */
int qmbx_matrix_apply_many(int64_t n, int64_t nnz, int32_t m, const int64_t* row_ptr, const int32_t* col,
                           const double* val, const double* x, double* y, qmbx_stream_t stream);

/* ---------------------------------------------------------------------------
 * Hit logs (no counterpart in the reference): a forward apply_within that
 * also records what its walk found, and the adjoint product on the same rows
 * computed from that record without a second walk -- the backward of an
 * energy gradient needs exactly the (term, row) pairs the forward found.
 *
 * qmbx_hitlog_bytes sizes the caller's log buffer (device, 256-byte aligned)
 * for n_i x n_j rows and log_cap hit records (16 bytes each); the buffer also
 * holds the forward's workspace, whose row sets the adjoint reuses, so the
 * _logged forwards take no workspace.  They take the arguments of
 * qmbx_apply_within / qmbx_apply_within_f32c plus the log.  The _logged
 * adjoints take the log, the same table, row counts, same_configs and
 * log_cap (and include_diagonal for the FP32 path) and g_j, and give what
 * qmbx_apply_within_adjoint(_f32c) gives, without synchronising: a kernel
 * reads the log's header on the device and either replays the record, or,
 * when the forward found more than log_cap hits, walks the adjoint over the
 * row sets the forward left in the buffer.  A buffer no logged forward wrote
 * with these arguments gives NaN outputs.  qmbx_hitlog_count enqueues a copy
 * of the forward's hit count to *count (host pinned or device memory), for
 * sizing the next log.  The replay adds with FP64 atomics (not bitwise
 * repeatable).  The log must stay allocated until the adjoint's work ends.
 * ------------------------------------------------------------------------- */

int qmbx_hitlog_bytes(const void* table_host, int64_t n_i, int64_t n_j, int32_t same_configs, int64_t log_cap,
                      uint64_t* bytes);

int qmbx_hitlog_count(const void* log, unsigned long long* count, qmbx_stream_t stream);

int qmbx_apply_within_logged(const void* table_host, const void* table_dev, const uint8_t* configs_i,
                             const double* psi_i, int64_t n_i, const uint8_t* configs_j, int64_t n_j,
                             int32_t same_configs, double* psi_j, void* log, uint64_t log_bytes, int64_t log_cap,
                             qmbx_stream_t stream);

int qmbx_apply_within_f32c_logged(const void* table_host, const void* table_dev, const uint8_t* configs_i,
                                  const float* psi_i, int64_t n_i, const uint8_t* configs_j, int64_t n_j,
                                  int32_t same_configs, int32_t include_diagonal, double* out_f64, float* out_f32,
                                  void* log, uint64_t log_bytes, int64_t log_cap, qmbx_stream_t stream);

int qmbx_apply_within_adjoint_logged(const void* table_host, const void* table_dev, const void* log,
                                     uint64_t log_bytes, int64_t log_cap, int64_t n_i, int64_t n_j,
                                     int32_t same_configs, const double* g_j, double* out_i, qmbx_stream_t stream);

int qmbx_apply_within_adjoint_f32c_logged(const void* table_host, const void* table_dev, const void* log,
                                          uint64_t log_bytes, int64_t log_cap, int64_t n_i, int64_t n_j,
                                          int32_t same_configs, int32_t include_diagonal, const float* g_j,
                                          double* out_f64, float* out_f32, qmbx_stream_t stream);

/* ---------------------------------------------------------------------------
 * diagonal_term: out[c] = sum of s * coef_t over terms with t|c> = s|c>.
 * Replaces diagonal_term_interface (qmb/_hamiltonian_cuda.cu:710-803).
 * Needs no workspace.
 * ------------------------------------------------------------------------- */

int qmbx_diagonal_term(const void* table_host, const void* table_dev, const uint8_t* configs, int64_t n, double* out,
                       qmbx_stream_t stream);

/* ---------------------------------------------------------------------------
 * find_relative: the count_selected heaviest (term, source) records with
 * weight |s * coef_t * psi_i|^2 among images not in configs_exclude, records
 * of weight zero dropped, rows sorted and de-duplicated.  Replaces
 * find_relative_interface (qmb/_hamiltonian_cuda.cu:551-675).  Records of
 * equal weight are ranked by the reference's visiting order (term-major),
 * later first.  out must hold count_selected rows; *n_out receives the row
 * count.  This call synchronises the stream before it returns (the output
 * size is data dependent).
 *
 * The workspace holds the records near the selection threshold, whose number
 * is known only after a first pass over the candidates.  When the workspace
 * is too small the call returns QMBX_ERR_WORKSPACE and stores the bytes it
 * needs in *workspace_needed (when non-NULL); call again with at least that
 * much.  qmbx_find_relative_workspace returns a starting size.
 * ------------------------------------------------------------------------- */

int qmbx_find_relative_workspace(const void* table_host, int64_t n_i, int64_t count_selected, int64_t n_exclude,
                                 uint64_t* bytes);

int qmbx_find_relative(const void* table_host, const void* table_dev, const uint8_t* configs_i, const double* psi_i,
                       int64_t n_i, int64_t count_selected, const uint8_t* configs_exclude, int64_t n_exclude,
                       uint8_t* out, int64_t* n_out, void* workspace, uint64_t workspace_bytes,
                       uint64_t* workspace_needed, qmbx_stream_t stream);

/* Figures of the calling thread's last qmbx_find_relative call, for tracing
 * and rooflines (no counterpart in the reference): [0] records emitted by the
 * selection pass, [1] term walks run, [2] radix passes over records and
 * selected rows, [3] bytes those passes move (passes x 2 x items x item
 * bytes), [4] records selected before de-duplication, [5] rows returned. */
int qmbx_find_relative_stats(int64_t stats[6]);

/* ---------------------------------------------------------------------------
 * The Epstein-Nesbet PT2 step of qmb/pert.py:37-61 in one call (the
 * reference composes it in Python from apply_within, find_relative,
 * apply_within and diagonal_term):
 *   energies[0] = E0 = Re<psi|H|psi> / <psi|psi> over configs (n distinct rows),
 *   other = find_relative(configs, psi, count_selected, configs),
 *   energies[1] = E2 = sum over other of |(H psi)_j|^2 / <psi|psi> / (E0 - Re H_jj),
 * *n_other = the number of rows of other.  One apply_within from configs
 * onto configs and other together gives E0's H psi and other's, so the step
 * walks the terms once fewer than the composition.  count_selected >= 1.
 * Synchronises the stream.  Workspace as for qmbx_find_relative: on
 * QMBX_ERR_WORKSPACE *workspace_needed holds the size to retry with.
 * ------------------------------------------------------------------------- */

int qmbx_pt2_workspace(const void* table_host, int64_t n, int64_t count_selected, uint64_t* bytes);

int qmbx_pt2(const void* table_host, const void* table_dev, const uint8_t* configs, const double* psi, int64_t n,
             int64_t count_selected, double* energies, int64_t* n_other, void* workspace, uint64_t workspace_bytes,
             uint64_t* workspace_needed, qmbx_stream_t stream);

/* ---------------------------------------------------------------------------
 * single_relative: for every row, one image outside the row set drawn with
 * probability proportional to |coef_t| (Efraimidis-Spirakis keys from a
 * per-term uniform variate derived from seed); all-zero rows where none
 * exists.  Replaces single_relative_interface
 * (qmb/_hamiltonian_cuda.cu:907-996).
 * ------------------------------------------------------------------------- */

int qmbx_single_relative_workspace(const void* table_host, int64_t n, uint64_t* bytes);

int qmbx_single_relative(const void* table_host, const void* table_dev, const uint8_t* configs, int64_t n,
                         uint64_t seed, uint8_t* out, void* workspace, uint64_t workspace_bytes,
                         qmbx_stream_t stream);

/* ---------------------------------------------------------------------------
 * The elementwise parts of the autoregressive network of qmb/mlp.py:60-314
 * (WaveFunctionElectronUpDown, the caller that samples the configurations
 * the engine works on).  The site networks' matrix products stay with the
 * caller (cuBLAS); these kernels do what lies between them.  A site's four
 * entries k = 2 up + down; counts are (up, down) electrons so far; FP32 as
 * the reference's network.
 *
 * qmbx_sampler_log_amplitude: total[r] = sum over sites i of the masked,
 * normalised log amplitude deltas[i][r][occ[r][i]] (replaces the site loop
 * of the reference's forward, :188-205); deltas float [sites][rows][4], occ
 * uint8 [rows][sites], total double [rows].  _grad: d total / d deltas
 * times grad (double [rows]) into grad_deltas (float [sites][rows][4]).
 *
 * qmbx_sampler_site: one site of generate_unique (:232-266) for n partial
 * rows: from delta float [n][4], counts int32 [n][2], the rows' log
 * probability lp and Gumbel value gp (float [n]) and uniforms float [n][4],
 * the children's log probabilities l_out and conditioned Gumbel values
 * t_out (float [4][n], child k of row r at k n + r, the reference's order).
 * Optionally (both or neither) la, the rows' log amplitudes so far (double
 * [n]), and a_out (double [4][n]): each child's la + its normalised log
 * amplitude -- after the last site, the log amplitude the forward gives the
 * configuration, so psi needs only the phase network.  Rows whose gp is not
 * finite have no children (-inf).  Optionally bad (device int32, zeroed by
 * the caller): children whose value is NaN or +inf are written as -FLT_MAX
 * and counted, so a descending sort puts them after the finite values.
 * qmbx_sampler_take: the m chosen children (index int64 [m] into [4][n]):
 * occupations occ_out uint8 [m][sites] from occ_in, network inputs xf_out
 * float [m][2 sites] (sites up to `site` written), counts, lp, gp, and
 * (optionally, both or neither) la_out from a_in.  With bad (the site
 * call's counter), chosen rows the reference's selection would drop get gp
 * -inf: those written as -FLT_MAX, and those at places batch - *bad and
 * beyond (the places its NaN / +inf values take at the top of its sort).
 * ------------------------------------------------------------------------- */

int qmbx_sampler_log_amplitude(int64_t rows, int32_t sites, int32_t spin_up, int32_t spin_down, const float* deltas,
                               const uint8_t* occ, double* total, qmbx_stream_t stream);

int qmbx_sampler_log_amplitude_grad(int64_t rows, int32_t sites, int32_t spin_up, int32_t spin_down,
                                    const float* deltas, const uint8_t* occ, const double* grad, float* grad_deltas,
                                    qmbx_stream_t stream);

int qmbx_sampler_site(int64_t n, int32_t site, int32_t sites, int32_t spin_up, int32_t spin_down, const float* delta,
                      const int32_t* counts, const float* lp, const float* gp, const float* uniforms, float* l_out,
                      float* t_out, const double* la, double* a_out, int32_t* bad, qmbx_stream_t stream);

int qmbx_sampler_take(int64_t m, int64_t n, int32_t site, int32_t sites, const int64_t* index, const uint8_t* occ_in,
                      const int32_t* counts_in, const float* l_in, const float* t_in, uint8_t* occ_out, float* xf_out,
                      int32_t* counts_out, float* lp_out, float* gp_out, const double* a_in, double* la_out,
                      int64_t batch, const int32_t* bad, qmbx_stream_t stream);

/* ---------------------------------------------------------------------------
 * Tracing (no counterpart in the reference, which has none).
 * Every kernel launch of this library increments a process-wide counter.
 * qmbx_profile_enable(1) additionally brackets the launches of seven groups
 * (0 term walk, 1 key packing/hashing, 2 selection, 3 other, 4 the separate
 * passes over diagonal terms, 5 radix sorts, 6 products with a materialised
 * matrix or replayed from a hit log) with CUDA events on the
 * launching stream and resets the totals; qmbx_profile_read waits for the
 * recorded events and returns the launch counter and, per group, the number
 * of timed launches and their total milliseconds (arrays of
 * QMBX_PROFILE_GROUPS).
 * ------------------------------------------------------------------------- */

#define QMBX_PROFILE_GROUPS 7

int qmbx_profile_enable(int32_t on);

int qmbx_profile_read(int64_t* launches, int64_t* counts, double* ms);

#ifdef __cplusplus
}
#endif

#endif /* QMBX_H */
