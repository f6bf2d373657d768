// The elementwise parts of the autoregressive network of qmb/mlp.py:60-314
// (WaveFunctionElectronUpDown): the particle-number mask, the normalisation
// of each site's four log amplitudes, the per-row sum over sites, and one
// site of the unique sampler (Gumbel-perturbed log probabilities conditioned
// on the parent's, https://arxiv.org/pdf/2408.07625).  The reference runs each
// of these as a chain of small torch operations per site; here each is one
// kernel.  The networks' matrix products stay with cuBLAS (torch.nn.Linear).
//
// A site's four entries k = 2a + b are (up, down) = (a, b) occupations; a
// partial configuration of i sites with u up and d down electrons may take
// up = 0 while i - u < sites - spin_up, up = 1 while u < spin_up, and the
// same for down (qmb/mlp.py _mask).  Disallowed entries get log amplitude
// -inf.  Arithmetic is FP32 as in the reference (the network's dtype).
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>

#include "device.cuh"

namespace qmbx {
namespace {

__device__ __forceinline__ void site_mask(int i, int sites, int up, int down, int n_up, int n_down, bool (&ok)[4]) {
    const bool up0 = (i - n_up) < sites - up, up1 = n_up < up;
    const bool dn0 = (i - n_down) < sites - down, dn1 = n_down < down;
    ok[0] = up0 && dn0;
    ok[1] = up0 && dn1;
    ok[2] = up1 && dn0;
    ok[3] = up1 && dn1;
}

// The masked log amplitudes d[k] shifted by log(sum_k exp(2 d[k])) / 2.  The
// four terms are summed as (e0 + e1) + (e2 + e3), the order torch's CUDA sum
// over a row of four takes, so that the values match the reference's torch
// expression bit for bit on the GPU.
__device__ __forceinline__ void normalized(const float4 raw, const bool (&ok)[4], float (&nd)[4]) {
    float d[4] = {raw.x, raw.y, raw.z, raw.w};
    float e[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        d[k] = ok[k] ? d[k] : -INFINITY;
        e[k] = expf(2.f * d[k]);
    }
    const float sum = __fadd_rn(__fadd_rn(e[0], e[1]), __fadd_rn(e[2], e[3]));
    const float shift = logf(sum) / 2.f;
#pragma unroll
    for (int k = 0; k < 4; ++k) nd[k] = d[k] - shift;
}

// total[r] = sum over sites of the normalised log amplitude of row r's own
// occupations (FP32 terms summed in FP64, as the reference does).
// deltas: [sites][rows] float4 (site-major); occ: [rows][sites] uint8, 2 a + b.
__global__ void log_amplitude_kernel(int64_t rows, int sites, int up, int down, const float4* __restrict__ deltas,
                                     const uint8_t* __restrict__ occ, double* __restrict__ total) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    int n_up = 0, n_down = 0;
    double acc = 0.0;
    for (int i = 0; i < sites; ++i) {
        bool ok[4];
        site_mask(i, sites, up, down, n_up, n_down, ok);
        float nd[4];
        normalized(__ldg(deltas + (int64_t)i * rows + r), ok, nd);
        const int k = occ[r * sites + i] & 3;
        acc += (double)nd[k];
        n_up += k >> 1;
        n_down += k & 1;
    }
    total[r] = acc;
}

// Gradient of log_amplitude_kernel: d total / d delta[i][k] = [k is the row's
// entry] - exp(2 nd[k]) (zero for disallowed entries), times grad[r].
__global__ void log_amplitude_grad_kernel(int64_t rows, int sites, int up, int down, const float4* __restrict__ deltas,
                                          const uint8_t* __restrict__ occ, const double* __restrict__ grad,
                                          float4* __restrict__ grad_deltas) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const float g = (float)grad[r];
    int n_up = 0, n_down = 0;
    for (int i = 0; i < sites; ++i) {
        bool ok[4];
        site_mask(i, sites, up, down, n_up, n_down, ok);
        float nd[4];
        normalized(__ldg(deltas + (int64_t)i * rows + r), ok, nd);
        const int k = occ[r * sites + i] & 3;
        float out[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) out[j] = ok[j] ? g * ((j == k ? 1.f : 0.f) - expf(2.f * nd[j])) : 0.f;
        grad_deltas[(int64_t)i * rows + r] = make_float4(out[0], out[1], out[2], out[3]);
        n_up += k >> 1;
        n_down += k & 1;
    }
}

// One site of the sampler for n partial rows: from the raw log amplitudes
// (delta), the rows' electron counts, their log probability lp and Gumbel
// value gp, and uniforms u, the four children's log probabilities
//   l_k = lp + 2 nd_k,  G_k = l_k - log(-log u_k),  Z = max_k G_k,
//   t_k = -log(exp(-gp) - exp(-Z) + exp(-G_k)),
// written child-major (child k of row r at k * n + r), as the reference
// lays out its four appended copies.  Rows whose gp is not finite have no
// children (all four -inf).  With la (the rows' log amplitudes so
// far, FP64) the children's a_k = la + nd_k are written too: after the last
// site they are the log amplitudes the network's forward gives the sampled
// configurations (the same FP32 terms summed in FP64 in the same order).
// With `bad` (a device counter the caller zeroes), a child whose value is
// NaN or +inf is written as -FLT_MAX and counted: the reference's descending
// sort puts such values first and then drops them, so they take places of
// the cut without being kept; sampler_take_kernel marks the places they took.
__global__ void sampler_site_kernel(int64_t n, int site, int sites, int up, int down, const float4* __restrict__ delta,
                                    const int2* __restrict__ counts, const float* __restrict__ lp,
                                    const float* __restrict__ gp, const float4* __restrict__ uniforms,
                                    float* __restrict__ l_out, float* __restrict__ t_out,
                                    const double* __restrict__ la, double* __restrict__ a_out,
                                    int* __restrict__ bad) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int2 c = counts[r];
    bool ok[4];
    site_mask(site, sites, up, down, c.x, c.y, ok);
    float nd[4];
    normalized(delta[r], ok, nd);
    const float4 u4 = uniforms[r];
    const float u[4] = {u4.x, u4.y, u4.z, u4.w};
    const float base = lp[r], parent = gp[r];
    float l[4], g[4];
    float z = -INFINITY;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        l[k] = base + 2.f * nd[k];
        g[k] = l[k] - logf(-logf(u[k]));
        z = fmaxf(z, g[k]);
    }
    const float ep = expf(-parent), ez = expf(-z);
    // a row carried with a value that is not finite is one the reference has
    // dropped (its selection keeps finite values only): no children
    const bool dead = !isfinite(parent);
    int n_bad = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        float t = dead ? -INFINITY : -logf(ep - ez + expf(-g[k]));
        if (bad != nullptr && (isnan(t) || t == INFINITY)) {
            t = -FLT_MAX;
            ++n_bad;
        }
        l_out[k * n + r] = dead ? -INFINITY : l[k];
        t_out[k * n + r] = t;
    }
    if (n_bad) atomicAdd(bad, n_bad);
    if (la != nullptr) {
        const double a = la[r];
#pragma unroll
        for (int k = 0; k < 4; ++k) a_out[k * n + r] = a + (double)nd[k];
    }
}

// The m chosen children (index = k * n + parent): their occupations (the
// parent's, site `site` set to k), network inputs, electron counts and
// log probabilities.  occ/xf are [rows][sites] and [rows][2 sites].
// With `bad` (the site kernel's count of NaN / +inf values), the chosen rows
// the reference would not keep get gp -inf: those written as -FLT_MAX, and
// those past batch - *bad (the places the reference's NaN / +inf values
// took at the top of its sort).
__global__ void sampler_take_kernel(int64_t m, int64_t n, int site, int sites, const int64_t* __restrict__ index,
                                    const uint8_t* __restrict__ occ_in, const int2* __restrict__ counts_in,
                                    const float* __restrict__ l_in, const float* __restrict__ t_in,
                                    uint8_t* __restrict__ occ_out, float* __restrict__ xf_out,
                                    int2* __restrict__ counts_out, float* __restrict__ lp_out,
                                    float* __restrict__ gp_out, const double* __restrict__ a_in,
                                    double* __restrict__ la_out, int64_t batch, const int* __restrict__ bad) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    const int64_t idx = index[j];
    const int64_t parent = idx % n;
    const int k = (int)(idx / n);
    for (int i = 0; i < site; ++i) {
        const uint8_t v = occ_in[parent * sites + i];
        occ_out[j * sites + i] = v;
        xf_out[j * 2 * sites + 2 * i] = (float)(v >> 1);
        xf_out[j * 2 * sites + 2 * i + 1] = (float)(v & 1);
    }
    occ_out[j * sites + site] = (uint8_t)k;
    xf_out[j * 2 * sites + 2 * site] = (float)(k >> 1);
    xf_out[j * 2 * sites + 2 * site + 1] = (float)(k & 1);
    const int2 c = counts_in[parent];
    counts_out[j] = make_int2(c.x + (k >> 1), c.y + (k & 1));
    lp_out[j] = l_in[idx];
    const float t = t_in[idx];
    const bool dropped = bad != nullptr && (t == -FLT_MAX || j >= batch - (int64_t)*bad);
    gp_out[j] = dropped ? -INFINITY : t;
    if (a_in != nullptr) la_out[j] = a_in[idx];
}

int check_sites(int sites, int up, int down) {
    if (sites < 1 || up < 0 || down < 0 || up > sites || down > sites) {
        return fail(QMBX_ERR_ARGUMENT, "sites %d, spin_up %d, spin_down %d out of range", sites, up, down);
    }
    return QMBX_OK;
}

}  // namespace
}  // namespace qmbx

using namespace qmbx;

extern "C" int qmbx_sampler_log_amplitude(int64_t rows, int32_t sites, int32_t spin_up, int32_t spin_down,
                                          const float* deltas, const uint8_t* occ, double* total,
                                          qmbx_stream_t stream) {
    clear_error();
    int st = check_sites(sites, spin_up, spin_down);
    if (st != QMBX_OK) return st;
    if (rows < 0) return fail(QMBX_ERR_ARGUMENT, "rows must not be negative");
    if (rows == 0) return QMBX_OK;
    if (deltas == nullptr || occ == nullptr || total == nullptr) return fail(QMBX_ERR_ARGUMENT, "pointers must not be NULL");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    QMBX_KERNEL(kGroupOther, s, log_amplitude_kernel<<<grid_for(rows, kThreads), kThreads, 0, s>>>(rows, sites, spin_up, spin_down, reinterpret_cast<const float4*>(deltas), occ, total));
    QMBX_LAUNCH_CHECK("log_amplitude_kernel");
    return QMBX_OK;
}

extern "C" int qmbx_sampler_log_amplitude_grad(int64_t rows, int32_t sites, int32_t spin_up, int32_t spin_down,
                                               const float* deltas, const uint8_t* occ, const double* grad,
                                               float* grad_deltas, qmbx_stream_t stream) {
    clear_error();
    int st = check_sites(sites, spin_up, spin_down);
    if (st != QMBX_OK) return st;
    if (rows < 0) return fail(QMBX_ERR_ARGUMENT, "rows must not be negative");
    if (rows == 0) return QMBX_OK;
    if (deltas == nullptr || occ == nullptr || grad == nullptr || grad_deltas == nullptr) {
        return fail(QMBX_ERR_ARGUMENT, "pointers must not be NULL");
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    QMBX_KERNEL(kGroupOther, s, log_amplitude_grad_kernel<<<grid_for(rows, kThreads), kThreads, 0, s>>>(rows, sites, spin_up, spin_down, reinterpret_cast<const float4*>(deltas), occ, grad, reinterpret_cast<float4*>(grad_deltas)));
    QMBX_LAUNCH_CHECK("log_amplitude_grad_kernel");
    return QMBX_OK;
}

extern "C" int qmbx_sampler_site(int64_t n, int32_t site, int32_t sites, int32_t spin_up, int32_t spin_down,
                                 const float* delta, const int32_t* counts, const float* lp, const float* gp,
                                 const float* uniforms, float* l_out, float* t_out, const double* la,
                                 double* a_out, int32_t* bad, qmbx_stream_t stream) {
    clear_error();
    int st = check_sites(sites, spin_up, spin_down);
    if (st != QMBX_OK) return st;
    if (site < 0 || site >= sites) return fail(QMBX_ERR_ARGUMENT, "site %d out of range", site);
    if (n < 0) return fail(QMBX_ERR_ARGUMENT, "row count must not be negative");
    if (n == 0) return QMBX_OK;
    if (!delta || !counts || !lp || !gp || !uniforms || !l_out || !t_out) {
        return fail(QMBX_ERR_ARGUMENT, "pointers must not be NULL");
    }
    if ((la == nullptr) != (a_out == nullptr)) return fail(QMBX_ERR_ARGUMENT, "la and a_out go together");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    QMBX_KERNEL(kGroupOther, s, sampler_site_kernel<<<grid_for(n, kThreads), kThreads, 0, s>>>(n, site, sites, spin_up, spin_down, reinterpret_cast<const float4*>(delta), reinterpret_cast<const int2*>(counts), lp, gp, reinterpret_cast<const float4*>(uniforms), l_out, t_out, la, a_out, bad));
    QMBX_LAUNCH_CHECK("sampler_site_kernel");
    return QMBX_OK;
}

extern "C" int qmbx_sampler_take(int64_t m, int64_t n, int32_t site, int32_t sites, const int64_t* index,
                                 const uint8_t* occ_in, const int32_t* counts_in, const float* l_in,
                                 const float* t_in, uint8_t* occ_out, float* xf_out, int32_t* counts_out,
                                 float* lp_out, float* gp_out, const double* a_in, double* la_out,
                                 int64_t batch, const int32_t* bad, qmbx_stream_t stream) {
    clear_error();
    if (sites < 1 || site < 0 || site >= sites) return fail(QMBX_ERR_ARGUMENT, "site %d of %d out of range", site, sites);
    if (m < 0 || n < 0 || m > 4 * n) return fail(QMBX_ERR_ARGUMENT, "row counts out of range");
    if (m == 0) return QMBX_OK;
    if (!index || !occ_in || !counts_in || !l_in || !t_in || !occ_out || !xf_out || !counts_out || !lp_out || !gp_out) {
        return fail(QMBX_ERR_ARGUMENT, "pointers must not be NULL");
    }
    if ((a_in == nullptr) != (la_out == nullptr)) return fail(QMBX_ERR_ARGUMENT, "a_in and la_out go together");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    QMBX_KERNEL(kGroupOther, s, sampler_take_kernel<<<grid_for(m, kThreads), kThreads, 0, s>>>(m, n, site, sites, index, occ_in, reinterpret_cast<const int2*>(counts_in), l_in, t_in, occ_out, xf_out, reinterpret_cast<int2*>(counts_out), lp_out, gp_out, a_in, la_out, batch, bad));
    QMBX_LAUNCH_CHECK("sampler_take_kernel");
    return QMBX_OK;
}
