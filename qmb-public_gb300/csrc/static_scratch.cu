// apply_within without any allocation: the workspace lives in a fixed-size
// device array that is part of this library's module image.
//
// Some callers of this engine cannot allocate device memory: a host program
// that hands the GPU's memory to its own pool up front and forbids further
// allocation, a latency-critical loop that cannot afford the implicit
// synchronisation of cudaMalloc/cudaFree, or a plain C program that has no
// allocator of its own and does not want to size and keep a workspace
// buffer.  qmbx_apply_within_static serves them with the same kernels as
// qmbx_apply_within, carving its workspace out of g_scratch.
//
// g_scratch is a __device__ array: every GPU that loads this library holds
// kStaticScratchBytes for it until the process exits.  Its name is only a
// host-side stand-in; the device address comes from cudaGetSymbolAddress,
// with the calling device current.  A call on a stream that is not being
// captured looks the address up again (cheap), so that a device reset, after
// which the module is loaded anew, cannot leave a stale address behind; a
// call on a capturing stream uses the address of the last call on that
// device.  The first call per device should therefore be made before any
// stream capture begins.  All calls share the one array: two calls
// whose work overlaps on the GPU (different streams, or different host
// threads) race on it and must be serialised by the caller.  The array keeps
// the previous call's contents; every buffer carved from it that has to start
// from a known value (the hash-set slots, the output) is cleared by the call
// itself.
#include <cuda_runtime.h>

#include <mutex>

#include "device.cuh"

namespace {

constexpr uint64_t kStaticScratchBytes = QMBX_STATIC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_scratch[kStaticScratchBytes];

std::mutex g_scratch_mu;
void* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_scratch on the current device: looked up again unless
// `stream` is capturing, in which case the address of the last call is used.
int scratch_address(cudaStream_t stream, void** out) {
    int dev = -1;
    QMBX_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        return qmbx::fail(QMBX_ERR_ARGUMENT, "device ordinal %d is beyond the %d supported", dev, kMaxDevices);
    }
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    QMBX_CUDA_TRY(cudaStreamIsCapturing(stream, &capture));
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (capture != cudaStreamCaptureStatusNone && g_scratch_ptr[dev] == nullptr) {
        return qmbx::fail(QMBX_ERR_ARGUMENT,
                          "the first qmbx_apply_within_static call on a device must not be made during stream capture");
    }
    if (capture == cudaStreamCaptureStatusNone) {
        void* p = nullptr;
        cudaError_t err = cudaGetSymbolAddress(&p, g_scratch);
        if (err != cudaSuccess) {
            return qmbx::fail(QMBX_ERR_CUDA, "cudaGetSymbolAddress of the static scratch failed: %s",
                              cudaGetErrorString(err));
        }
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return QMBX_OK;
}

}  // namespace

extern "C" int qmbx_apply_within_static(const void* table_host, const void* table_dev, const uint8_t* configs_i,
                                        const double* psi_i, int64_t n_i, const uint8_t* configs_j, int64_t n_j,
                                        int32_t same_configs, double* psi_j, qmbx_stream_t stream) {
    qmbx::clear_error();
    uint64_t need = 0;
    int st = qmbx::apply_within_workspace_for(table_host, n_i, n_j, same_configs != 0, &need);
    if (st != QMBX_OK) return st;
    if (need > kStaticScratchBytes) {
        return qmbx::fail(QMBX_ERR_ARGUMENT,
                          "apply_within on %lld x %lld rows needs %llu bytes of scratch; the static scratch holds %llu "
                          "(use qmbx_apply_within with a caller workspace)",
                          (long long)n_i, (long long)n_j, (unsigned long long)need,
                          (unsigned long long)kStaticScratchBytes);
    }
    void* scratch = nullptr;
    if ((st = scratch_address(reinterpret_cast<cudaStream_t>(stream), &scratch)) != QMBX_OK) return st;
    return qmbx_apply_within(table_host, table_dev, configs_i, psi_i, n_i, configs_j, n_j, same_configs, psi_j, scratch,
                             kStaticScratchBytes, stream);
}
