// gx_cholesky_step_noalloc: one pivot step of the device-resident Cholesky
// factorisation that allocates no device memory.
//
// Who needs it: callers that manage every byte of device memory themselves
// (a framework's pooling allocator, a process with a hard memory cap, a
// long-running service) and so cannot let a library call cudaMalloc or
// cudaFree, which also synchronise the whole device and would stall their
// other streams.  They pass the factor rows, the raw pivot column, the
// residual diagonal and the output row as device memory of their own; the
// step's scratch (the updated column and the reduction partials) lives in the
// file-scope arrays below, which every GPU that loads this library holds until
// process exit: 1 MiB + 8 KiB per device.
//
// Limit: n * n <= GX_NOALLOC_MAX_ENTRIES (65,536 ordered AO pairs, i.e.
// n <= 256); larger problems are rejected with GX_ELENGTH.
//
// Precondition, as in the allocating driver (which only pivots on entries
// above its stopping threshold): residual[pivot] > 0.  A non-positive pivot
// residual makes the scale 1/sqrt(residual) non-finite, and the new row,
// the residual and result->min_residual then hold non-finite values.
//
// The kernels are the ones gx_cholesky runs for the same step
// (launch_chol_step in gx_chol.cu); only the scratch pointers differ.
#include <mutex>
#include <string>

#include "../../include/giao_gb300.h"
#include "gx_internal.h"

namespace {

constexpr long long kMaxEntries = GX_NOALLOC_MAX_ENTRIES;
constexpr int kMaxDevices = 64;

// Scratch shared by every call on a device.  Each call overwrites every entry
// it later reads (the whole work column, every reduction partial, the scale),
// so nothing has to start at zero; calls that overlap on the GPU race on it.
static __device__ __align__(256) double2 g_work[kMaxEntries];
static __device__ __align__(256) unsigned char g_partial[8192];
static __device__ __align__(256) double g_scale[2];

struct Addresses {
    void* work = nullptr;
    void* partial = nullptr;
    void* scale = nullptr;
    bool ready = false;
};

Addresses g_addr[kMaxDevices];
std::mutex g_mu;

int fail(int code, const std::string& m) { return gx::set_error(code, m); }

// Device addresses of the scratch arrays on `device` (current).  Looked up
// again on every call made outside stream capture, so that a context
// re-created after cudaDeviceReset (which reloads this module and moves the
// arrays) is followed; under capture the addresses recorded by the last
// uncaptured call on the device are used, so the first call on a device must
// come before any stream capture.
int resolve(int device, cudaStream_t stream, Addresses& out) {
    std::lock_guard<std::mutex> lock(g_mu);
    Addresses& a = g_addr[device];
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(stream, &cap);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(GX_ECUDA, std::string("cudaStreamIsCapturing failed: ") + cudaGetErrorString(e));
    }
    if (cap == cudaStreamCaptureStatusNone) {
        Addresses fresh;
        e = cudaGetSymbolAddress(&fresh.work, g_work);
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&fresh.partial, g_partial);
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&fresh.scale, g_scale);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(GX_ECUDA, std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
        }
        fresh.ready = true;
        a = fresh;
    } else if (!a.ready) {
        return fail(GX_EINVAL, "gx_cholesky_step_noalloc: the first call on a device must come before stream capture");
    }
    out = a;
    return GX_OK;
}

}  // namespace

extern "C" int gx_cholesky_step_noalloc(const void* factors, int64_t rank, int64_t pivot, const void* column, int n,
                                        int real, double* residual, void* new_row, void* result, void* stream) {
    if (n <= 0) return fail(GX_EINVAL, "n must be positive");
    const long long N = (long long)n * n;
    if (N > kMaxEntries)
        return fail(GX_ELENGTH, "gx_cholesky_step_noalloc supports n*n <= " + std::to_string(kMaxEntries) +
                                    " ordered AO pairs (n <= 256); got n = " + std::to_string(n));
    if (rank < 0 || rank > N) return fail(GX_EINVAL, "rank must be in [0, n*n]");
    if (pivot < 0 || pivot >= N) return fail(GX_ERANGE, "Cholesky pivot index is out of range");
    if (!column || !residual || !new_row || !result || (rank > 0 && !factors))
        return fail(GX_EINVAL, "null device pointer");
    if ((size_t)gx::chol_partial_bytes() > sizeof(g_partial))
        return fail(GX_ECUDA, "reduction scratch is smaller than the kernels need");
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return fail(GX_ECUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (device < 0 || device >= kMaxDevices) return fail(GX_EINVAL, "device index out of range");
    Addresses a;
    if (int rc = resolve(device, static_cast<cudaStream_t>(stream), a)) return rc;
    e = gx::launch_chol_step(real != 0, factors, N, (int)rank, pivot, column, a.work, n, residual,
                             static_cast<double*>(a.scale), new_row, a.partial, result,
                             static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(GX_ECUDA, std::string("launch: ") + cudaGetErrorString(e));
    return GX_OK;
}
