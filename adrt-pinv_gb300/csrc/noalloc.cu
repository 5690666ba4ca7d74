// bfly_rows on device pointers for callers that cannot allocate device memory.
//
// Who needs it: a process that hands all of a GPU's memory to its own pool at start-up (a serving process that
// reserves HBM once and never lets a library allocate), code that must not call cudaMalloc / cudaFree because those
// can synchronize the device and stall its other streams, and callers on threads where entering the CUDA allocator
// is not allowed (host callbacks, some foreign-function runtimes). The host-pointer bfly_rows allocates its device
// buffers; this entry point instead takes the rows and frequencies already on the device and keeps its own scratch
// (the per-row twiddle table and the work counter of the row kernel) in a fixed array of the library's device
// memory, so that it calls no allocator at all.
//
// Limits and rules, for the caller:
//   * the array is kNoAllocScratchBytes = 4 MiB on every GPU that loads the library, held until the process exits;
//     a call needs 256 + K (N/2 + 1) 16 bytes of it and is rejected (ADRT_EINVAL) above that;
//   * the first call on a device looks up the array's device address (cudaGetSymbolAddress) with that device
//     current; make that first call before any stream capture. The address is cached for the life of the
//     device's context: after cudaDeviceReset (or anything else that destroys and recreates the primary context)
//     the cached address is stale, so a process that resets a device must not call this entry point again;
//   * every call shares the one array and leaves its contents behind; the twiddle table is rewritten and the counter
//     is reset (stream-ordered memset) by each call, so nothing stale is read, but two calls whose work overlaps on
//     the GPU (different streams, no ordering between them) race on the array and give wrong results.
#include <mutex>

#include "common.cuh"
#include "launch.h"

namespace adrt {

constexpr size_t kNoAllocScratchBytes = 4u << 20;
constexpr size_t kCounterSlot = 256;  // the work counter, then the twiddle table at a 256-byte boundary
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
static void* g_scratch_addr[kMaxDevices];
static std::mutex g_scratch_mu;

// device address of g_noalloc_scratch on the current device (looked up once per device)
static int scratch_address(void** out) {
    int dev = 0;
    if (int rc = cuda_status(cudaGetDevice(&dev), "cudaGetDevice")) return rc;
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("bfly_rows_noalloc: device %d beyond the %d supported", dev, kMaxDevices);
        return ADRT_EUNSUPPORTED;
    }
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        if (int rc = cuda_status(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(scratch)")) return rc;
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return ADRT_OK;
}

}  // namespace adrt

using namespace adrt;

extern "C" int adrt_bfly_rows_noalloc(int n, int K, const double* z, double* X, int m_lo, int m_hi, int transpose,
                                      void* stream) {
    if (n < 1 || n > 11 || K < 0 || m_lo < 1 || m_hi > n || m_lo > m_hi) {
        set_error("bfly_rows_noalloc: bad arguments (n=%d K=%d levels [%d, %d])", n, K, m_lo, m_hi);
        return ADRT_EINVAL;
    }
    if (!K) return ADRT_OK;
    if (!z || !X) { set_error("bfly_rows_noalloc: null pointer"); return ADRT_EINVAL; }
    const size_t N = (size_t)1 << n;
    const size_t need = kCounterSlot + (size_t)K * (N / 2 + 1) * 16;
    if (need > kNoAllocScratchBytes) {
        set_error("bfly_rows_noalloc: K=%d rows of N=%zu need %zu bytes of scratch, the fixed array holds %zu "
                  "(K * (N/2 + 1) <= %zu)", K, N, need, kNoAllocScratchBytes, (kNoAllocScratchBytes - kCounterSlot) / 16);
        return ADRT_EINVAL;
    }
    if ((reinterpret_cast<uintptr_t>(X) & 15) || (reinterpret_cast<uintptr_t>(z) & 15)) {
        set_error("bfly_rows_noalloc: z and X must be 16-byte aligned");
        return ADRT_EINVAL;
    }
    void* base = nullptr;
    if (int rc = scratch_address(&base)) return rc;
    cudaStream_t st = as_stream(stream);
    int32_t* counter = reinterpret_cast<int32_t*>(base);
    void* table = static_cast<unsigned char*>(base) + kCounterSlot;
    if (int rc = twiddle_table(ADRT_F64, n, K, z, table, st)) return rc;
    adrt_row_job J = {};
    J.dtype = ADRT_F64;
    J.n = n;
    J.nimg = 1;
    J.nsel = K;
    J.X = X;
    J.freq_mod = K;
    J.twtab = table;
    J.nops = 1;
    J.op[0] = transpose ? ADRT_OP_BT : ADRT_OP_B;
    J.lo[0] = m_lo;
    J.hi[0] = m_hi;
    J.counter = counter;  // reset by rows_run with a stream-ordered memset
    return rows_run(&J, 0, 0.0, nullptr, st);
}
