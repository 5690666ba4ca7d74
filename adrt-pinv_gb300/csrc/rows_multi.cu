// Several row-program jobs in ONE persistent launch: the polynomial rows of many inverses of different sizes N and
// op lists (the classes of an uneven batch, each with its own rows, degrees, tables and images) share one work
// queue. The jobs' rows are split into warp items (the rows one warp processes at a time: 32/T rows of a job, T lanes
// per row) and concatenated in the caller's order (costliest job first); every warp of the persistent grid takes the
// next warp item from a single atomic counter, finds its job by the prefix offsets (held in shared memory) and runs
// the compile-time program of that job's size and op list (rows_core.cuh), so no job waits for another to finish
// and the tail of one size is filled by the rows of the others. Sizes n = 6..9 (one warp or less per row), FP32.
#include "rows_core.cuh"

namespace adrt {

constexpr int MULTI_THREADS = 256;
constexpr int MULTI_MAX_JOBS = 128;
constexpr int MULTI_NMIN = 6, MULTI_NMAX = 9;

// complex elements of shared memory per warp: the largest (groups per warp x group size) of the supported sizes
template <int n> constexpr int warp_slot_of() { return (32 / FastCfg<n>::T) * FastCfg<n>::GS; }
constexpr int MULTI_WARP_SLOT = imax(imax(warp_slot_of<6>(), warp_slot_of<7>()), imax(warp_slot_of<8>(), warp_slot_of<9>()));

template <int n, int PROG>
__device__ __noinline__ void multi_item(const adrt_row_job& J, int local, float2* wbuf, int lane) {
    using F = FastCfg<n>;
    static_assert(F::WPG == 1, "one warp or less per row");
    constexpr int T = F::T, GPW = 32 / T;
    const int giw = T >= 32 ? 0 : lane / T;
    const int u = lane & (T - 1);
    const int item = local * GPW + giw;
    const unsigned gm = (T >= 32) ? 0xffffffffu : (((1u << T) - 1u) << (giw * T));
    TwSrc<float> tw;
    tw.roots = reinterpret_cast<const float2*>(J.roots);
    tw.tab = reinterpret_cast<const float2*>(J.twtab);
    tw.Lmask = (2 << n) - 1;
    tw.tstride = (1 << n) / 2 + 1;
    if (item < J.nimg * J.nsel) prog_item<float, n, PROG>(J, tw, item, wbuf + giw * F::GS, u, gm);
}

#define ADRT_MULTI_CASE(nn)                                                         \
    case nn * 8 + PROG_GH_HYB: multi_item<nn, PROG_GH_HYB>(J, local, wbuf, lane); break;   \
    case nn * 8 + PROG_BP_HYB: multi_item<nn, PROG_BP_HYB>(J, local, wbuf, lane); break;   \
    case nn * 8 + PROG_FRAME_LP: multi_item<nn, PROG_FRAME_LP>(J, local, wbuf, lane); break; \
    case nn * 8 + PROG_BP_LP: multi_item<nn, PROG_BP_LP>(J, local, wbuf, lane); break;

// jobs[j] with code[j] = n * 8 + program; wstart[j] = first warp item of job j (wstart[njobs] = total)
__global__ void __launch_bounds__(MULTI_THREADS, 1)
    rows_multi_kernel(const adrt_row_job* __restrict__ jobs, const int* __restrict__ code,
                      const int* __restrict__ wstart, int njobs, int* __restrict__ counter) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_start[MULTI_MAX_JOBS + 1];
    __shared__ int s_code[MULTI_MAX_JOBS];
    for (int j = threadIdx.x; j <= njobs; j += MULTI_THREADS) {
        s_start[j] = wstart[j];
        if (j < njobs) s_code[j] = code[j];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float2* wbuf = reinterpret_cast<float2*>(smem_raw) + (size_t)warp * MULTI_WARP_SLOT;
    const int total = s_start[njobs];
    for (;;) {
        int w = 0;
        if (lane == 0) w = atomicAdd(counter, 1);
        w = __shfl_sync(0xffffffffu, w, 0);
        if (w >= total) break;
        int j = 0;
        while (s_start[j + 1] <= w) ++j;
        const int local = w - s_start[j];
        const adrt_row_job& J = jobs[j];
        switch (s_code[j]) {
            ADRT_MULTI_CASE(6)
            ADRT_MULTI_CASE(7)
            ADRT_MULTI_CASE(8)
            ADRT_MULTI_CASE(9)
            default: break;
        }
    }
}

}  // namespace adrt

using namespace adrt;

extern "C" int adrt_rows_multi_code(const adrt_row_job* J) {
    if (!J || J->dtype != ADRT_F32 || J->n < MULTI_NMIN || J->n > MULTI_NMAX || J->rows == nullptr || !J->roots) {
        return -1;
    }
    const int prog = match_prog(*J);
    if (!prog) return -1;
    return J->n * 8 + prog;
}

extern "C" int adrt_rows_lanes_per_row(int n) {
    switch (n) {
        case 6: return FastCfg<6>::T;
        case 7: return FastCfg<7>::T;
        case 8: return FastCfg<8>::T;
        case 9: return FastCfg<9>::T;
    }
    return -1;
}

extern "C" int adrt_rows_run_multi(const adrt_row_job* jobs, const int32_t* code, const int32_t* wstart, int njobs,
                                   int32_t* counter, int grid, void* stream) {
    if (njobs < 1 || njobs > MULTI_MAX_JOBS || !jobs || !code || !wstart || !counter) {
        set_error("rows_multi: bad arguments (njobs=%d, at most %d)", njobs, MULTI_MAX_JOBS);
        return ADRT_EINVAL;
    }
    cudaStream_t st = as_stream(stream);
    const size_t smem = (size_t)(MULTI_THREADS / 32) * MULTI_WARP_SLOT * sizeof(float2);
    if (int rc = ensure_smem((const void*)rows_multi_kernel, smem)) return rc;
    if (int rc = cuda_status(cudaMemsetAsync(counter, 0, sizeof(int32_t), st), "rows_multi counter reset")) return rc;
    const int g = grid > 0 ? grid : device_sm_count();
    rows_multi_kernel<<<g, MULTI_THREADS, smem, st>>>(jobs, code, wstart, njobs, counter);
    return launch_status("rows_multi_kernel");
}
