// extern "C" entry points of libadrt_pinv_gb300.so (declared in include/adrt_pinv_gb300.h).
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "launch.h"

namespace adrt {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int cuda_status(cudaError_t e, const char* where) {
    if (e == cudaSuccess) return ADRT_OK;
    set_error("%s: %s", where, cudaGetErrorString(e));
    cudaGetLastError();  // consume a non-sticky error so that later, unrelated calls do not report it again
    return e == cudaErrorMemoryAllocation ? ADRT_ENOMEM : ADRT_ECUDA;
}

static std::atomic<long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int launch_status(const char* where) {
    count_launch();
    return cuda_status(cudaGetLastError(), where);
}

int launch_ex_status(cudaError_t launched, const char* where) {
    if (launched != cudaSuccess) {
        cudaGetLastError();  // the refusal is reported here; leave no stale error for the next launch
        return cuda_status(launched, where);
    }
    return launch_status(where);
}

int ensure_smem(const void* func, size_t bytes) {
    static std::mutex mu;
    static std::map<const void*, size_t> done;
    std::lock_guard<std::mutex> lock(mu);
    auto it = done.find(func);
    if (it != done.end() && it->second >= bytes) return ADRT_OK;
    int rc = cuda_status(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes),
                         "cudaFuncSetAttribute(MaxDynamicSharedMemorySize)");
    if (!rc) done[func] = bytes;
    return rc;
}

// device buffers for the host-pointer drop-ins: stream-ordered allocations on a private stream, freed on scope exit
struct Scratch {
    cudaStream_t st = nullptr;
    std::vector<void*> ptrs;
    int rc = ADRT_OK;
    Scratch() {
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) rc = cuda_status(cudaGetLastError(), "stream");
    }
    void* get(size_t bytes) {
        if (rc) return nullptr;
        void* p = nullptr;
        cudaError_t e = cudaMallocAsync(&p, bytes ? bytes : 16, st);
        if (e != cudaSuccess) {
            rc = cuda_status(e, "cudaMallocAsync");
            return nullptr;
        }
        ptrs.push_back(p);
        return p;
    }
    int h2d(void* d, const void* h, size_t bytes) {
        if (!rc && bytes) rc = cuda_status(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st), "H2D copy");
        return rc;
    }
    int d2h(void* h, const void* d, size_t bytes) {
        if (!rc && bytes) rc = cuda_status(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, st), "D2H copy");
        return rc;
    }
    int sync() {
        if (!rc) rc = cuda_status(cudaStreamSynchronize(st), "synchronize");
        return rc;
    }
    ~Scratch() {
        for (void* p : ptrs) cudaFreeAsync(p, st);
        if (st) {
            cudaStreamSynchronize(st);
            cudaStreamDestroy(st);
        }
    }
};

static int check_levels(const char* who, int n, int K, int m_lo, int m_hi) {
    if (n < 1 || n > 11) { set_error("%s: n=%d out of range 1..11", who, n); return ADRT_EINVAL; }
    if (K < 0) { set_error("%s: K=%d < 0", who, K); return ADRT_EINVAL; }
    if (m_lo < 1 || m_hi > n || m_lo > m_hi) {
        set_error("%s: levels [%d, %d] outside 1..%d", who, m_lo, m_hi, n);
        return ADRT_EINVAL;
    }
    return ADRT_OK;
}

// per-row coefficient table: a_k, then (omega_j, omega_j a_k, omega_j - 1), j = 1..d_k-1 (cpp/oblique.cpp:83-98)
static std::vector<double> coef_table(int K, const int* deg, const double* a, const double* c, int* stride) {
    int dmax = 1;
    for (int k = 0; k < K; ++k) dmax = deg[k] > dmax ? deg[k] : dmax;
    *stride = 1 + 3 * (dmax - 1);
    std::vector<double> tab((size_t)K * *stride, 0.0);
    for (int k = 0; k < K; ++k) {
        double* row = tab.data() + (size_t)k * *stride;
        row[0] = a[k];
        double om = 1.0;
        for (int j = 1; j < deg[k]; ++j) {
            om = (j == 1) ? 1.0 / (1.0 - c[k] * c[k] / 2.0) : 1.0 / (1.0 - c[k] * c[k] * om / 4.0);
            row[3 * j - 2] = om;
            row[3 * j - 1] = om * a[k];
            row[3 * j] = om - 1.0;
        }
    }
    return tab;
}

}  // namespace adrt

using namespace adrt;

extern "C" {

const char* adrt_last_error(void) { return g_err; }
long long adrt_launch_count(void) { return g_launches.load(); }
int adrt_abi_version(void) { return 1; }

int omp_max_threads(void) { return device_sm_count(); }

int bfly_rows(int n, int K, const double* z, double* X, int m_lo, int m_hi, int transpose, int nthreads) {
    (void)nthreads;
    int rc = check_levels("bfly_rows", n, K, m_lo, m_hi);
    if (rc) return rc;
    if (!K) return ADRT_OK;
    if (!z || !X) { set_error("bfly_rows: null pointer"); return ADRT_EINVAL; }
    const int N = 1 << n;
    Scratch s;
    const size_t xb = (size_t)K * N * 16;
    void* dz = s.get((size_t)K * 16);
    void* dX = s.get(xb);
    void* dtw = s.get((size_t)K * (N / 2 + 1) * 16);
    int32_t* cnt = (int32_t*)s.get(16);
    if (s.rc) return s.rc;
    if (s.h2d(dz, z, (size_t)K * 16) || s.h2d(dX, X, xb)) return s.rc;
    if ((rc = twiddle_table(ADRT_F64, n, K, (const double*)dz, dtw, s.st))) return rc;
    adrt_row_job J;
    memset(&J, 0, sizeof(J));
    J.dtype = ADRT_F64; J.n = n; J.nimg = 1; J.nsel = K; J.img_stride = 0; J.X = dX; J.rows = nullptr;
    J.freq_mod = K; J.roots = nullptr; J.twtab = dtw; J.nops = 1;
    J.op[0] = transpose ? ADRT_OP_BT : ADRT_OP_B; J.lo[0] = m_lo; J.hi[0] = m_hi;
    J.counter = cnt;
    if ((rc = rows_run(&J, 0, 0.0, nullptr, s.st))) return rc;
    if (s.d2h(X, dX, xb)) return s.rc;
    return s.sync();
}

int cheb_rows(int n, int K, const double* z, const int* deg, const double* a, const double* c, double tau, const double* Y,
              double* Z, int m_lo, int m_hi, int nthreads, long long* steps) {
    (void)nthreads;
    int rc = check_levels("cheb_rows", n, K, m_lo, m_hi);
    if (rc) return rc;
    if (!K) return ADRT_OK;
    if (!z || !deg || !a || !c || !Y || !Z) { set_error("cheb_rows: null pointer"); return ADRT_EINVAL; }
    const int N = 1 << n;
    int stride = 1;
    std::vector<double> coef = coef_table(K, deg, a, c, &stride);
    Scratch s;
    const size_t xb = (size_t)K * N * 16;
    void* dz = s.get((size_t)K * 16);
    void* dX = s.get(xb);
    void* dtw = s.get((size_t)K * (N / 2 + 1) * 16);
    void* dcoef = s.get(coef.size() * 8);
    void* ddeg = s.get((size_t)K * 4);
    int32_t* cnt = (int32_t*)s.get(16);
    if (s.rc) return s.rc;
    if (s.h2d(dz, z, (size_t)K * 16) || s.h2d(dX, Y, xb) || s.h2d(dcoef, coef.data(), coef.size() * 8) ||
        s.h2d(ddeg, deg, (size_t)K * 4))
        return s.rc;
    if ((rc = twiddle_table(ADRT_F64, n, K, (const double*)dz, dtw, s.st))) return rc;
    adrt_row_job J;
    memset(&J, 0, sizeof(J));
    J.dtype = ADRT_F64; J.n = n; J.nimg = 1; J.nsel = K; J.X = dX; J.freq_mod = K; J.twtab = dtw;
    J.deg = (const int32_t*)ddeg; J.coef = dcoef; J.coef_stride = stride; J.tau = tau;
    J.nops = 1; J.op[0] = ADRT_OP_P; J.lo[0] = m_lo; J.hi[0] = m_hi; J.counter = cnt;
    if ((rc = rows_run(&J, 0, 0.0, nullptr, s.st))) return rc;
    if (s.d2h(Z, dX, xb) || s.sync()) return s.rc;
    if (steps) {
        long long tot = 0;
        for (int k = 0; k < K; ++k)
            if (deg[k] > 1) tot += (long long)(deg[k] - 1) * 2 * (m_hi - m_lo + 1);
        *steps += tot;
    }
    return ADRT_OK;
}

int cert_rowsum(int n, int K, const double* omega, int m_lo, double* out, int nthreads) {
    (void)nthreads;
    if (n < 1 || n > 12 || K < 0 || m_lo < 1) { set_error("cert_rowsum: bad arguments (n <= 12)"); return ADRT_EINVAL; }
    if (!K) return ADRT_OK;
    if (!omega || !out) { set_error("cert_rowsum: null pointer"); return ADRT_EINVAL; }
    Scratch s;
    void* dom = s.get((size_t)K * 8);
    void* dout = s.get((size_t)K * 8);
    if (s.rc || s.h2d(dom, omega, (size_t)K * 8)) return s.rc;
    int rc = cert_rowsum_dev(n, K, (const double*)dom, m_lo, (double*)dout, s.st);
    if (rc) return rc;
    if (s.d2h(out, dout, (size_t)K * 8)) return s.rc;
    return s.sync();
}

int adrt_rows_run(const adrt_row_job* job, void* stream) {
    return rows_run(job, 0, 0.0, nullptr, as_stream(stream));
}

int adrt_twiddle_table(int dtype, int n, int K, const double* z, void* tab, void* stream) {
    return twiddle_table(dtype, n, K, z, tab, as_stream(stream));
}

int adrt_power_rows(int dtype, int n, int K, void* V, const void* twtab, int m_lo, int iters, double safety, double* out,
                    int32_t* counter, void* stream) {
    int rc = check_levels("power_rows", n, K, m_lo, n);
    if (rc) return rc;
    if (!K) return ADRT_OK;
    if (!V || !twtab || !out || !counter || iters < 0) { set_error("power_rows: bad arguments"); return ADRT_EINVAL; }
    cudaStream_t st = as_stream(stream);
    adrt_row_job J;
    memset(&J, 0, sizeof(J));
    J.dtype = dtype; J.n = n; J.nimg = 1; J.nsel = K; J.X = V; J.freq_mod = K; J.twtab = twtab;
    J.nops = 1; J.op[0] = 16 /* power iteration */; J.lo[0] = m_lo; J.hi[0] = n; J.counter = counter;
    return rows_run(&J, iters, safety, out, st);
}

int adrt_cert_rowsum_dev(int n, int K, const double* omega, int m_lo, double* out, void* stream) {
    return cert_rowsum_dev(n, K, omega, m_lo, out, as_stream(stream));
}

int adrt_pack_fft(int dtype, int n, int nimg, int src_kind, int src_dtype, const void* src, long long src_stride,
                  void* Y, const void* roots, int cols, void* stream) {
    return pack_fft(dtype, n, nimg, src_kind, src_dtype, src, src_stride, Y, roots, cols, as_stream(stream));
}

int adrt_ifft_unpack(int dtype, int n, int nimg, const void* Z, void* colpart, void* rowpart0, void* rowpart3,
                     const void* roots, int cols, void* stream) {
    return ifft_unpack(dtype, n, nimg, Z, colpart, rowpart0, rowpart3, roots, cols, as_stream(stream));
}

int adrt_resid(int dtype, int n, int nimg, int ydtype, const void* y, const void* p0, const void* p1, const void* p2,
               void* s, void* stream) {
    return image_resid(dtype, n, nimg, ydtype, y, p0, p1, p2, s, as_stream(stream));
}

int adrt_g1_step(int dtype, int n, int nimg, const void* s, const void* x, const void* xp, void* xn, double om_a,
                 double om_1, double a0, void* stream) {
    return image_g1_step(dtype, n, nimg, s, x, xp, xn, om_a, om_1, a0, as_stream(stream));
}

int adrt_lorr(int dtype, int n, int nimg, const void* s, void* out, void* stream) {
    return image_lorr(dtype, n, nimg, s, out, as_stream(stream));
}

int adrt_outer_update(int dtype, int n, int nimg, const void* x, const void* x_prev, const void* r, int rdtype,
                      void* x_new, double om_a, double om_1, double a0, const double* om_img, void* stream) {
    return image_outer(dtype, n, nimg, x, x_prev, r, rdtype, x_new, om_a, om_1, a0, om_img, as_stream(stream));
}

int adrt_sum3(int dtype, int n, int nimg, const void* p0, const void* p1, const void* p2, void* out, int out_dtype,
              void* stream) {
    return image_sum3(dtype, n, nimg, p0, p1, p2, out, out_dtype, as_stream(stream));
}

int adrt_outer_step(int dtype, int parts_dtype, int n, int nimg, const double* y, const void* p0, const void* p1,
                    const void* p2, const double* x, const double* x_prev, double* x_new, double om_a, double om_1,
                    double a0, int precond, int g1_deg, const double* g1_coef, const double* om_img, int band,
                    void* stream) {
    return outer_step(dtype, parts_dtype, n, nimg, y, p0, p1, p2, x, x_prev, x_new, om_a, om_1, a0, precond, g1_deg,
                      g1_coef, om_img, band, as_stream(stream));
}

int adrt_outer_step_max_n(int dtype) { return outer_step_max_n(dtype); }

int adrt_outer_step_ff(int n, int nimg, const float* y, const float* p0, const float* p1, const float* p2,
                       const float* x, const float* x_prev, float* x_new, double om_a, double om_1, double a0,
                       int precond, int g1_deg, const double* g1_coef, const double* om_img, int band, void* stream) {
    return outer_step_ff(n, nimg, y, p0, p1, p2, x, x_prev, x_new, om_a, om_1, a0, precond, g1_deg, g1_coef, om_img,
                         band, as_stream(stream));
}

int adrt_ff_to_f64(int n, int nimg, const float* x, double* out, void* stream) {
    return ff_to_f64(n, nimg, x, out, as_stream(stream));
}

int adrt_dense_rows(int dtype, int n, int nimg, int nrows, const int32_t* rows, const void* W, void* Y,
                    long long img_stride, void* Zd, int32_t* err, int use_tc, int tile, void* stream) {
    return dense_rows(dtype, n, nimg, nrows, rows, W, Y, img_stride, Zd, err, use_tc, tile, as_stream(stream));
}

int adrt_dense_split(int n, int nrows, const void* W, void* Ws, void* stream) {
    return dense_split(n, nrows, W, Ws, as_stream(stream));
}

int adrt_forward(int dtype, int n, int nimg, const void* x, void* b, void* scratch, void* stream) {
    return adrt_fwd(dtype, n, nimg, x, b, scratch, as_stream(stream));
}

int adrt_transpose(int dtype, int n, int nimg, const void* b, void* x, void* scratch, void* stream) {
    return adrt_adj(dtype, n, nimg, b, x, scratch, as_stream(stream));
}

// FP32 FMA throughput probe: every thread runs `iters` rounds of 8 independent FMA chains (16 flop per chain and
// round); out receives one value per thread so the work cannot be elided.
__global__ void fma_probe_kernel(int iters, float seed, float* out) {
    float a[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = seed + threadIdx.x * 1e-7f + i;
    const float m = 0.999999f, c = 1e-7f;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int r = 0; r < 8; ++r) {
#pragma unroll
            for (int i = 0; i < 8; ++i) a[i] = fmaf(a[i], m, c);
        }
    }
    float s = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += a[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

int adrt_fp32_probe(int blocks, int threads, int iters, float* out, void* stream) {
    if (blocks < 1 || threads < 32 || threads > 1024 || iters < 1 || !out) { set_error("fp32_probe: bad arguments"); return ADRT_EINVAL; }
    fma_probe_kernel<<<blocks, threads, 0, as_stream(stream)>>>(iters, 1.0f, out);
    return launch_status("fma_probe_kernel");
}

}  // extern "C"
