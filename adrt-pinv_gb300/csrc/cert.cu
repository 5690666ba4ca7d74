// Certified spectral bounds Lambda_k >= lambda_max(M_k) by the row-sum recursion (reference: cpp/oblique.cpp:106-130,
// fasthybrid.cert_rowsum_levels fasthybrid.py:134-150). One CTA per frequency; the recursion arrays live in shared
// memory in FP64: r_m(a) = |1+z^a| r(2a) + max(|1+z^(a+1)| r(2a+1), |1+z^(a-1)| r(2a-1)), |a| <= 2^(n-m) - 1.
#include "common.cuh"
#include "launch.h"

namespace adrt {

__global__ void cert_kernel(int n, int K, const double* __restrict__ omega, int m_lo, double* __restrict__ out) {
    extern __shared__ double sm[];
    const long A = 1L << n;
    double* r = sm;
    double* rn = sm + 2 * A + 1;
    for (int k = blockIdx.x; k < K; k += gridDim.x) {
        const double om = omega[k];
        for (long i = threadIdx.x; i <= 2 * A; i += blockDim.x) r[i] = 1.0;
        __syncthreads();
        for (int m = m_lo; m <= n; ++m) {
            const long amax = (1L << (n - m)) - 1;
            for (long a = -amax + threadIdx.x; a <= amax; a += blockDim.x) {
                const double t0 = 2.0 * fabs(cos(0.5 * om * (double)a)) * r[2 * a + A];
                const double tp = 2.0 * fabs(cos(0.5 * om * (double)(a + 1))) * r[2 * a + 1 + A];
                const double tm = 2.0 * fabs(cos(0.5 * om * (double)(a - 1))) * r[2 * a - 1 + A];
                rn[a + A] = t0 + (tp > tm ? tp : tm);
            }
            __syncthreads();
            double* s = r; r = rn; rn = s;
        }
        if (threadIdx.x == 0) out[k] = r[A];
        __syncthreads();
    }
}

int cert_rowsum_dev(int n, int K, const double* omega, int m_lo, double* out, cudaStream_t st) {
    if (n < 1 || n > 12 || K < 0 || m_lo < 1 || (K && (!omega || !out))) {
        set_error("cert_rowsum: bad arguments (n=%d K=%d m_lo=%d)", n, K, m_lo);
        return ADRT_EINVAL;
    }
    if (!K) return ADRT_OK;
    const size_t smem = 2 * (size_t)(2 * (1L << n) + 1) * sizeof(double);
    if (int rc = ensure_smem((const void*)cert_kernel, smem)) return rc;
    int grid = K < 4096 ? K : 4096;
    cert_kernel<<<grid, 256, smem, st>>>(n, K, omega, m_lo, out);
    return launch_status("cert_kernel");
}

}  // namespace adrt
