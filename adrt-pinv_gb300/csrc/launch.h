// Host-side launchers shared between the translation units of the library (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>

#include "adrt_pinv_gb300.h"

namespace adrt {
int device_sm_count();
int rows_run(const adrt_row_job* J, int power_iters, double power_safety, double* power_out, cudaStream_t st);
int twiddle_table(int dtype, int n, int K, const double* z, void* tab, cudaStream_t st);
int pack_fft(int dtype, int n, int nimg, int src_kind, int src_dtype, const void* src, long long src_stride, void* Y,
             const void* roots, int cols, cudaStream_t st);
int ifft_unpack(int dtype, int n, int nimg, const void* Z, void* colpart, void* row0, void* row3, const void* roots,
                int cols, cudaStream_t st);
int image_resid(int dtype, int n, int nimg, int ydtype, const void* y, const void* p0, const void* p1, const void* p2,
                void* s, cudaStream_t st);
int image_sum3(int dtype, int n, int nimg, const void* p0, const void* p1, const void* p2, void* out, int out_dtype,
               cudaStream_t st);
int image_g1_step(int dtype, int n, int nimg, const void* s, const void* x, const void* xp, void* xn, double om_a,
                  double om_1, double a0, cudaStream_t st);
int image_lorr(int dtype, int n, int nimg, const void* s, void* out, cudaStream_t st);
int image_outer(int dtype, int n, int nimg, const void* x, const void* xp, const void* r, int rdtype, void* xn,
                double om_a, double om_1, double a0, const double* om_img, cudaStream_t st);
// set the dynamic shared-memory limit of a kernel once per size (safe to call before and during stream capture)
int ensure_smem(const void* func, size_t bytes);
// spatial ADRT levels; active (nullable): images with active[img] == 0 are skipped
int adrt_fwd(int dtype, int n, int nimg, const void* x, void* b, void* scratch, cudaStream_t st,
             const int* active = nullptr);
int adrt_adj(int dtype, int n, int nimg, const void* b, void* x, void* scratch, cudaStream_t st,
             const int* active = nullptr);
int outer_step(int dtype, int parts_dtype, int n, int nimg, const double* y, const void* p0, const void* p1,
               const void* p2, const double* x, const double* xp, double* xn, double om_a, double om_1, double a0,
               int precond, int g1_deg, const double* g1_coef, const double* om_img, int band, cudaStream_t st);
int outer_step_max_n(int dtype);
int outer_step_ff(int n, int nimg, const float* y, const float* p0, const float* p1, const float* p2, const float* x,
                  const float* xp, float* xn, double om_a, double om_1, double a0, int precond, int g1_deg,
                  const double* g1_coef, const double* om_img, int band, cudaStream_t st);
int ff_to_f64(int n, int nimg, const float* x, double* out, cudaStream_t st);
int dense_rows(int dtype, int n, int nimg, int nrows, const int* rows, const void* W, void* Y, long long img_stride,
               void* Zd, int* err, int use_tc, int tile, cudaStream_t st);
int dense_split(int n, int nrows, const void* W, void* Ws, cudaStream_t st);
int cert_rowsum_dev(int n, int K, const double* omega, int m_lo, double* out, cudaStream_t st);
}  // namespace adrt
