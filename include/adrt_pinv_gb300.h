/* C ABI of the GB300 (sm_103a) implementation of the explicit oblique inverses of the ADRT.
 *
 * Two groups of entry points:
 *  1. Drop-in replacements for the reference's native row kernels, cpp/oblique.cpp of dsrim/adrt-pinv, with the
 *     same names, argument order and meaning (the reference binds them with ctypes at fastcpp.py:22-32). They
 *     take HOST pointers, copy to the GPU, run the CUDA kernels and copy back before returning. The reference
 *     returns void; these return an int status (0 = ok), which a binding with restype None simply ignores.
 *     Complex arrays are interleaved (re, im) doubles, C-contiguous rows of N = 2^n values.
 *  2. Device-pointer entry points used by the Python host (adrt-pinv_gb300/): stream-ordered, asynchronous,
 *     no allocation inside (scratch comes from the caller), FP32 or FP64 data. `stream` is a cudaStream_t
 *     passed as void* (NULL = legacy default stream).
 * All functions return ADRT_OK or an error code; adrt_last_error() gives a message for the calling thread.
 */
#ifndef ADRT_PINV_GB300_H
#define ADRT_PINV_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ADRT_OK 0
#define ADRT_EINVAL 1       /* bad argument (shape, range, null pointer) */
#define ADRT_ECUDA 2       /* CUDA runtime or launch error */
#define ADRT_ENOMEM 3      /* device allocation failed */
#define ADRT_EUNSUPPORTED 4

#define ADRT_F32 0
#define ADRT_F64 1
#define ADRT_I32 2
#define ADRT_I64 3
#define ADRT_F32X2 4 /* float-float: the unevaluated sum of two FP32 values, about 48 significant bits (stencils) */

/* row-program operations (the op lists of fastops.RowEngine.run, fastops.py:156-167) */
#define ADRT_OP_B 0  /* forward butterflies B_hi ... B_lo */
#define ADRT_OP_BT 1 /* adjoint butterflies */
#define ADRT_OP_M 2  /* B then BT over the same levels (M = B^* B) */
#define ADRT_OP_P 3  /* Chebyshev filter p_k(M) over levels lo..hi */
#define ADRT_MAX_OPS 8

/* ------------------------------------------------------------------ 1. reference drop-ins (host pointers) */

/* cpp/oblique.cpp:56 bfly_rows: X (K x N complex) in place; transpose = 0: B_{m_hi}...B_{m_lo}, 1: adjoint.
 * z: K complex frequencies z_k. nthreads is accepted and ignored (the GPU supplies the parallelism). */
int bfly_rows(int n, int K, const double* z, double* X, int m_lo, int m_hi, int transpose, int nthreads);

/* cpp/oblique.cpp:74 cheb_rows: Z[k] = p_k(M) Y[k] with deg[k] Chebyshev steps, constants a[k], c[k]
 * (fastspec.cheb_coeffs), shift tau, M = B^* B over levels m_lo..m_hi. steps (nullable) += level-rows applied. */
int cheb_rows(int n, int K, const double* z, const int* deg, const double* a, const double* c, double tau,
              const double* Y, double* Z, int m_lo, int m_hi, int nthreads, long long* steps);

/* cpp/oblique.cpp:108 cert_rowsum: certified bounds Lambda_k >= lambda_max(M_k), levels m_lo..n, K frequencies. */
int cert_rowsum(int n, int K, const double* omega, int m_lo, double* out, int nthreads);

/* cpp/oblique.cpp:132 omp_max_threads: here the number of SMs of the current device (the row parallelism). */
int omp_max_threads(void);

/* bfly_rows on DEVICE pointers for callers that cannot allocate device memory (a process that gives all GPU memory
 * to its own pool, code that must not let cudaMalloc/cudaFree synchronize the device, threads that may not enter the
 * CUDA allocator). No counterpart in the reference. Same arguments and result as bfly_rows, with z (K complex128)
 * and X (K x N complex128, transformed in place) in device memory, 16-byte aligned, ordered on `stream`. It calls no
 * allocator: its scratch (twiddle table + work counter) is a fixed 4 MiB device array held by every GPU that loads
 * the library until exit; calls needing more than 256 + 16 K (N/2 + 1) bytes of it are rejected with ADRT_EINVAL.
 * The first call on a device looks the array's address up (cudaGetSymbolAddress): make it before any stream capture.
 * All calls share the array: calls that overlap on the GPU race on it. */
int adrt_bfly_rows_noalloc(int n, int K, const double* z, double* X, int m_lo, int m_hi, int transpose, void* stream);

/* message of the last error on the calling thread ("" if none) */
const char* adrt_last_error(void);
/* library ABI version */
int adrt_abi_version(void);
/* number of CUDA kernels the library has launched so far (all threads); for launch accounting */
long long adrt_launch_count(void);
/* measurement utility: FP32 FMA throughput probe, blocks x threads threads each doing iters x 64 dependent-free
 * FMAs (128 flop per thread and iteration); out: blocks*threads floats (device). Used to measure the FP32 peak
 * that bounds the row engine. */
int adrt_fp32_probe(int blocks, int threads, int iters, float* out, void* stream);

/* ------------------------------------------------------------------ 2. device entry points */

/* One launch of the row engine over nimg images x nsel selected rows (fastops.RowEngine.run /
 * fastcpp.CppEngine._B/_BT/_P, fastops.py:70-167, fastcpp.py:62-99). Every selected row runs the same op list.
 * Rows are processed in the given order (callers sort by cost, descending) by persistent warps that take work
 * from *counter; the call resets *counter to 0 on the stream before the launch. Rows are read and written in
 * natural (logical) order whatever the op list. */
typedef struct adrt_row_job {
    int dtype;              /* ADRT_F32 / ADRT_F64: precision of X, twiddles and coefficients */
    int n;                  /* N = 2^n values per row, 1 <= n <= 11 */
    int nimg;               /* images in the batch */
    int nsel;               /* selected rows per image */
    int64_t img_stride;     /* complex elements between consecutive images of X */
    void* X;                /* rows (complex interleaved, row stride N), transformed in place */
    const int32_t* rows;    /* nsel row indices (row r of image b is X + b*img_stride + r*N) */
    int freq_mod;           /* frequency index of row r: k = r % freq_mod */
    const void* roots;      /* twiddle mode 0: L = 2N roots of unity exp(2 pi i j / L) (z_k = root[k]), or NULL */
    const void* twtab;      /* twiddle mode 1 (roots == NULL): per-row table z^t, t = 0..N/2, row stride N/2+1 */
    const int32_t* deg;     /* per frequency inner degree d_k (ADRT_OP_P) */
    const void* coef;       /* per frequency: a_k, then (omega_j, omega_j a_k, omega_j - 1) for j = 1..d_k-1 */
    int coef_stride;        /* elements per frequency in coef */
    double tau;             /* Tikhonov shift of the filter */
    int nops;
    int op[ADRT_MAX_OPS], lo[ADRT_MAX_OPS], hi[ADRT_MAX_OPS];
    int32_t* counter;       /* device int used as the work counter */
    int grid;               /* persistent CTAs (0 = one per SM) */
} adrt_row_job;

int adrt_rows_run(const adrt_row_job* job, void* stream);

/* The same op lists on FP32 rows (dtype ADRT_F32) in float-float arithmetic (compensated rows, about 48 significant
 * bits on the FP32 pipe), for the high-condition low-frequency rows where the FP32 filter loses accuracy
 * (cpp/oblique.cpp:74-104 evaluated in extended precision). Here `roots` (mode 0 only) holds the L roots of unity in
 * FP64 (complex128) and `coef` the filter table in FP64; rows are read and written in FP32. */
int adrt_rows_ff_run(const adrt_row_job* job, void* stream);

/* Several row jobs in ONE persistent launch (the polynomial rows of many inverses of different N and op lists, e.g.
 * the classes of an uneven batch; the reference runs one RowEngine.run per image, fastops.py:156-167). jobs: njobs
 * DEVICE-resident job structs; code[j] = adrt_rows_multi_code(job j) (FP32, n = 6..9, a compile-time op list, a row
 * selection, roots of unity; -1 when the job cannot join); wstart[j] = the first warp item of job j, wstart[njobs]
 * the total, where job j has ceil(nimg * nsel / (32 / adrt_rows_lanes_per_row(n))) warp items (device int arrays).
 * Every warp of the grid (0: one CTA per SM) takes warp items from the one counter (reset here). */
int adrt_rows_multi_code(const adrt_row_job* job);
int adrt_rows_lanes_per_row(int n);
int adrt_rows_run_multi(const adrt_row_job* jobs, const int32_t* code, const int32_t* wstart, int njobs,
                        int32_t* counter, int grid, void* stream);

/* Per-row twiddle table tab[k*(N/2+1) + t] = z_k^t (t = 0..N/2) from K complex z (FP64 in, dtype out),
 * by binary powering in FP64. */
int adrt_twiddle_table(int dtype, int n, int K, const double* z, void* tab, void* stream);

/* Power iteration for Lambda_k (fastcpp.py:102-118): V (K x N, dtype) is iterated `iters` times
 * V <- M V / ||M V|| row-wise (M = B^* B over levels m_lo..n) and out[k] = safety * Re <V_k, M V_k> (FP64 out).
 * Twiddles from the K x (N/2+1) table twtab. */
int adrt_power_rows(int dtype, int n, int K, void* V, const void* twtab, int m_lo, int iters, double safety,
                    double* out, int32_t* counter, void* stream);

/* cert_rowsum on device pointers (cpp/oblique.cpp:108-130). */
int adrt_cert_rowsum_dev(int n, int K, const double* omega, int m_lo, double* out, void* stream);

/* Quadrant packing + FFT along the offset axis (fastops._packed, fastops.py:209-214): for each image, the two
 * pairs (0,1), (2,3) of quadrant strips s_qa + i s_qb are transformed with a length L = 2N DFT along axis 0 into
 * Y (nimg x 2L x N complex, dtype). src_kind 0: src is nimg images N x N (real, src_dtype), strips = Tq(q, E x)
 * (fastspec.py:142-152); src_kind 1: src is nimg sinograms 4 x (2N-1) x N, strips = iota(b_q) (fastspec.py:170-174).
 * roots: L roots of unity in dtype. src_stride (src_kind 0): elements from one image to the next (0: N*N; e.g.
 * 2 N*N to read the hi planes of float-float images). cols: strip columns per CTA (0: the default). */
int adrt_pack_fft(int dtype, int n, int nimg, int src_kind, int src_dtype, const void* src, long long src_stride,
                  void* Y, const void* roots, int cols, void* stream);

/* Inverse FFT along the offset axis + unpacking (fastops.py:216-220): from Z (nimg x 2L x N complex) produce the
 * three image-space partial sums whose total is E^T sum_q T_q^T Re/Im(ifft Z) (fastspec.py:154-168):
 * colpart (quadrants II, III), rowpart0 (quadrant I) and rowpart3 (quadrant IV), each nimg x N x N, dtype real. */
int adrt_ifft_unpack(int dtype, int n, int nimg, const void* Z, void* colpart, void* rowpart0, void* rowpart3,
                     const void* roots, int cols, void* stream);
/* cols (both): strip columns per CTA, 0 for the default (as many as fit, up to 16 in FP32 and 8 in FP64) or a
 * quarter of the default (narrower CTAs, more of them per SM); other values are rejected. */

/* Image-space kernels on nimg N x N images (dtype = ADRT_F32 / ADRT_F64 for all image arguments).
 * resid:   s = y - (p0 + p1 + p2)  (y in ydtype; parts in dtype, all NULL = 0, which casts y; s in dtype)
 * g1_step: one step of cheb_solve(G1_apply, s, 4, 16, deg) (fasthybrid.py:95-130): with G1 x = 8x + J K x + (J K x^T)^T,
 *          xn = x + om_a*(s - G1 x) + om_1*(x - xp); first step (xp == NULL, x == NULL): xn = a*s.
 * lorr:    out = (s - Pi s)/4 + Pi s/12 (fasthybrid.py:101-111).
 * outer:   x_new = x + om_a * r + om_1 * (x - x_prev) (fastops.py:247-258); x, x_prev, x_new in dtype, r in
 *          rdtype (no wider than dtype); x == NULL: x_new = a0 * r; x_prev == NULL: zero. */
int adrt_resid(int dtype, int n, int nimg, int ydtype, const void* y, const void* p0, const void* p1, const void* p2,
               void* s, void* stream);
int adrt_g1_step(int dtype, int n, int nimg, const void* s, const void* x, const void* xp, void* xn, double om_a,
                 double om_1, double a0, void* stream);
int adrt_lorr(int dtype, int n, int nimg, const void* s, void* out, void* stream);
int adrt_outer_update(int dtype, int n, int nimg, const void* x, const void* x_prev, const void* r, int rdtype,
                      void* x_new, double om_a, double om_1, double a0, const double* om_img, void* stream);
int adrt_sum3(int dtype, int n, int nimg, const void* p0, const void* p1, const void* p2, void* out, int out_dtype,
              void* stream);

/* One fused outer step (fastops._outer, fastops.py:247-258, with P of fasthybrid.py:101-130):
 *   s = y - (p0 + p1 + p2) (parts in parts_dtype, F32 or F64; all NULL: s = y);  r = P s  (precond 0: identity,
 *   1: g1_inv with g1_deg steps, 2: lorr_inv);  x_new = x + om_a r + om_1 (x - x_prev)  (x == NULL: x_new = a0 r;
 *   x_prev NULL: 0).
 * y, x, x_prev, x_new are FP64; s and the stencil iterates are dtype (F32, F64 or F32X2, float-float on the FP32
 * pipe). One thread-block cluster per image keeps the image on chip for every stencil step: in registers (FP32
 * stencil and parts, 64 <= N <= 512) or in shared memory (the other types and sizes, or band | ADRT_OS_SHARED).
 * g1_coef is a HOST array: a, then (omega_k a, omega_k - 1) for
 * k = 1..g1_deg-1 (cheb_solve, fasthybrid.py:114-126). om_img (nullable, DEVICE, with x given): per-image pairs
 * (om_a, om_1) that replace om_a and om_1, so that images at different outer iterations step together (slot-level
 * serving). band: rows of an image per CTA, 16 or 32 (0: chosen from the batch). Supported:
 * n <= adrt_outer_step_max_n(dtype). */
#define ADRT_OS_SHARED 0x100 /* band flag: the shared-memory form of the fused outer step */
int adrt_outer_step(int dtype, int parts_dtype, int n, int nimg, const double* y, const void* p0, const void* p1,
                    const void* p2, const double* x, const double* x_prev, double* x_new, double om_a, double om_1,
                    double a0, int precond, int g1_deg, const double* g1_coef, const double* om_img, int band,
                    void* stream);
int adrt_outer_step_max_n(int dtype);

/* The fused outer step with a float-float outer state (FP32 stencil and partial images, 64 <= N <= 512): y is FP32
 * (nimg x N x N); x, x_prev and x_new hold per image an FP32 hi plane then an FP32 lo plane (nimg x 2 x N x N,
 * value = hi + lo, about 48 significant bits). The residual is y - (p0 + p1 + p2) in FP32 (the value the FP64 form
 * computes when y is an FP32 sum), the update adds om_a r + om_1 (x - x_prev) with an exact two-sum, and no FP64
 * arithmetic runs. Other arguments as adrt_outer_step. */
int adrt_outer_step_ff(int n, int nimg, const float* y, const float* p0, const float* p1, const float* p2,
                       const float* x, const float* x_prev, float* x_new, double om_a, double om_1, double a0,
                       int precond, int g1_deg, const double* g1_coef, const double* om_img, int band, void* stream);
/* float-float planes (nimg x 2 x N x N) to FP64 (nimg x N x N). */
int adrt_ff_to_f64(int n, int nimg, const float* x, double* out, void* stream);

/* Dense low-frequency rows (fastops.py:28-40, 100-117): for r < nrows and every image b,
 *   Y[b, rows[r], :] <- W_r Y[b, rows[r], :]     (W: nrows x N x N complex, row-major, dtype; Y rows of N complex at
 *   image stride img_stride complex elements), computed out of place in Zd (nrows x nimg x N complex scratch) and
 * copied back. use_tc = 1 with FP32 and n >= 6: tensor cores (tcgen05.mma kind::tf32, 3xTF32 split, FP32 accumulate);
 * *err (device int) is set to 1 if a tensor-core completion wait ran out. use_tc = 2 (FP32, nimg <= 16): W is given
 * TRANSPOSED (W[r][i][o] = W_r[o][i]) and a CUDA-core kernel streams it once per group of 8 images (small batches,
 * where the product is bound by reading the operators). use_tc = 3 (FP32, 7 <= n <= 10): W is the pre-split table of
 * adrt_dense_split and the tensor cores run the complex-blocked product (operator tiles by bulk copy through a
 * four-stage ring), writing the rows in place (Zd unused, may be NULL). Otherwise (use_tc = 0) CUDA cores. tile (tensor cores): images per CTA, 16, 32 or 64 (0: chosen
 * from nimg). */
int adrt_dense_rows(int dtype, int n, int nimg, int nrows, const int32_t* rows, const void* W, void* Y,
                    long long img_stride, void* Zd, int32_t* err, int use_tc, int tile, void* stream);
/* The operators W (nrows x N x N complex FP32, row-major) split once for use_tc = 3: Ws holds nrows x N/128 x N/16
 * chunks of four TF32 tiles (Re hi, Re lo, Im hi, Im lo; 128 output rows x 16 input columns each, in the K-major
 * core-matrix layout of tcgen05.mma), 16 N^2 bytes per row. 7 <= n <= 10. */
int adrt_dense_split(int n, int nrows, const void* W, void* Ws, void* stream);

/* Spatial ADRT in the reference's sinogram layout (adrtcore.py:122-137), nimg images, exact for integer dtypes
 * (ADRT_I32, ADRT_I64; sums only), FP32 / FP64 otherwise. scratch: 2 * nimg * 4 * (2N-1) * N elements of dtype.
 * forward: x (nimg x N x N) -> b (nimg x 4 x (2N-1) x N); transpose: b -> x. */
int adrt_forward(int dtype, int n, int nimg, const void* x, void* b, void* scratch, void* stream);
int adrt_transpose(int dtype, int n, int nimg, const void* b, void* x, void* scratch, void* stream);

/* ------------------------------------------------------------------ iterative Moore-Penrose pseudoinverse
 * pinv.py:23-48 cgls and pinv.py:51-82 pcg_normal on the GPU for nimg right-hand sides at once, FP64 throughout.
 * The caller owns every buffer (device memory) and drives the iteration: start once, then launch blocks of
 * iterations (or replay them from a CUDA graph) and read the per-image `active` flags between blocks; an image whose
 * test has passed (or that reached maxit) stops changing, so every image ends with the iterate the reference's own
 * loop returns. hist[img * (maxit + 1) + k] is the reference's history entry k (CGLS: ||R^T r_k||, PCG: ||r_k||),
 * it[img] its last index. nblk: CTAs per image of the inner products (partial: nimg * nblk doubles), scal: nimg * 4
 * doubles, scratch: 2 * nimg * 4 * (2N-1) * N doubles (the spatial ADRT's level buffers). */
typedef struct adrt_cgls {
    int n, nimg, maxit, nblk;
    double tol;
    double* x;       /* nimg x N x N: x0 in, the solution out */
    double* p;       /* nimg x N x N search direction */
    double* s;       /* nimg x N x N: R^T r */
    double* r;       /* nimg x 4 x (2N-1) x N residual b - R x */
    double* q;       /* nimg x 4 x (2N-1) x N: R p */
    double* scratch;
    double* partial;
    double* scal;
    int32_t* it;
    int32_t* active;
    double* hist;
} adrt_cgls;

/* r = b - R x, s = R^T r, p = s, gamma = <s,s>, hist[0] = sqrt(gamma) (pinv.py:26-33). b: nimg sinograms. */
int adrt_cgls_start(const adrt_cgls* S, const double* b, void* stream);
/* `iters` CGLS iterations (pinv.py:34-47), stream-ordered, no host synchronisation. */
int adrt_cgls_iterate(const adrt_cgls* S, int iters, void* stream);

typedef struct adrt_pcg {
    int n, nimg, maxit, nblk;
    double tol;
    double* x;       /* nimg x N x N: x0 in, the solution out */
    double* r;       /* nimg x N x N residual rhs - R^T R x */
    double* z;       /* nimg x N x N preconditioned residual M r (may alias r: M = identity) */
    double* p;       /* nimg x N x N search direction */
    double* q;       /* nimg x N x N: R^T R p */
    double* t;       /* nimg x 4 x (2N-1) x N: R p */
    double* scratch;
    double* partial;
    double* scal;
    int32_t* it;
    int32_t* active;
    double* hist;
} adrt_pcg;

/* r = rhs - R^T R x, hist[0] = ||r|| (pinv.py:62-69); the caller then forms z = M r and calls adrt_pcg_rho. */
int adrt_pcg_start(const adrt_pcg* S, const double* rhs, void* stream);
/* rho = <r, z>, p = z (pinv.py:64-66). */
int adrt_pcg_rho(const adrt_pcg* S, void* stream);
/* q = R^T R p, alpha = rho / <p,q>, x += alpha p, r -= alpha q, hist and the test (pinv.py:70-75); the caller then
 * forms z = M r (for active images) and calls adrt_pcg_direction. */
int adrt_pcg_step(const adrt_pcg* S, void* stream);
/* rho' = <r, z>, p = z + (rho'/rho) p, rho = rho' (pinv.py:76-79). */
int adrt_pcg_direction(const adrt_pcg* S, void* stream);

#ifdef __cplusplus
}
#endif
#endif
