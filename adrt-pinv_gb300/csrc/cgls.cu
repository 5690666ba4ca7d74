// Iterative Moore-Penrose pseudoinverse of the spatial ADRT on the GPU (reference: pinv.py:23-82):
//   CGLS (Hestenes-Stiefel / Paige-Saunders) on min ||R x - b||, and PCG on R^T R x = R^T b.
// Many right-hand sides at once: every image has its own scalars (gamma, alpha, beta, iteration count, history) and
// stops on its own test; a converged image's state is frozen (its updates are skipped) while the others go on, so
// that a batch returns, image by image, the iterate the reference's loop returns. All arithmetic is FP64; vector
// updates are written as separately rounded products and sums (no fused multiply-add), as NumPy evaluates them.
//
// Per iteration (CGLS): q = R p (n level passes), <q,q>, alpha; x += alpha p, r -= alpha q; s = R^T r (n passes),
// <s,s>, the convergence test and beta; p = s + beta p. Inner products are per-image partial sums over fixed
// segments (one CTA each) summed in a fixed order by one thread per image, so results do not depend on timing.
// Nothing here waits on the host: the host launches blocks of iterations (or records them in a CUDA graph) and
// reads the per-image active flags between blocks.
#include "common.cuh"
#include "launch.h"

namespace adrt {

constexpr int LSQ_THREADS = 256;

enum { SC_GAMMA = 0, SC_G0 = 1, SC_ALPHA = 2, SC_BETA = 3, SC_SLOTS = 4 };

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// partial[img * nblk + blk] = sum over this CTA's segment of a[img] . b[img] (len even; segments even-sized)
__global__ void __launch_bounds__(LSQ_THREADS) dot_partial_kernel(const double* __restrict__ a,
                                                                 const double* __restrict__ b, long long len, int nblk,
                                                                 double* __restrict__ partial,
                                                                 const int* __restrict__ active) {
    const int img = blockIdx.y, blk = blockIdx.x;
    if (active && !active[img]) return;
    long long seg = (len + nblk - 1) / nblk;
    seg += seg & 1;
    const long long s0 = (long long)blk * seg;
    const long long s1 = s0 + seg < len ? s0 + seg : len;
    const double* pa = a + (size_t)img * len;
    const double* pb = b + (size_t)img * len;
    double acc = 0.0;
    for (long long i = s0 + 2 * threadIdx.x; i < s1; i += 2 * LSQ_THREADS) {
        const double2 u = *reinterpret_cast<const double2*>(pa + i);
        const double2 v = *reinterpret_cast<const double2*>(pb + i);
        acc = fma(u.x, v.x, acc);
        acc = fma(u.y, v.y, acc);
    }
    __shared__ double red[LSQ_THREADS / 32];
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
#pragma unroll
        for (int w = 0; w < LSQ_THREADS / 32; ++w) t += red[w];
        partial[(size_t)img * nblk + blk] = t;
    }
}

__device__ __forceinline__ double sum_partials(const double* partial, int img, int nblk) {
    double t = 0.0;
    for (int k = 0; k < nblk; ++k) t += partial[(size_t)img * nblk + k];
    return t;
}

// ------------------------------------------------------------------ elementwise kernels (one image per grid row y)
// out = a - b
__global__ void sub_kernel(const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out,
                           long long len) {
    const size_t base = (size_t)blockIdx.y * len;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x)
        out[base + i] = __dsub_rn(a[base + i], b[base + i]);
}

// x += alpha p (image length lx), r -= alpha q (length lr), for active images
__global__ void update2_kernel(double* __restrict__ x, const double* __restrict__ p, long long lx,
                               double* __restrict__ r, const double* __restrict__ q, long long lr,
                               const double* __restrict__ scal, const int* __restrict__ active) {
    const int img = blockIdx.y;
    if (!active[img]) return;
    const double alpha = scal[img * SC_SLOTS + SC_ALPHA];
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long i0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    double* xi = x + (size_t)img * lx;
    const double* pi = p + (size_t)img * lx;
    for (long long i = i0; i < lx; i += stride) xi[i] = __dadd_rn(xi[i], __dmul_rn(alpha, pi[i]));
    double* ri = r + (size_t)img * lr;
    const double* qi = q + (size_t)img * lr;
    for (long long i = i0; i < lr; i += stride) ri[i] = __dsub_rn(ri[i], __dmul_rn(alpha, qi[i]));
}

// p = s + beta p, for active images
__global__ void direction_kernel(double* __restrict__ p, const double* __restrict__ s, long long len,
                                 const double* __restrict__ scal, const int* __restrict__ active) {
    const int img = blockIdx.y;
    if (!active[img]) return;
    const double beta = scal[img * SC_SLOTS + SC_BETA];
    double* pi = p + (size_t)img * len;
    const double* si = s + (size_t)img * len;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x)
        pi[i] = __dadd_rn(si[i], __dmul_rn(beta, pi[i]));
}

// ------------------------------------------------------------------ per-image scalar steps (one thread per image)
// start: gamma = sum (CGLS: <s,s>; PCG: rho = <r,z>), g0 = sqrt of the first norm, hist[0], active unless the
// starting residual is already zero (then x0 is a least-squares solution) or maxit == 0
__global__ void start_scalars_kernel(int nimg, int nblk, const double* __restrict__ partial_g,
                                     const double* __restrict__ partial_norm, double* __restrict__ scal,
                                     int* __restrict__ it, int* __restrict__ active, double* __restrict__ hist,
                                     int maxit) {
    const int img = blockIdx.x * blockDim.x + threadIdx.x;
    if (img >= nimg) return;
    const double g = sum_partials(partial_g, img, nblk);
    const double nrm = sqrt(partial_norm ? sum_partials(partial_norm, img, nblk) : g);
    scal[img * SC_SLOTS + SC_GAMMA] = g;
    scal[img * SC_SLOTS + SC_G0] = nrm;
    hist[(size_t)img * (maxit + 1)] = nrm;
    it[img] = 0;
    active[img] = (maxit > 0 && nrm > 0.0) ? 1 : 0;
}

// gamma = the sum (PCG: rho = <r, z> of the start), every image
__global__ void set_gamma_kernel(int nimg, int nblk, const double* __restrict__ partial, double* __restrict__ scal) {
    const int img = blockIdx.x * blockDim.x + threadIdx.x;
    if (img < nimg) scal[img * SC_SLOTS + SC_GAMMA] = sum_partials(partial, img, nblk);
}

// alpha = gamma / (sum of the partials of the curvature product)
__global__ void alpha_kernel(int nimg, int nblk, const double* __restrict__ partial, double* __restrict__ scal,
                             const int* __restrict__ active) {
    const int img = blockIdx.x * blockDim.x + threadIdx.x;
    if (img >= nimg || !active[img]) return;
    scal[img * SC_SLOTS + SC_ALPHA] = scal[img * SC_SLOTS + SC_GAMMA] / sum_partials(partial, img, nblk);
}

// CGLS: gnew = <s,s>; hist[it+1] = sqrt(gnew); stop if sqrt(gnew) <= tol g0 or it == maxit, else beta = gnew/gamma,
// gamma = gnew (pinv.py:40-47)
__global__ void cgls_test_kernel(int nimg, int nblk, const double* __restrict__ partial, double* __restrict__ scal,
                                 int* __restrict__ it, int* __restrict__ active, double* __restrict__ hist, int maxit,
                                 double tol) {
    const int img = blockIdx.x * blockDim.x + threadIdx.x;
    if (img >= nimg || !active[img]) return;
    const double gnew = sum_partials(partial, img, nblk);
    const int k = it[img] + 1;
    it[img] = k;
    const double gn = sqrt(gnew);
    hist[(size_t)img * (maxit + 1) + k] = gn;
    if (gn <= tol * scal[img * SC_SLOTS + SC_G0] || k >= maxit) {
        active[img] = 0;
        return;
    }
    scal[img * SC_SLOTS + SC_BETA] = gnew / scal[img * SC_SLOTS + SC_GAMMA];
    scal[img * SC_SLOTS + SC_GAMMA] = gnew;
}

// PCG, after the update: rn = ||r||; hist[it+1] = rn; stop if rn <= tol r0 or it == maxit (pinv.py:69-75)
__global__ void pcg_test_kernel(int nimg, int nblk, const double* __restrict__ partial, double* __restrict__ scal,
                                int* __restrict__ it, int* __restrict__ active, double* __restrict__ hist, int maxit,
                                double tol) {
    const int img = blockIdx.x * blockDim.x + threadIdx.x;
    if (img >= nimg || !active[img]) return;
    const double rn = sqrt(sum_partials(partial, img, nblk));
    const int k = it[img] + 1;
    it[img] = k;
    hist[(size_t)img * (maxit + 1) + k] = rn;
    if (rn <= tol * scal[img * SC_SLOTS + SC_G0] || k >= maxit) active[img] = 0;
}

// PCG, after z = M r: rho_new = <r,z>; beta = rho_new / rho; rho = rho_new (pinv.py:76-79)
__global__ void pcg_beta_kernel(int nimg, int nblk, const double* __restrict__ partial, double* __restrict__ scal,
                                const int* __restrict__ active) {
    const int img = blockIdx.x * blockDim.x + threadIdx.x;
    if (img >= nimg || !active[img]) return;
    const double rho = sum_partials(partial, img, nblk);
    scal[img * SC_SLOTS + SC_BETA] = rho / scal[img * SC_SLOTS + SC_GAMMA];
    scal[img * SC_SLOTS + SC_GAMMA] = rho;
}

// ------------------------------------------------------------------ host side
static int elem_grid(long long len) {
    const int sms = device_sm_count();
    long long g = (len + 4 * LSQ_THREADS - 1) / (4 * LSQ_THREADS);
    if (g > 4LL * sms) g = 4LL * sms;
    return (int)(g > 0 ? g : 1);
}

static int check_common(const char* what, int n, int nimg, int nblk, int maxit) {
    if (n < 1 || n > 12 || nimg < 1 || nimg > 65535 || nblk < 1 || nblk > 4096 || maxit < 0) {
        set_error("%s: bad sizes (n=%d nimg=%d nblk=%d maxit=%d)", what, n, nimg, nblk, maxit);
        return ADRT_EINVAL;
    }
    return ADRT_OK;
}

static int dot(const double* a, const double* b, long long len, int nimg, int nblk, double* partial, const int* active,
               cudaStream_t st) {
    dot_partial_kernel<<<dim3(nblk, nimg), LSQ_THREADS, 0, st>>>(a, b, len, nblk, partial, active);
    return launch_status("dot_partial_kernel");
}

static int scalar_grid(int nimg) { return (nimg + 127) / 128; }

}  // namespace adrt

using namespace adrt;

extern "C" int adrt_cgls_start(const adrt_cgls* S, const double* b, void* stream) {
    if (!S || !b) { set_error("adrt_cgls_start: null argument"); return ADRT_EINVAL; }
    if (int rc = check_common("adrt_cgls_start", S->n, S->nimg, S->nblk, S->maxit)) return rc;
    if (!S->x || !S->p || !S->s || !S->r || !S->q || !S->scratch || !S->partial || !S->scal || !S->it || !S->active ||
        !S->hist) {
        set_error("adrt_cgls_start: null buffer in the state");
        return ADRT_EINVAL;
    }
    cudaStream_t st = as_stream(stream);
    const long long N = 1LL << S->n, li = N * N, ls = 4 * (2 * N - 1) * N;
    const int nimg = S->nimg;
    // r = b - R x; s = R^T r; p = s; gamma = <s,s>
    if (int rc = adrt_fwd(ADRT_F64, S->n, nimg, S->x, S->q, S->scratch, st)) return rc;
    sub_kernel<<<dim3(elem_grid(ls), nimg), LSQ_THREADS, 0, st>>>(b, S->q, S->r, ls);
    if (int rc = launch_status("sub_kernel")) return rc;
    if (int rc = adrt_adj(ADRT_F64, S->n, nimg, S->r, S->s, S->scratch, st)) return rc;
    if (int rc = cuda_status(cudaMemcpyAsync(S->p, S->s, (size_t)nimg * li * 8, cudaMemcpyDeviceToDevice, st),
                             "cudaMemcpyAsync(p)"))
        return rc;
    if (int rc = dot(S->s, S->s, li, nimg, S->nblk, S->partial, nullptr, st)) return rc;
    start_scalars_kernel<<<scalar_grid(nimg), 128, 0, st>>>(nimg, S->nblk, S->partial, nullptr, S->scal, S->it,
                                                             S->active, S->hist, S->maxit);
    return launch_status("start_scalars_kernel");
}

extern "C" int adrt_cgls_iterate(const adrt_cgls* S, int iters, void* stream) {
    if (!S) { set_error("adrt_cgls_iterate: null state"); return ADRT_EINVAL; }
    if (int rc = check_common("adrt_cgls_iterate", S->n, S->nimg, S->nblk, S->maxit)) return rc;
    if (iters < 0) { set_error("adrt_cgls_iterate: iters=%d", iters); return ADRT_EINVAL; }
    cudaStream_t st = as_stream(stream);
    const long long N = 1LL << S->n, li = N * N, ls = 4 * (2 * N - 1) * N;
    const int nimg = S->nimg, nblk = S->nblk;
    const dim3 eg(elem_grid(ls), nimg), sg(scalar_grid(nimg));
    for (int k = 0; k < iters; ++k) {
        if (int rc = adrt_fwd(ADRT_F64, S->n, nimg, S->p, S->q, S->scratch, st, S->active)) return rc;  // q = R p
        if (int rc = dot(S->q, S->q, ls, nimg, nblk, S->partial, S->active, st)) return rc;
        alpha_kernel<<<sg, 128, 0, st>>>(nimg, nblk, S->partial, S->scal, S->active);
        if (int rc = launch_status("alpha_kernel")) return rc;
        update2_kernel<<<eg, LSQ_THREADS, 0, st>>>(S->x, S->p, li, S->r, S->q, ls, S->scal, S->active);
        if (int rc = launch_status("update2_kernel")) return rc;
        if (int rc = adrt_adj(ADRT_F64, S->n, nimg, S->r, S->s, S->scratch, st, S->active)) return rc;  // s = R^T r
        if (int rc = dot(S->s, S->s, li, nimg, nblk, S->partial, S->active, st)) return rc;
        cgls_test_kernel<<<sg, 128, 0, st>>>(nimg, nblk, S->partial, S->scal, S->it, S->active, S->hist, S->maxit,
                                             S->tol);
        if (int rc = launch_status("cgls_test_kernel")) return rc;
        direction_kernel<<<dim3(elem_grid(li), nimg), LSQ_THREADS, 0, st>>>(S->p, S->s, li, S->scal, S->active);
        if (int rc = launch_status("direction_kernel")) return rc;
    }
    return ADRT_OK;
}

// G v = R^T R v into out (sinogram-sized temporary t); active (nullable) skips frozen images
static int normal_op(const adrt_pcg* S, const double* v, double* out, const int* active, cudaStream_t st) {
    if (int rc = adrt_fwd(ADRT_F64, S->n, S->nimg, v, S->t, S->scratch, st, active)) return rc;
    return adrt_adj(ADRT_F64, S->n, S->nimg, S->t, out, S->scratch, st, active);
}

static int check_pcg(const char* what, const adrt_pcg* S) {
    if (!S) { set_error("%s: null state", what); return ADRT_EINVAL; }
    if (int rc = check_common(what, S->n, S->nimg, S->nblk, S->maxit)) return rc;
    if (!S->x || !S->r || !S->z || !S->p || !S->q || !S->t || !S->scratch || !S->partial || !S->scal || !S->it ||
        !S->active || !S->hist) {
        set_error("%s: null buffer in the state", what);
        return ADRT_EINVAL;
    }
    return ADRT_OK;
}

extern "C" int adrt_pcg_start(const adrt_pcg* S, const double* rhs, void* stream) {
    if (int rc = check_pcg("adrt_pcg_start", S)) return rc;
    if (!rhs) { set_error("adrt_pcg_start: null rhs"); return ADRT_EINVAL; }
    cudaStream_t st = as_stream(stream);
    const long long N = 1LL << S->n, li = N * N;
    const int nimg = S->nimg;
    // r = rhs - G x; r0 = ||r||, hist[0] (rho follows once z = M r exists: adrt_pcg_rho)
    if (int rc = normal_op(S, S->x, S->q, nullptr, st)) return rc;
    sub_kernel<<<dim3(elem_grid(li), nimg), LSQ_THREADS, 0, st>>>(rhs, S->q, S->r, li);
    if (int rc = launch_status("sub_kernel")) return rc;
    if (int rc = dot(S->r, S->r, li, nimg, S->nblk, S->partial, nullptr, st)) return rc;
    start_scalars_kernel<<<scalar_grid(nimg), 128, 0, st>>>(nimg, S->nblk, S->partial, nullptr, S->scal, S->it,
                                                             S->active, S->hist, S->maxit);
    return launch_status("start_scalars_kernel");
}

extern "C" int adrt_pcg_rho(const adrt_pcg* S, void* stream) {
    if (int rc = check_pcg("adrt_pcg_rho", S)) return rc;
    cudaStream_t st = as_stream(stream);
    const long long N = 1LL << S->n, li = N * N;
    // rho = <r, z>; p = z
    if (int rc = dot(S->r, S->z, li, S->nimg, S->nblk, S->partial, nullptr, st)) return rc;
    set_gamma_kernel<<<scalar_grid(S->nimg), 128, 0, st>>>(S->nimg, S->nblk, S->partial, S->scal);
    if (int rc = launch_status("set_gamma_kernel")) return rc;
    return cuda_status(cudaMemcpyAsync(S->p, S->z, (size_t)S->nimg * li * 8, cudaMemcpyDeviceToDevice, st),
                       "cudaMemcpyAsync(p)");
}

extern "C" int adrt_pcg_step(const adrt_pcg* S, void* stream) {
    if (int rc = check_pcg("adrt_pcg_step", S)) return rc;
    cudaStream_t st = as_stream(stream);
    const long long N = 1LL << S->n, li = N * N;
    const int nimg = S->nimg, nblk = S->nblk;
    const dim3 eg(elem_grid(li), nimg), sg(scalar_grid(nimg));
    // q = G p; alpha = rho / <p,q>; x += alpha p; r -= alpha q; rn = ||r||, the test
    if (int rc = normal_op(S, S->p, S->q, S->active, st)) return rc;
    if (int rc = dot(S->p, S->q, li, nimg, nblk, S->partial, S->active, st)) return rc;
    alpha_kernel<<<sg, 128, 0, st>>>(nimg, nblk, S->partial, S->scal, S->active);
    if (int rc = launch_status("alpha_kernel")) return rc;
    update2_kernel<<<eg, LSQ_THREADS, 0, st>>>(S->x, S->p, li, S->r, S->q, li, S->scal, S->active);
    if (int rc = launch_status("update2_kernel")) return rc;
    if (int rc = dot(S->r, S->r, li, nimg, nblk, S->partial, S->active, st)) return rc;
    pcg_test_kernel<<<sg, 128, 0, st>>>(nimg, nblk, S->partial, S->scal, S->it, S->active, S->hist, S->maxit, S->tol);
    return launch_status("pcg_test_kernel");
}

extern "C" int adrt_pcg_direction(const adrt_pcg* S, void* stream) {
    if (int rc = check_pcg("adrt_pcg_direction", S)) return rc;
    cudaStream_t st = as_stream(stream);
    const long long N = 1LL << S->n, li = N * N;
    const int nimg = S->nimg, nblk = S->nblk;
    // rho_new = <r, z>; beta = rho_new / rho; p = z + beta p
    if (int rc = dot(S->r, S->z, li, nimg, nblk, S->partial, S->active, st)) return rc;
    pcg_beta_kernel<<<scalar_grid(nimg), 128, 0, st>>>(nimg, nblk, S->partial, S->scal, S->active);
    if (int rc = launch_status("pcg_beta_kernel")) return rc;
    direction_kernel<<<dim3(elem_grid(li), nimg), LSQ_THREADS, 0, st>>>(S->p, S->z, li, S->scal, S->active);
    return launch_status("direction_kernel");
}
