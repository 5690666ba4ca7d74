// Image-space kernels of the outer iterations (reference: fasthybrid.py:81-130 stencils and cheb_solve,
// fastops._outer fastops.py:247-258). All are memory-bound elementwise or 5-point-cell stencil passes over
// nimg N x N images, one thread per pixel (grid-stride).
#include "common.cuh"
#include "launch.h"

namespace adrt {

template <typename T> __device__ __forceinline__ double ldd(const T* p, size_t i) { return (double)p[i]; }

static int grid_for(size_t total) {
    size_t g = (total + 255) / 256;
    if (g > 65535u * 8) g = 65535u * 8;
    return (int)(g ? g : 1);
}

// s = y - (p0 + p1 + p2)
template <typename T, typename TY>
__global__ void resid_kernel(size_t total, const TY* __restrict__ y, const T* __restrict__ p0, const T* __restrict__ p1,
                             const T* __restrict__ p2, T* __restrict__ s) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const T t = p0 ? (p0[i] + p1[i]) + p2[i] : (T)0;
        s[i] = (T)((TY)y[i] - (TY)t);
    }
}

template <typename T, typename TO>
__global__ void sum3_kernel(size_t total, const T* __restrict__ p0, const T* __restrict__ p1, const T* __restrict__ p2,
                            TO* __restrict__ out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x)
        out[i] = (TO)((p0[i] + p1[i]) + p2[i]);
}

// G_1 x at (i, j) = 8x + [2 x(i, j^1) + x(i-1, j^1) + x(i+1, j^1)] + [2 x(i^1, j) + x(i^1, j-1) + x(i^1, j+1)]
// (fasthybrid.py:95-98: J_cols(K_rows(x)) and its transposed counterpart; out-of-range neighbours are absent).
template <typename T>
__device__ __forceinline__ T g1_at(const T* __restrict__ x, int N, int i, int j) {
    const int jp = j ^ 1, ip = i ^ 1;
    T a = (T)2 * x[(size_t)i * N + jp];
    if (i > 0) a += x[(size_t)(i - 1) * N + jp];
    if (i < N - 1) a += x[(size_t)(i + 1) * N + jp];
    T b = (T)2 * x[(size_t)ip * N + j];
    if (j > 0) b += x[(size_t)ip * N + j - 1];
    if (j < N - 1) b += x[(size_t)ip * N + j + 1];
    return ((T)8 * x[(size_t)i * N + j] + a) + b;
}

// one step of cheb_solve(G1_apply, s, 4, 16, deg) (fasthybrid.py:114-126); x == NULL: xn = a0 s
template <typename T>
__global__ void g1_step_kernel(int n, size_t total, const T* __restrict__ s, const T* __restrict__ x, const T* __restrict__ xp,
                               T* __restrict__ xn, T om_a, T om_1, T a0) {
    const int N = 1 << n;
    const size_t NN = (size_t)N * N;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        if (!x) {
            xn[e] = a0 * s[e];
            continue;
        }
        const size_t img = e / NN, rem = e - img * NN;
        const int i = (int)(rem >> n), j = (int)(rem & (N - 1));
        const T* xi = x + img * NN;
        const T xv = x[e];
        const T r = s[e] - g1_at(xi, N, i, j);
        const T prev = xp ? xp[e] : (T)0;
        xn[e] = xv + om_a * r + om_1 * (xv - prev);
    }
}

// (4I + 8 Pi)^{-1} s = (s - Pi s)/4 + Pi s / 12, Pi = 2x2-cell mean (fasthybrid.py:101-111)
template <typename T>
__global__ void lorr_kernel(int n, size_t total, const T* __restrict__ s, T* __restrict__ out) {
    const int N = 1 << n;
    const size_t NN = (size_t)N * N;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const size_t img = e / NN, rem = e - img * NN;
        const int i = (int)(rem >> n), j = (int)(rem & (N - 1));
        const T* si = s + img * NN;
        const int i0 = i & ~1, j0 = j & ~1;
        const T m = ((si[(size_t)i0 * N + j0] + si[(size_t)i0 * N + j0 + 1]) + (si[(size_t)(i0 + 1) * N + j0] +
                                                                                  si[(size_t)(i0 + 1) * N + j0 + 1])) / (T)4;
        out[e] = (s[e] - m) / (T)4 + m / (T)12;
    }
}

// x_new = x + om_a r + om_1 (x - x_prev); x == NULL: x_new = a0 r (fastops.py:251-257). r may be narrower than x.
// om_img (nullable): per-image (om_a, om_1) pairs, images of `per` elements
template <typename T, typename TR>
__global__ void outer_kernel(size_t total, const T* __restrict__ x, const T* __restrict__ xp, const TR* __restrict__ r,
                             T* __restrict__ xn, T om_a, T om_1, T a0, const double* __restrict__ om_img, size_t per) {
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const T rv = (T)r[e];
        if (!x) {
            xn[e] = a0 * rv;
        } else {
            const T xv = x[e];
            const T prev = xp ? xp[e] : (T)0;
            T oa = om_a, o1 = om_1;
            if (om_img) {
                const size_t img = e / per;
                oa = (T)om_img[2 * img];
                o1 = (T)om_img[2 * img + 1];
            }
            xn[e] = xv + oa * rv + o1 * (xv - prev);
        }
    }
}

static bool img_args_ok(int dtype, int n, int nimg, const char* who) {
    if ((dtype != ADRT_F32 && dtype != ADRT_F64) || n < 1 || n > 12 || nimg < 0) {
        set_error("%s: bad arguments (dtype=%d n=%d nimg=%d)", who, dtype, n, nimg);
        return false;
    }
    return true;
}

int image_resid(int dtype, int n, int nimg, int ydtype, const void* y, const void* p0, const void* p1, const void* p2, void* s,
                cudaStream_t st) {
    if (!img_args_ok(dtype, n, nimg, "resid") || (ydtype != ADRT_F32 && ydtype != ADRT_F64)) return ADRT_EINVAL;
    const size_t total = (size_t)nimg << (2 * n);
    if (!total) return ADRT_OK;
    if (!y || !s || (p0 && (!p1 || !p2))) { set_error("resid: null pointer"); return ADRT_EINVAL; }
    const int g = grid_for(total);
    if (dtype == ADRT_F32 && ydtype == ADRT_F32)
        resid_kernel<float, float><<<g, 256, 0, st>>>(total, (const float*)y, (const float*)p0, (const float*)p1, (const float*)p2, (float*)s);
    else if (dtype == ADRT_F32)
        resid_kernel<float, double><<<g, 256, 0, st>>>(total, (const double*)y, (const float*)p0, (const float*)p1, (const float*)p2, (float*)s);
    else if (ydtype == ADRT_F64)
        resid_kernel<double, double><<<g, 256, 0, st>>>(total, (const double*)y, (const double*)p0, (const double*)p1, (const double*)p2, (double*)s);
    else
        resid_kernel<double, float><<<g, 256, 0, st>>>(total, (const float*)y, (const double*)p0, (const double*)p1, (const double*)p2, (double*)s);
    return launch_status("resid_kernel");
}

int image_sum3(int dtype, int n, int nimg, const void* p0, const void* p1, const void* p2, void* out, int out_dtype, cudaStream_t st) {
    if (!img_args_ok(dtype, n, nimg, "sum3") || (out_dtype != ADRT_F32 && out_dtype != ADRT_F64)) return ADRT_EINVAL;
    const size_t total = (size_t)nimg << (2 * n);
    if (!total) return ADRT_OK;
    if (!p0 || !p1 || !p2 || !out) { set_error("sum3: null pointer"); return ADRT_EINVAL; }
    const int g = grid_for(total);
    if (dtype == ADRT_F32 && out_dtype == ADRT_F32)
        sum3_kernel<float, float><<<g, 256, 0, st>>>(total, (const float*)p0, (const float*)p1, (const float*)p2, (float*)out);
    else if (dtype == ADRT_F32)
        sum3_kernel<float, double><<<g, 256, 0, st>>>(total, (const float*)p0, (const float*)p1, (const float*)p2, (double*)out);
    else if (out_dtype == ADRT_F64)
        sum3_kernel<double, double><<<g, 256, 0, st>>>(total, (const double*)p0, (const double*)p1, (const double*)p2, (double*)out);
    else
        sum3_kernel<double, float><<<g, 256, 0, st>>>(total, (const double*)p0, (const double*)p1, (const double*)p2, (float*)out);
    return launch_status("sum3_kernel");
}

// float-float planes (nimg, 2, N, N), hi then lo per image, to FP64 (nimg, N, N): the result of an inverse whose
// outer state is kept as float-float
__global__ void ff_to_f64_kernel(int n, size_t total, const float* __restrict__ x, double* __restrict__ out) {
    const size_t NN = (size_t)1 << (2 * n);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const size_t img = i >> (2 * n), e = i & (NN - 1);
        const float* p = x + img * 2 * NN + e;
        out[i] = (double)p[0] + (double)p[NN];
    }
}

int ff_to_f64(int n, int nimg, const float* x, double* out, cudaStream_t st) {
    if (n < 1 || n > 11 || nimg < 0) { set_error("ff_to_f64: bad arguments (n=%d nimg=%d)", n, nimg); return ADRT_EINVAL; }
    const size_t total = (size_t)nimg << (2 * n);
    if (!total) return ADRT_OK;
    if (!x || !out) { set_error("ff_to_f64: null pointer"); return ADRT_EINVAL; }
    ff_to_f64_kernel<<<grid_for(total), 256, 0, st>>>(n, total, x, out);
    return launch_status("ff_to_f64_kernel");
}

int image_g1_step(int dtype, int n, int nimg, const void* s, const void* x, const void* xp, void* xn, double om_a, double om_1,
                  double a0, cudaStream_t st) {
    if (!img_args_ok(dtype, n, nimg, "g1_step")) return ADRT_EINVAL;
    const size_t total = (size_t)nimg << (2 * n);
    if (!total) return ADRT_OK;
    if (!s || !xn) { set_error("g1_step: null pointer"); return ADRT_EINVAL; }
    const int g = grid_for(total);
    if (dtype == ADRT_F32)
        g1_step_kernel<float><<<g, 256, 0, st>>>(n, total, (const float*)s, (const float*)x, (const float*)xp, (float*)xn,
                                                 (float)om_a, (float)om_1, (float)a0);
    else
        g1_step_kernel<double><<<g, 256, 0, st>>>(n, total, (const double*)s, (const double*)x, (const double*)xp, (double*)xn,
                                                  om_a, om_1, a0);
    return launch_status("g1_step_kernel");
}

int image_lorr(int dtype, int n, int nimg, const void* s, void* out, cudaStream_t st) {
    if (!img_args_ok(dtype, n, nimg, "lorr")) return ADRT_EINVAL;
    const size_t total = (size_t)nimg << (2 * n);
    if (!total) return ADRT_OK;
    if (!s || !out) { set_error("lorr: null pointer"); return ADRT_EINVAL; }
    const int g = grid_for(total);
    if (dtype == ADRT_F32)
        lorr_kernel<float><<<g, 256, 0, st>>>(n, total, (const float*)s, (float*)out);
    else
        lorr_kernel<double><<<g, 256, 0, st>>>(n, total, (const double*)s, (double*)out);
    return launch_status("lorr_kernel");
}

int image_outer(int dtype, int n, int nimg, const void* x, const void* xp, const void* r, int rdtype, void* xn,
                double om_a, double om_1, double a0, const double* om_img, cudaStream_t st) {
    if (!img_args_ok(dtype, n, nimg, "outer_update") || (rdtype != ADRT_F32 && rdtype != ADRT_F64) ||
        (dtype == ADRT_F32 && rdtype == ADRT_F64)) {
        set_error("outer_update: bad dtypes (%d, r %d)", dtype, rdtype);
        return ADRT_EINVAL;
    }
    const size_t total = (size_t)nimg << (2 * n);
    if (!total) return ADRT_OK;
    if (!r || !xn || (om_img && !x)) { set_error("outer_update: null pointer"); return ADRT_EINVAL; }
    const int g = grid_for(total);
    const size_t per = (size_t)1 << (2 * n);
    if (dtype == ADRT_F32)
        outer_kernel<float, float><<<g, 256, 0, st>>>(total, (const float*)x, (const float*)xp, (const float*)r, (float*)xn,
                                                      (float)om_a, (float)om_1, (float)a0, om_img, per);
    else if (rdtype == ADRT_F64)
        outer_kernel<double, double><<<g, 256, 0, st>>>(total, (const double*)x, (const double*)xp, (const double*)r,
                                                        (double*)xn, om_a, om_1, a0, om_img, per);
    else
        outer_kernel<double, float><<<g, 256, 0, st>>>(total, (const double*)x, (const double*)xp, (const float*)r,
                                                       (double*)xn, om_a, om_1, a0, om_img, per);
    return launch_status("outer_kernel");
}

}  // namespace adrt
