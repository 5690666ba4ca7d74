// One image-space outer step of the inverse, fused: residual, preconditioner and outer Chebyshev update
// (reference: fastops._outer fastops.py:247-258 with P = g1_inv / lorr_inv / identity, fasthybrid.py:101-130):
//     s = y - (p0 + p1 + p2)                           (p* = the three partial images of G x; absent: s = y)
//     r = P s                                          (g1: deg-step Chebyshev on the G_1 stencil over [4, 16])
//     x_new = x + om_a r + om_1 (x - x_prev)           (x absent: x_new = a0 r)
// One thread-block cluster per image: CTA c of the cluster keeps rows [BAND c, BAND (c+1)) of s and of the two
// stencil iterates in shared memory for all steps; the G_1 stencil needs one row above and below the band, read
// from the neighbouring CTAs' shared memory (distributed shared memory) after a cluster barrier per step.
// Pair rows (2i, 2i+1) never straddle a band (BAND is even), so the i^1 neighbour is always local.
#include <cooperative_groups.h>
#include <type_traits>

#include "common.cuh"
#include "ff.cuh"
#include "launch.h"

namespace cg = cooperative_groups;

namespace adrt {

// ------------------------------------------------------------------ stencil arithmetic: FP32, FP64 or float-float (ff.cuh)
// arithmetic of one stencil element type: add, sub, mul, exact scaling by powers of two, conversions from/to FP64
template <typename T> struct StencilArith {
    using V = T;
    static __device__ __forceinline__ V add(V a, V b) { return a + b; }
    static __device__ __forceinline__ V sub(V a, V b) { return a - b; }
    static __device__ __forceinline__ V mul(V a, V b) { return a * b; }
    static __device__ __forceinline__ V scale(V a, float p2) { return (T)p2 * a; }
    static __device__ __forceinline__ V div12(V a) { return a / (T)12; }
    static __device__ __forceinline__ V zero() { return (T)0; }
    static __device__ __forceinline__ V from_d(double d) { return (T)d; }
    static __device__ __forceinline__ double to_d(V v) { return (double)v; }
};
template <> struct StencilArith<ff> {
    using V = ff;
    static __device__ __forceinline__ V add(V a, V b) { return ff_add(a, b); }
    static __device__ __forceinline__ V sub(V a, V b) { return ff_add(a, ff_neg(b)); }
    static __device__ __forceinline__ V mul(V a, V b) { return ff_mul(a, b); }
    static __device__ __forceinline__ V scale(V a, float p2) { return {p2 * a.hi, p2 * a.lo}; }  // exact
    static __device__ __forceinline__ V div12(V a) { return ff_mul(a, from_d(1.0 / 12.0)); }
    static __device__ __forceinline__ V zero() { return {0.f, 0.f}; }
    static __device__ __forceinline__ V from_d(double d) {
        const float h = __double2float_rn(d);
        return {h, __double2float_rn(d - (double)h)};
    }
    static __device__ __forceinline__ double to_d(V v) { return (double)v.hi + (double)v.lo; }
};

constexpr int OS_THREADS = 512;
constexpr int OS_MAX_STEPS = 32;

struct OuterStepArgs {
    const double* y;
    const void* p0;
    const void* p1;
    const void* p2;
    const double* x;
    const double* xp;
    double* xn;
    // the float-float form (register-resident kernel only): y in FP32 (nimg, N, N); x, xp, xn as (nimg, 2, N, N)
    // FP32 planes, hi then lo per image (value = hi + lo)
    const float* yf;
    const float* xf;
    const float* xpf;
    float* xnf;
    double om_a, om_1, a0;
    const double* om_img;  // nullable: per-image (om_a, om_1) pairs replacing om_a, om_1 (slot-level serving)
    int precond;  // 0 none, 1 g1, 2 lorr
    int g1_deg;
    double g1_a0;
    double g1_om_a[OS_MAX_STEPS];
    double g1_om_1[OS_MAX_STEPS];
    // the same coefficients rounded to FP32 once on the host (the register-resident kernel runs no FP64 per thread):
    // the stencil's, and hi + lo splits of the outer ones
    float g1f_a0;
    float g1f_a[OS_MAX_STEPS];
    float g1f_1[OS_MAX_STEPS];
    float oa_hi, oa_lo, o1_hi, o1_lo, a0_hi, a0_lo;
};

// fill the FP32 copies of the coefficients (host)
static void fill_f32_coefficients(OuterStepArgs& A) {
    auto split = [](double v, float& hi, float& lo) {
        hi = (float)v;
        lo = (float)(v - (double)hi);
    };
    A.g1f_a0 = (float)A.g1_a0;
    for (int k = 0; k + 1 < A.g1_deg && k < OS_MAX_STEPS; ++k) {
        A.g1f_a[k] = (float)A.g1_om_a[k];
        A.g1f_1[k] = (float)A.g1_om_1[k];
    }
    split(A.om_a, A.oa_hi, A.oa_lo);
    split(A.om_1, A.o1_hi, A.o1_lo);
    split(A.a0, A.a0_hi, A.a0_lo);
}

template <typename TS, typename TP, int n, int BAND>
__global__ void __launch_bounds__(OS_THREADS) outer_step_kernel(const OuterStepArgs A) {
    using Ar = StencilArith<TS>;
    using T = typename Ar::V;
    constexpr int N = 1 << n;
    constexpr int CL = N / BAND;
    constexpr int E = BAND * N;  // elements per CTA
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    const int img = blockIdx.x / CL;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* s = reinterpret_cast<T*>(smem_raw);
    T* bufA = s + E;
    T* bufB = bufA + E;
    const size_t base = (size_t)img * N * N + (size_t)rank * E;
    const TP* p0 = reinterpret_cast<const TP*>(A.p0);
    const TP* p1 = reinterpret_cast<const TP*>(A.p1);
    const TP* p2 = reinterpret_cast<const TP*>(A.p2);

    // residual into shared memory (the partial images summed in their own precision, the difference in FP64); two
    // neighbouring elements per thread and load (E and the image offsets are even)
    using TP2 = typename std::conditional<sizeof(TP) == 4, float2, double2>::type;
    for (int e = 2 * threadIdx.x; e < E; e += 2 * OS_THREADS) {
        const size_t g = base + e;
        TP t0 = (TP)0, t1 = (TP)0;
        if (p0) {
            const TP2 a = *reinterpret_cast<const TP2*>(p0 + g), b = *reinterpret_cast<const TP2*>(p1 + g),
                      c = *reinterpret_cast<const TP2*>(p2 + g);
            t0 = (a.x + b.x) + c.x;
            t1 = (a.y + b.y) + c.y;
        }
        const double2 yv = *reinterpret_cast<const double2*>(A.y + g);
        s[e] = Ar::from_d(yv.x - (double)t0);
        s[e + 1] = Ar::from_d(yv.y - (double)t1);
    }
    __syncthreads();

    T* r = s;
    if (A.precond == 1) {
        // x_1 = a s ; x_{k+1} = x_k + om_a (s - G1 x_k) + om_1 (x_k - x_{k-1})   (x_0 = 0)
        T* cur = bufA;
        T* prv = bufB;
        const T a0 = Ar::from_d(A.g1_a0);
        for (int e = threadIdx.x; e < E; e += OS_THREADS) {
            cur[e] = Ar::mul(a0, s[e]);
            prv[e] = Ar::zero();
        }
        cluster.sync();
        const T* up = rank > 0 ? cluster.map_shared_rank(bufA, rank - 1) : nullptr;     // neighbour buffers, same
        const T* dn = rank < CL - 1 ? cluster.map_shared_rank(bufA, rank + 1) : nullptr; // offsets in every CTA
        // thread -> (column j, group of row pairs); a row pair (2m, 2m+1) is updated together: the transposed
        // stencil term of each row reads the other row of the pair, the K term the rows above and below
        constexpr int CPP = N < OS_THREADS ? N : OS_THREADS;  // columns covered per pass of the CTA
        constexpr int RG = OS_THREADS / CPP;                  // row-pair groups
        const int j0 = threadIdx.x % CPP, grp = threadIdx.x / CPP;
        for (int k = 1; k < A.g1_deg; ++k) {
            const T om_a = Ar::from_d(A.g1_om_a[k - 1]), om_1 = Ar::from_d(A.g1_om_1[k - 1]);
            const ptrdiff_t off = cur - bufA;  // the current iterate lives at the same offset in every CTA
            const T* upc = up ? up + off : nullptr;
            const T* dnc = dn ? dn + off : nullptr;
            // the step reads cur (and s) and writes only prv: distinct buffers, so loads of later row pairs may be
            // issued ahead of earlier stores
            const T* __restrict__ cr = cur;
            T* __restrict__ pv = prv;
            const T* __restrict__ sr = s;
            for (int j = j0; j < N; j += CPP) {
                const int jp = j ^ 1;
                const bool hl = j > 0, hr = j < N - 1;
                constexpr int ITS = (BAND / 2 + RG - 1) / RG;  // row pairs per thread (compile-time trip count)
#pragma unroll
                for (int it = 0; it < ITS; ++it) {
                    const int m = grp + it * RG;
                    if (ITS * RG > BAND / 2 && m >= BAND / 2) break;
                    const int r0 = 2 * m, r1 = r0 + 1;
                    const T c0 = cr[r0 * N + j], c1 = cr[r1 * N + j];
                    const T q0 = cr[r0 * N + jp], q1 = cr[r1 * N + jp];
                    const T qm = r0 > 0 ? cr[(r0 - 1) * N + jp] : (upc ? upc[(BAND - 1) * N + jp] : Ar::zero());
                    const T qp = r1 < BAND - 1 ? cr[(r1 + 1) * N + jp] : (dnc ? dnc[jp] : Ar::zero());
                    T b0 = Ar::scale(c1, 2.f), b1 = Ar::scale(c0, 2.f);
                    if (hl) {
                        b0 = Ar::add(b0, cr[r1 * N + j - 1]);
                        b1 = Ar::add(b1, cr[r0 * N + j - 1]);
                    }
                    if (hr) {
                        b0 = Ar::add(b0, cr[r1 * N + j + 1]);
                        b1 = Ar::add(b1, cr[r0 * N + j + 1]);
                    }
                    const T a0 = Ar::add(Ar::add(Ar::scale(q0, 2.f), qm), q1);  // K along rows (i-1, then i+1)
                    const T a1 = Ar::add(Ar::add(Ar::scale(q1, 2.f), q0), qp);
                    const T g0 = Ar::add(Ar::add(Ar::scale(c0, 8.f), a0), b0);
                    const T g1 = Ar::add(Ar::add(Ar::scale(c1, 8.f), a1), b1);
                    const int e0 = r0 * N + j, e1 = r1 * N + j;
                    pv[e0] = Ar::add(Ar::add(c0, Ar::mul(om_a, Ar::sub(sr[e0], g0))), Ar::mul(om_1, Ar::sub(c0, pv[e0])));
                    pv[e1] = Ar::add(Ar::add(c1, Ar::mul(om_a, Ar::sub(sr[e1], g1))), Ar::mul(om_1, Ar::sub(c1, pv[e1])));
                }
            }
            cluster.sync();
            T* t = cur;
            cur = prv;
            prv = t;
        }
        r = cur;
    } else if (A.precond == 2) {
        // (s - Pi s)/4 + Pi s/12 with Pi the 2x2-cell mean (cells never straddle a band)
        T* out = bufA;
        for (int e = threadIdx.x; e < E; e += OS_THREADS) {
            const int i = e / N, j = e - (e / N) * N;
            const int i0 = i & ~1, j0 = j & ~1;
            const T m = Ar::scale(Ar::add(Ar::add(s[i0 * N + j0], s[i0 * N + j0 + 1]),
                                          Ar::add(s[(i0 + 1) * N + j0], s[(i0 + 1) * N + j0 + 1])), 0.25f);
            out[e] = Ar::add(Ar::scale(Ar::sub(s[e], m), 0.25f), Ar::div12(m));
        }
        __syncthreads();
        r = out;
    }

    // outer update in FP64
    const double oa = A.om_img ? A.om_img[2 * img] : A.om_a;
    const double o1 = A.om_img ? A.om_img[2 * img + 1] : A.om_1;
    for (int e = 2 * threadIdx.x; e < E; e += 2 * OS_THREADS) {
        const size_t g = base + e;
        const double r0 = Ar::to_d(r[e]), r1 = Ar::to_d(r[e + 1]);
        double2 out;
        if (!A.x) {
            out = make_double2(A.a0 * r0, A.a0 * r1);
        } else {
            const double2 xv = *reinterpret_cast<const double2*>(A.x + g);
            const double2 pv = A.xp ? *reinterpret_cast<const double2*>(A.xp + g) : make_double2(0.0, 0.0);
            out = make_double2(xv.x + oa * r0 + o1 * (xv.x - pv.x), xv.y + oa * r1 + o1 * (xv.y - pv.y));
        }
        *reinterpret_cast<double2*>(A.xn + g) = out;
    }
}

// CPT consecutive FP32 values of a row (CPT even; 16-byte accesses where CPT is a multiple of 4)
template <int CPT> __device__ __forceinline__ void ld_row(const float* p, float (&v)[CPT]) {
    if constexpr (CPT % 4 == 0) {
#pragma unroll
        for (int q = 0; q < CPT / 4; ++q) {
            const float4 t = *reinterpret_cast<const float4*>(p + 4 * q);
            v[4 * q] = t.x; v[4 * q + 1] = t.y; v[4 * q + 2] = t.z; v[4 * q + 3] = t.w;
        }
    } else {
#pragma unroll
        for (int q = 0; q < CPT / 2; ++q) {
            const float2 t = *reinterpret_cast<const float2*>(p + 2 * q);
            v[2 * q] = t.x; v[2 * q + 1] = t.y;
        }
    }
}
template <int CPT> __device__ __forceinline__ void st_row(float* p, const float (&v)[CPT]) {
    if constexpr (CPT % 4 == 0) {
#pragma unroll
        for (int q = 0; q < CPT / 4; ++q)
            *reinterpret_cast<float4*>(p + 4 * q) = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    } else {
#pragma unroll
        for (int q = 0; q < CPT / 2; ++q) *reinterpret_cast<float2*>(p + 2 * q) = make_float2(v[2 * q], v[2 * q + 1]);
    }
}

// ------------------------------------------------------------------ register-resident form (FP32 stencil and partial
// images, 64 <= N <= 512). Warp w of a CTA owns a strip of R = 1024 / N rows spanning the whole row: lane l holds
// columns l CPT .. l CPT + CPT - 1 (CPT = N / 32) of those rows, so its residual, both stencil iterates and its outer
// update stay in registers for the whole launch, and every 2x2 cell (row pair, column pair) of the G_1 stencil lies
// inside one thread. Per cell, with S the cell's sum, the stencil is
//     (G_1 c)(i, j) = 6 c(i, j) + 2 S + c(i', j') + c(i'', j^1)       i'' = the other row of the pair, j' = the column
//                                                                       beside the cell on i''; i' = the row beside
//                                                                       the cell on column j^1
// (the K term along rows and the transposed term along columns of fasthybrid.py:81-99, regrouped). The only values
// from outside a thread are the columns beside its first and last column (warp shuffles; zero at the image border)
// and, for the strip's first and last rows, the rows above and below the strip: other warps publish those into shared
// memory once per step (the strip above / below in the neighbouring CTA of the image's cluster through distributed
// shared memory). The cluster barrier is split: a step is computed without the strip-boundary terms while the
// barrier completes, then the boundary terms are read and applied (the step is linear in them). Two copies of the
// boundary buffer alternate, so each write is ordered after the previous step's reads of that copy.
template <int n, int BAND, bool FF>
__global__ void __launch_bounds__(32 * (BAND / (1024 >> n)), (1 << n) <= 256 ? 2 : 1)
    outer_step_reg_kernel(const OuterStepArgs A) {
    constexpr int N = 1 << n;
    constexpr int CPT = N / 32;    // columns per thread
    constexpr int R = 32 / CPT;    // rows per strip (warp)
    constexpr int W = BAND / R;    // strips per CTA
    constexpr int CL = N / BAND;   // CTAs per image (the cluster)
    constexpr int HC = W * 2 * N;  // floats per copy of the boundary buffer [strip][first / last row][column]
    static_assert(CPT >= 2 && CPT % 2 == 0 && R % 2 == 0 && BAND % R == 0, "cells inside a thread, row pairs per strip");
    extern __shared__ __align__(16) float bnd[];  // [2][W][2][N]
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    const int img = blockIdx.x / CL;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int j0 = lane * CPT;
    const size_t gbase = (size_t)img * N * N + (size_t)(rank * BAND + w * R) * N + j0;
    constexpr unsigned FULL = 0xffffffffu;

    // residual: the partial images summed in FP32, the difference in FP64 rounded to FP32 (FP64 y), or in FP32 (FP32
    // y: the same value, since the exact difference of two FP32 numbers is rounded once either way)
    float s[R][CPT];
    {
        const float* p0 = reinterpret_cast<const float*>(A.p0);
        const float* p1 = reinterpret_cast<const float*>(A.p1);
        const float* p2 = reinterpret_cast<const float*>(A.p2);
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const size_t gi = gbase + (size_t)r * N;
            double2 yv[CPT / 2];
            float yfv[CPT];
            if constexpr (FF) {
                ld_row<CPT>(A.yf + gi, yfv);
            } else {
#pragma unroll
                for (int q = 0; q < CPT / 2; ++q) yv[q] = *reinterpret_cast<const double2*>(A.y + gi + 2 * q);
            }
            float t[CPT];
#pragma unroll
            for (int q = 0; q < CPT; ++q) t[q] = 0.f;
            if (p0) {
#pragma unroll
                for (int q = 0; q < CPT / 2; ++q) {
                    const float2 a = *reinterpret_cast<const float2*>(p0 + gi + 2 * q);
                    const float2 b = *reinterpret_cast<const float2*>(p1 + gi + 2 * q);
                    const float2 c = *reinterpret_cast<const float2*>(p2 + gi + 2 * q);
                    t[2 * q] = (a.x + b.x) + c.x;
                    t[2 * q + 1] = (a.y + b.y) + c.y;
                }
            }
#pragma unroll
            for (int q = 0; q < CPT / 2; ++q) {
                if constexpr (FF) {
                    s[r][2 * q] = yfv[2 * q] - t[2 * q];
                    s[r][2 * q + 1] = yfv[2 * q + 1] - t[2 * q + 1];
                } else {
                    s[r][2 * q] = (float)(yv[q].x - (double)t[2 * q]);
                    s[r][2 * q + 1] = (float)(yv[q].y - (double)t[2 * q + 1]);
                }
            }
        }
    }

    float cA[R][CPT], cB[R][CPT];
    bool in_b = false;  // the result of the preconditioner is in cB (else in cA)
    if (A.precond == 1) {
        const float* up = rank > 0 ? cluster.map_shared_rank(bnd, rank - 1) : nullptr;
        const float* dn = rank < CL - 1 ? cluster.map_shared_rank(bnd, rank + 1) : nullptr;
        // the strip's first and last rows of iterate v into copy b, then arrive at the cluster barrier
        auto publish = [&](const float (&v)[R][CPT], int b) {
            float* f = bnd + b * HC + (w * 2) * N + j0;
#pragma unroll
            for (int q = 0; q < CPT / 2; ++q) {
                *reinterpret_cast<float2*>(f + 2 * q) = make_float2(v[0][2 * q], v[0][2 * q + 1]);
                *reinterpret_cast<float2*>(f + N + 2 * q) = make_float2(v[R - 1][2 * q], v[R - 1][2 * q + 1]);
            }
            asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
        };
        // one Chebyshev step p <- c + om_a (s - G1 c) + om_1 (c - p); the boundary of c is in copy b
        auto step = [&](const float (&c)[R][CPT], float (&p)[R][CPT], float om_a, float om_1, int b) {
#pragma unroll
            for (int m = 0; m < R / 2; ++m) {
                const int r0 = 2 * m, r1 = r0 + 1;
                // the columns beside the thread's first and last column, on both rows of the pair
                const float l0 = __shfl_up_sync(FULL, c[r0][CPT - 1], 1), l1 = __shfl_up_sync(FULL, c[r1][CPT - 1], 1);
                const float q0 = __shfl_down_sync(FULL, c[r0][0], 1), q1 = __shfl_down_sync(FULL, c[r1][0], 1);
                const float L0 = lane == 0 ? 0.f : l0, L1 = lane == 0 ? 0.f : l1;
                const float R0 = lane == 31 ? 0.f : q0, R1 = lane == 31 ? 0.f : q1;
#pragma unroll
                for (int v = 0; v < CPT / 2; ++v) {
                    const int a = 2 * v, bb = a + 1;
                    const float c00 = c[r0][a], c01 = c[r0][bb], c10 = c[r1][a], c11 = c[r1][bb];
                    const float t = 2.f * ((c00 + c01) + (c10 + c11));
                    float g00 = fmaf(6.f, c00, t), g01 = fmaf(6.f, c01, t);
                    float g10 = fmaf(6.f, c10, t), g11 = fmaf(6.f, c11, t);
                    if (r0 > 0) {  // the row above the pair, pair column (the strip's first row: deferred)
                        g00 += c[r0 - 1][bb];
                        g01 += c[r0 - 1][a];
                    }
                    if (r1 < R - 1) {  // the row below
                        g10 += c[r1 + 1][bb];
                        g11 += c[r1 + 1][a];
                    }
                    g00 += v > 0 ? c[r1][a - 1] : L1;  // beside the cell, on the other row of the pair
                    g10 += v > 0 ? c[r0][a - 1] : L0;
                    g01 += v < CPT / 2 - 1 ? c[r1][bb + 1] : R1;
                    g11 += v < CPT / 2 - 1 ? c[r0][bb + 1] : R0;
                    p[r0][a] = (c00 + om_a * (s[r0][a] - g00)) + om_1 * (c00 - p[r0][a]);
                    p[r0][bb] = (c01 + om_a * (s[r0][bb] - g01)) + om_1 * (c01 - p[r0][bb]);
                    p[r1][a] = (c10 + om_a * (s[r1][a] - g10)) + om_1 * (c10 - p[r1][a]);
                    p[r1][bb] = (c11 + om_a * (s[r1][bb] - g11)) + om_1 * (c11 - p[r1][bb]);
                }
            }
            asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
            // the rows above and below the strip (zero beyond the image): G_1 c gains c(above, j^1) on the first
            // row and c(below, j^1) on the last, so p loses om_a times those
            const float* fa = w > 0 ? bnd + b * HC + ((w - 1) * 2 + 1) * N
                                    : (up ? up + b * HC + ((W - 1) * 2 + 1) * N : nullptr);
            const float* fb = w < W - 1 ? bnd + b * HC + ((w + 1) * 2) * N : (dn ? dn + b * HC : nullptr);
#pragma unroll
            for (int q = 0; q < CPT / 2; ++q) {
                const float2 ta = fa ? *reinterpret_cast<const float2*>(fa + j0 + 2 * q) : make_float2(0.f, 0.f);
                const float2 tb = fb ? *reinterpret_cast<const float2*>(fb + j0 + 2 * q) : make_float2(0.f, 0.f);
                p[0][2 * q] = fmaf(-om_a, ta.y, p[0][2 * q]);
                p[0][2 * q + 1] = fmaf(-om_a, ta.x, p[0][2 * q + 1]);
                p[R - 1][2 * q] = fmaf(-om_a, tb.y, p[R - 1][2 * q]);
                p[R - 1][2 * q + 1] = fmaf(-om_a, tb.x, p[R - 1][2 * q + 1]);
            }
        };
        const float a0 = A.g1f_a0;
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int q = 0; q < CPT; ++q) {
                cA[r][q] = a0 * s[r][q];
                cB[r][q] = 0.f;
            }
        publish(cA, 0);
        int k = 1;
        for (; k + 1 < A.g1_deg; k += 2) {
            step(cA, cB, A.g1f_a[k - 1], A.g1f_1[k - 1], (k - 1) & 1);
            publish(cB, k & 1);
            step(cB, cA, A.g1f_a[k], A.g1f_1[k], k & 1);
            publish(cA, (k + 1) & 1);
        }
        if (k < A.g1_deg) {
            step(cA, cB, A.g1f_a[k - 1], A.g1f_1[k - 1], (k - 1) & 1);
            publish(cB, k & 1);
            in_b = true;
        }
        // the last arrival's wait: no CTA leaves while a neighbour may still read its boundary rows
        asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
    } else if (A.precond == 2) {
        // (s - Pi s)/4 + Pi s/12, Pi the mean of the 2x2 cell
#pragma unroll
        for (int r0 = 0; r0 < R; r0 += 2)
#pragma unroll
            for (int a = 0; a < CPT; a += 2) {
                const float mu = ((s[r0][a] + s[r0][a + 1]) + (s[r0 + 1][a] + s[r0 + 1][a + 1])) * 0.25f;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int r = r0 + (q >> 1), c = a + (q & 1);
                    cA[r][c] = (s[r][c] - mu) * 0.25f + mu / 12.f;
                }
            }
    } else {
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int q = 0; q < CPT; ++q) cA[r][q] = s[r][q];
    }

    // outer update: in FP64 (FP64 state), or in float-float on the FP32 pipe (float-float state): the step
    // om_a r + om_1 (x - x_prev) in FP32 with the coefficients carried as hi + lo, added to x with an exact
    // two-sum, so the state keeps about 48 bits while no FP64 instruction runs (the FP64 pipe of this GPU is a small
    // fraction of its FP32 pipe)
    if constexpr (FF) {
        float oah = A.oa_hi, oal = A.oa_lo, o1h = A.o1_hi, o1l = A.o1_lo;
        if (A.om_img) {  // per-image coefficients (slot-level serving): split here
            const double oa = A.om_img[2 * img], o1 = A.om_img[2 * img + 1];
            oah = (float)oa;
            oal = (float)(oa - (double)oah);
            o1h = (float)o1;
            o1l = (float)(o1 - (double)o1h);
        }
        const float a0h = A.a0_hi, a0l = A.a0_lo;
        const size_t fo = gbase + (size_t)img * N * N;  // hi plane of this thread's first row; lo plane N^2 further
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const size_t gi = fo + (size_t)r * N;
            float rv[CPT], hv[CPT], lv[CPT];
#pragma unroll
            for (int q = 0; q < CPT; ++q) rv[q] = in_b ? cB[r][q] : cA[r][q];
            if (!A.xf) {
#pragma unroll
                for (int q = 0; q < CPT; ++q) {
                    const float h = a0h * rv[q];
                    const float l = fmaf(a0h, rv[q], -h) + a0l * rv[q];
                    hv[q] = h + l;
                    lv[q] = l - (hv[q] - h);
                }
            } else {
                float xh[CPT], xl[CPT], ph[CPT], pl[CPT];
                ld_row<CPT>(A.xf + gi, xh);
                ld_row<CPT>(A.xf + gi + (size_t)N * N, xl);
                if (A.xpf) {
                    ld_row<CPT>(A.xpf + gi, ph);
                    ld_row<CPT>(A.xpf + gi + (size_t)N * N, pl);
                } else {
#pragma unroll
                    for (int q = 0; q < CPT; ++q) ph[q] = pl[q] = 0.f;
                }
#pragma unroll
                for (int q = 0; q < CPT; ++q) {
                    const float d = (xh[q] - ph[q]) + (xl[q] - pl[q]);
                    const float del = fmaf(oah, rv[q], fmaf(o1h, d, fmaf(oal, rv[q], o1l * d)));
                    const float sh = xh[q] + del, bb = sh - xh[q];
                    const float lo = ((xh[q] - (sh - bb)) + (del - bb)) + xl[q];
                    hv[q] = sh + lo;
                    lv[q] = lo - (hv[q] - sh);
                }
            }
            st_row<CPT>(A.xnf + gi, hv);
            st_row<CPT>(A.xnf + gi + (size_t)N * N, lv);
        }
        return;
    }
    const double oa = A.om_img ? A.om_img[2 * img] : A.om_a;
    const double o1 = A.om_img ? A.om_img[2 * img + 1] : A.om_1;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const size_t gi = gbase + (size_t)r * N;
#pragma unroll
        for (int q = 0; q < CPT / 2; ++q) {
            const double r0 = (double)(in_b ? cB[r][2 * q] : cA[r][2 * q]);
            const double r1 = (double)(in_b ? cB[r][2 * q + 1] : cA[r][2 * q + 1]);
            double2 out;
            if (!A.x) {
                out = make_double2(A.a0 * r0, A.a0 * r1);
            } else {
                const double2 xv = *reinterpret_cast<const double2*>(A.x + gi + 2 * q);
                const double2 pv = A.xp ? *reinterpret_cast<const double2*>(A.xp + gi + 2 * q) : make_double2(0.0, 0.0);
                out = make_double2(xv.x + oa * r0 + o1 * (xv.x - pv.x), xv.y + oa * r1 + o1 * (xv.y - pv.y));
            }
            *reinterpret_cast<double2*>(A.xn + gi + 2 * q) = out;
        }
    }
}

template <int n, int BAND, bool FF>
static int launch_os_reg(const OuterStepArgs& A, int nimg, cudaStream_t st) {
    constexpr int N = 1 << n;
    constexpr int CL = N / BAND;
    constexpr int W = BAND / (1024 / N);
    const size_t smem = 2 * (size_t)W * 2 * N * sizeof(float);
    auto kern = outer_step_reg_kernel<n, BAND, FF>;
    if (int rc = ensure_smem((const void*)kern, smem)) return rc;
    if (CL > 8) {
        if (int rc = cuda_status(cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1),
                                 "outer_step cluster attribute"))
            return rc;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nimg * CL);
    cfg.blockDim = dim3(32 * W);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CL;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return launch_ex_status(cudaLaunchKernelEx(&cfg, kern, A), "outer_step_reg_kernel");
}

template <typename TS, typename TP, int n, int BAND>
static int launch_os_band(const OuterStepArgs& A, int nimg, cudaStream_t st) {
    constexpr int N = 1 << n;
    constexpr int CL = N / BAND;
    const size_t smem = 3 * (size_t)BAND * N * sizeof(TS);
    auto kern = outer_step_kernel<TS, TP, n, BAND>;
    if (int rc = ensure_smem((const void*)kern, smem)) return rc;
    if (CL > 8) {
        if (int rc = cuda_status(cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1),
                                 "outer_step cluster attribute"))
            return rc;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nimg * CL);
    cfg.blockDim = dim3(OS_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CL;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return launch_ex_status(cudaLaunchKernelEx(&cfg, kern, A), "outer_step_kernel");
}

// 32-row bands; when the batch's clusters cannot fill the SMs (N <= 256), 16-row bands instead: twice the CTAs per
// image (clusters of up to 16), half the rows each, so a small batch finishes its stencil steps sooner
template <typename TS, typename TP, int n>
static int launch_os(const OuterStepArgs& A, int nimg, int band, cudaStream_t st) {
    constexpr int N = 1 << n;
    if constexpr (N >= 32 && N / 16 <= 16) {
        const bool b16 = band ? band == 16 : (long)nimg * (N / 32) < device_sm_count();
        if (b16) return launch_os_band<TS, TP, n, 16>(A, nimg, st);
    }
    return launch_os_band<TS, TP, n, (N >= 32 ? 32 : N)>(A, nimg, st);
}

// largest n with a fused (cluster) outer step for stencil element type dtype: the band tiles must fit 227 KB and
// the cluster at most 16 CTAs (non-portable size above 8); 8-byte types (FP64, float-float) stop at n = 8
int outer_step_max_n(int dtype) { return dtype == ADRT_F32 ? 9 : 8; }

template <typename TS, typename TP>
static int dispatch_os(int n, const OuterStepArgs& A, int nimg, int band, cudaStream_t st) {
    switch (n) {
        case 1: return launch_os<TS, TP, 1>(A, nimg, band, st);
        case 2: return launch_os<TS, TP, 2>(A, nimg, band, st);
        case 3: return launch_os<TS, TP, 3>(A, nimg, band, st);
        case 4: return launch_os<TS, TP, 4>(A, nimg, band, st);
        case 5: return launch_os<TS, TP, 5>(A, nimg, band, st);
        case 6: return launch_os<TS, TP, 6>(A, nimg, band, st);
        case 7: return launch_os<TS, TP, 7>(A, nimg, band, st);
        case 8: return launch_os<TS, TP, 8>(A, nimg, band, st);
        case 9:
            if constexpr (sizeof(TS) == 4) return launch_os<TS, TP, 9>(A, nimg, band, st);
            break;
    }
    set_error("outer_step: n=%d unsupported for this stencil type", n);
    return ADRT_EUNSUPPORTED;
}

// register-resident form, FP32 stencil and partial images, n = 6..9; bands as in launch_os
template <int n, bool FF>
static int launch_os_reg_auto(const OuterStepArgs& A, int nimg, int band, cudaStream_t st) {
    constexpr int N = 1 << n;
    const bool b16 = band ? band == 16 : (long)nimg * (N / 32) < device_sm_count();
    if constexpr (N / 16 <= 16) {
        if (b16) return launch_os_reg<n, 16, FF>(A, nimg, st);
    }
    return launch_os_reg<n, 32, FF>(A, nimg, st);
}

template <bool FF>
static int dispatch_os_reg(int n, const OuterStepArgs& A, int nimg, int band, cudaStream_t st) {
    switch (n) {
        case 6: return launch_os_reg_auto<6, FF>(A, nimg, band, st);
        case 7: return launch_os_reg_auto<7, FF>(A, nimg, band, st);
        case 8: return launch_os_reg_auto<8, FF>(A, nimg, band, st);
        case 9: return launch_os_reg_auto<9, FF>(A, nimg, band, st);
    }
    set_error("outer_step: no register-resident form for n=%d", n);
    return ADRT_EUNSUPPORTED;
}

int outer_step(int dtype, int parts_dtype, int n, int nimg, const double* y, const void* p0, const void* p1,
               const void* p2, const double* x, const double* xp, double* xn, double om_a, double om_1, double a0,
               int precond, int g1_deg, const double* g1_coef, const double* om_img, int band, cudaStream_t st) {
    const bool sd_ok = dtype == ADRT_F32 || dtype == ADRT_F64 || dtype == ADRT_F32X2;
    const bool pd_ok = parts_dtype == ADRT_F32 || parts_dtype == ADRT_F64;
    if (!sd_ok || !pd_ok || n < 1 || n > outer_step_max_n(dtype) || nimg < 0 || precond < 0 || precond > 2 ||
        (precond == 1 && (g1_deg < 1 || g1_deg > OS_MAX_STEPS || !g1_coef)) || (p0 && (!p1 || !p2))) {
        set_error("outer_step: bad arguments (dtype=%d parts=%d n=%d precond=%d deg=%d)", dtype, parts_dtype, n, precond,
                  g1_deg);
        return ADRT_EINVAL;
    }
    if (!nimg) return ADRT_OK;
    if (!y || !xn || (om_img && !x)) { set_error("outer_step: null pointer"); return ADRT_EINVAL; }
    const bool shared_form = (band & ADRT_OS_SHARED) != 0;
    band &= ~ADRT_OS_SHARED;
    if (band != 0 && band != 16 && band != 32) {
        set_error("outer_step: band must be 0 (auto), 16 or 32, optionally with ADRT_OS_SHARED");
        return ADRT_EINVAL;
    }
    OuterStepArgs A = {};
    A.y = y; A.p0 = p0; A.p1 = p1; A.p2 = p2; A.x = x; A.xp = xp; A.xn = xn;
    A.om_a = om_a; A.om_1 = om_1; A.a0 = a0; A.om_img = om_img; A.precond = precond; A.g1_deg = g1_deg;
    if (precond == 1) {
        A.g1_a0 = g1_coef[0];
        for (int k = 1; k < g1_deg; ++k) {
            A.g1_om_a[k - 1] = g1_coef[2 * k - 1];
            A.g1_om_1[k - 1] = g1_coef[2 * k];
        }
    }
    fill_f32_coefficients(A);
    // FP32 stencil on FP32 partial images: the register-resident form where it exists, unless the shared-memory
    // form is asked for
    if (!shared_form && dtype == ADRT_F32 && parts_dtype == ADRT_F32 && n >= 6 && n <= 9)
        return dispatch_os_reg<false>(n, A, nimg, band, st);
    // instantiated pairs: FP32 partial images with any stencil type, FP64 partial images with the FP64 stencil
    if (parts_dtype == ADRT_F32) {
        switch (dtype) {
            case ADRT_F32: return dispatch_os<float, float>(n, A, nimg, band, st);
            case ADRT_F64: return dispatch_os<double, float>(n, A, nimg, band, st);
            default: return dispatch_os<ff, float>(n, A, nimg, band, st);
        }
    }
    if (dtype == ADRT_F64) return dispatch_os<double, double>(n, A, nimg, band, st);
    set_error("outer_step: FP64 partial images take the FP64 stencil only");
    return ADRT_EUNSUPPORTED;
}

// the float-float state form: FP32 stencil and partial images, y FP32, x / x_prev / x_new as float-float planes
int outer_step_ff(int n, int nimg, const float* y, const float* p0, const float* p1, const float* p2, const float* x,
                  const float* xp, float* xn, double om_a, double om_1, double a0, int precond, int g1_deg,
                  const double* g1_coef, const double* om_img, int band, cudaStream_t st) {
    if (n < 6 || n > 9 || nimg < 0 || precond < 0 || precond > 2 ||
        (precond == 1 && (g1_deg < 1 || g1_deg > OS_MAX_STEPS || !g1_coef)) || (p0 && (!p1 || !p2)) ||
        (band != 0 && band != 16 && band != 32)) {
        set_error("outer_step_ff: bad arguments (n=%d precond=%d deg=%d band=%d; n must be 6..9)", n, precond, g1_deg,
                  band);
        return ADRT_EINVAL;
    }
    if (!nimg) return ADRT_OK;
    if (!y || !xn || (om_img && !x)) { set_error("outer_step_ff: null pointer"); return ADRT_EINVAL; }
    OuterStepArgs A = {};
    A.yf = y; A.p0 = p0; A.p1 = p1; A.p2 = p2; A.xf = x; A.xpf = xp; A.xnf = xn;
    A.om_a = om_a; A.om_1 = om_1; A.a0 = a0; A.om_img = om_img; A.precond = precond; A.g1_deg = g1_deg;
    if (precond == 1) {
        A.g1_a0 = g1_coef[0];
        for (int k = 1; k < g1_deg; ++k) {
            A.g1_om_a[k - 1] = g1_coef[2 * k - 1];
            A.g1_om_1[k - 1] = g1_coef[2 * k];
        }
    }
    fill_f32_coefficients(A);
    return dispatch_os_reg<true>(n, A, nimg, band, st);
}

}  // namespace adrt
