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
    double om_a, om_1, a0;
    const double* om_img;  // nullable: per-image (om_a, om_1) pairs replacing om_a, om_1 (slot-level serving)
    int precond;  // 0 none, 1 g1, 2 lorr
    int g1_deg;
    double g1_a0;
    double g1_om_a[OS_MAX_STEPS];
    double g1_om_1[OS_MAX_STEPS];
};

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

// ------------------------------------------------------------------ register-resident form (FP32 stencil and partial
// images, 64 <= N <= 512). Thread (g, u) of a CTA owns the column pair (2u, 2u + 1) on the OSR_R rows of row group g
// (rows row0 .. row0 + OSR_R - 1 of the image): its residual, both stencil iterates and its outer update stay in
// registers for the whole launch. A stencil step finds the pair column j ^ 1 and the rows above and below inside the
// thread, and the columns 2u - 1 and 2u + 2 in the neighbouring lanes (warp shuffles). Only what crosses a thread
// boundary goes through shared memory, once per step: the first and last row of every row group (halo rows, read by
// the group above / below, in this CTA or over distributed shared memory in the neighbouring CTA of the image's
// cluster) and the first and last column of every warp (read by the edge lanes of the neighbouring warps). The
// buffers alternate between two copies, so one cluster barrier per step orders every write before its reads and
// every read before the next overwrite. The arithmetic is the shared-memory kernel's, term for term.
constexpr int OSR_R = 16;

template <int n, int BAND>
__global__ void __launch_bounds__((1 << n) / 2 * (BAND / OSR_R), (1 << n) <= 256 ? 2 : 1)
    outer_step_reg_kernel(const OuterStepArgs A) {
    constexpr int N = 1 << n;
    constexpr int R = OSR_R;
    constexpr int G = BAND / R;   // row groups per CTA
    constexpr int TPR = N / 2;    // threads per row group
    constexpr int NW = TPR / 32;  // warps per row group
    constexpr int CL = N / BAND;  // CTAs per image (the cluster)
    static_assert(TPR % 32 == 0 && BAND % R == 0 && R % 2 == 0, "whole warps per row group, row pairs per group");
    __shared__ __align__(16) float halo[2][G][2][N];  // [copy][group][first / last row][column]
    __shared__ float edge[2][G][NW][2][R];            // [copy][group][warp][first / last column][row]
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    const int img = blockIdx.x / CL;
    const int g = threadIdx.x / TPR, u = threadIdx.x - g * TPR;
    const int lane = threadIdx.x & 31, wg = u >> 5;
    const size_t gbase = (size_t)img * N * N + (size_t)(rank * BAND + g * R) * N + 2 * u;
    constexpr unsigned FULL = 0xffffffffu;

    // residual: the partial images summed in FP32, the difference in FP64, rounded to FP32
    float2 sv[R];
    {
        const float* p0 = reinterpret_cast<const float*>(A.p0);
        const float* p1 = reinterpret_cast<const float*>(A.p1);
        const float* p2 = reinterpret_cast<const float*>(A.p2);
#pragma unroll
        for (int r0 = 0; r0 < R; r0 += 8) {
            float2 t[8];
            double2 yv[8];
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                const size_t gi = gbase + (size_t)(r0 + r) * N;
                t[r] = make_float2(0.f, 0.f);
                if (p0) {
                    const float2 a = *reinterpret_cast<const float2*>(p0 + gi);
                    const float2 b = *reinterpret_cast<const float2*>(p1 + gi);
                    const float2 c = *reinterpret_cast<const float2*>(p2 + gi);
                    t[r] = make_float2((a.x + b.x) + c.x, (a.y + b.y) + c.y);
                }
                yv[r] = *reinterpret_cast<const double2*>(A.y + gi);
            }
#pragma unroll
            for (int r = 0; r < 8; ++r)
                sv[r0 + r] = make_float2((float)(yv[r].x - (double)t[r].x), (float)(yv[r].y - (double)t[r].y));
        }
    }

    float2 cA[R], cB[R];
    bool in_b = false;  // the result of the preconditioner is in cB (else in cA)
    if (A.precond == 1) {
        float* halo0 = &halo[0][0][0][0];
        const float* up = rank > 0 ? cluster.map_shared_rank(halo0, rank - 1) : nullptr;
        const float* dn = rank < CL - 1 ? cluster.map_shared_rank(halo0, rank + 1) : nullptr;
        constexpr int HCOPY = G * 2 * N;  // floats per halo copy
        // publish the boundary of iterate v into copy b
        auto publish = [&](const float2 (&v)[R], int b) {
            *reinterpret_cast<float2*>(&halo[b][g][0][2 * u]) = v[0];
            *reinterpret_cast<float2*>(&halo[b][g][1][2 * u]) = v[R - 1];
            if (lane == 0 || lane == 31) {
#pragma unroll
                for (int r = 0; r < R; ++r) edge[b][g][wg][lane == 31][r] = lane == 31 ? v[r].y : v[r].x;
            }
            cluster.sync();
        };
        // one Chebyshev step p <- c + om_a (s - G1 c) + om_1 (c - p), the boundary of c read from copy b
        auto step = [&](const float2 (&c)[R], float2 (&p)[R], float om_a, float om_1, int b) {
            // the pair columns of the rows above and below the group (zero beyond the image)
            float2 top = make_float2(0.f, 0.f), bot = make_float2(0.f, 0.f);
            if (g > 0) top = *reinterpret_cast<const float2*>(&halo[b][g - 1][1][2 * u]);
            else if (up) top = *reinterpret_cast<const float2*>(up + b * HCOPY + ((G - 1) * 2 + 1) * N + 2 * u);
            if (g < G - 1) bot = *reinterpret_cast<const float2*>(&halo[b][g + 1][0][2 * u]);
            else if (dn) bot = *reinterpret_cast<const float2*>(dn + b * HCOPY + 2 * u);
            // edge lanes: lane 0 takes column 2u - 1 from the last column of the warp before, lane 31 column
            // 2u + 2 from the first column of the warp after (zero at the image's first / last column)
            const float* ecol = lane == 0 ? &edge[b][g][wg > 0 ? wg - 1 : 0][1][0]
                                          : &edge[b][g][wg < NW - 1 ? wg + 1 : NW - 1][0][0];
            const bool zl = u == 0, zr = u == TPR - 1;
            float lf[R], rt[R];  // columns 2u - 1 and 2u + 2 of every row
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const float ev = ecol[r];
                const float l = __shfl_up_sync(FULL, c[r].y, 1);
                const float q = __shfl_down_sync(FULL, c[r].x, 1);
                lf[r] = zl ? 0.f : (lane == 0 ? ev : l);
                rt[r] = zr ? 0.f : (lane == 31 ? ev : q);
            }
#pragma unroll
            for (int m = 0; m < R / 2; ++m) {
                const int r0 = 2 * m, r1 = r0 + 1;
                const float2 c0 = c[r0], c1 = c[r1];
                const float2 qm = r0 > 0 ? c[r0 - 1] : top;  // row above, both columns
                const float2 qp = r1 < R - 1 ? c[r1 + 1] : bot;
                // column 2u (pair column 2u + 1; left neighbour lf, right neighbour the pair column)
                const float b0x = (2.f * c1.x + lf[r1]) + c1.y;
                const float b1x = (2.f * c0.x + lf[r0]) + c0.y;
                const float a0x = (2.f * c0.y + qm.y) + c1.y;
                const float a1x = (2.f * c1.y + c0.y) + qp.y;
                // column 2u + 1 (pair column 2u; left neighbour the pair column, right neighbour rt)
                const float b0y = (2.f * c1.y + c1.x) + rt[r1];
                const float b1y = (2.f * c0.y + c0.x) + rt[r0];
                const float a0y = (2.f * c0.x + qm.x) + c1.x;
                const float a1y = (2.f * c1.x + c0.x) + qp.x;
                const float g0x = (8.f * c0.x + a0x) + b0x, g1x = (8.f * c1.x + a1x) + b1x;
                const float g0y = (8.f * c0.y + a0y) + b0y, g1y = (8.f * c1.y + a1y) + b1y;
                p[r0].x = (c0.x + om_a * (sv[r0].x - g0x)) + om_1 * (c0.x - p[r0].x);
                p[r0].y = (c0.y + om_a * (sv[r0].y - g0y)) + om_1 * (c0.y - p[r0].y);
                p[r1].x = (c1.x + om_a * (sv[r1].x - g1x)) + om_1 * (c1.x - p[r1].x);
                p[r1].y = (c1.y + om_a * (sv[r1].y - g1y)) + om_1 * (c1.y - p[r1].y);
            }
        };
        const float a0 = (float)A.g1_a0;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            cA[r] = make_float2(a0 * sv[r].x, a0 * sv[r].y);
            cB[r] = make_float2(0.f, 0.f);
        }
        publish(cA, 0);
        int k = 1;
        for (; k + 1 < A.g1_deg; k += 2) {
            step(cA, cB, (float)A.g1_om_a[k - 1], (float)A.g1_om_1[k - 1], (k - 1) & 1);
            publish(cB, k & 1);
            step(cB, cA, (float)A.g1_om_a[k], (float)A.g1_om_1[k], k & 1);
            publish(cA, (k + 1) & 1);
        }
        if (k < A.g1_deg) {
            step(cA, cB, (float)A.g1_om_a[k - 1], (float)A.g1_om_1[k - 1], (k - 1) & 1);
            publish(cB, k & 1);
            in_b = true;
        }
    } else if (A.precond == 2) {
        // (s - Pi s)/4 + Pi s/12, Pi the mean of the 2x2 cell (rows r0, r0 + 1; columns 2u, 2u + 1)
#pragma unroll
        for (int r0 = 0; r0 < R; r0 += 2) {
            const float mu = ((sv[r0].x + sv[r0].y) + (sv[r0 + 1].x + sv[r0 + 1].y)) * 0.25f;
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const float2 v = sv[r0 + q];
                cA[r0 + q] = make_float2((v.x - mu) * 0.25f + mu / 12.f, (v.y - mu) * 0.25f + mu / 12.f);
            }
        }
    } else {
#pragma unroll
        for (int r = 0; r < R; ++r) cA[r] = sv[r];
    }

    // outer update in FP64
    const double oa = A.om_img ? A.om_img[2 * img] : A.om_a;
    const double o1 = A.om_img ? A.om_img[2 * img + 1] : A.om_1;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const size_t gi = gbase + (size_t)r * N;
        const float2 rv = in_b ? cB[r] : cA[r];
        const double r0 = (double)rv.x, r1 = (double)rv.y;
        double2 out;
        if (!A.x) {
            out = make_double2(A.a0 * r0, A.a0 * r1);
        } else {
            const double2 xv = *reinterpret_cast<const double2*>(A.x + gi);
            const double2 pv = A.xp ? *reinterpret_cast<const double2*>(A.xp + gi) : make_double2(0.0, 0.0);
            out = make_double2(xv.x + oa * r0 + o1 * (xv.x - pv.x), xv.y + oa * r1 + o1 * (xv.y - pv.y));
        }
        *reinterpret_cast<double2*>(A.xn + gi) = out;
    }
}

template <int n, int BAND>
static int launch_os_reg(const OuterStepArgs& A, int nimg, cudaStream_t st) {
    constexpr int N = 1 << n;
    constexpr int CL = N / BAND;
    auto kern = outer_step_reg_kernel<n, BAND>;
    if (CL > 8) {
        if (int rc = cuda_status(cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1),
                                 "outer_step cluster attribute"))
            return rc;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nimg * CL);
    cfg.blockDim = dim3(N / 2 * (BAND / OSR_R));
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CL;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kern, A);
    return launch_status("outer_step_reg_kernel");
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
    cudaLaunchKernelEx(&cfg, kern, A);
    return launch_status("outer_step_kernel");
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
template <int n>
static int launch_os_reg_auto(const OuterStepArgs& A, int nimg, int band, cudaStream_t st) {
    constexpr int N = 1 << n;
    const bool b16 = band ? band == 16 : (long)nimg * (N / 32) < device_sm_count();
    if constexpr (N / 16 <= 16) {
        if (b16) return launch_os_reg<n, 16>(A, nimg, st);
    }
    return launch_os_reg<n, 32>(A, nimg, st);
}

static int dispatch_os_reg(int n, const OuterStepArgs& A, int nimg, int band, cudaStream_t st) {
    switch (n) {
        case 6: return launch_os_reg_auto<6>(A, nimg, band, st);
        case 7: return launch_os_reg_auto<7>(A, nimg, band, st);
        case 8: return launch_os_reg_auto<8>(A, nimg, band, st);
        case 9: return launch_os_reg_auto<9>(A, nimg, band, st);
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
    // FP32 stencil on FP32 partial images: the register-resident form where it exists, unless the shared-memory
    // form is asked for
    if (!shared_form && dtype == ADRT_F32 && parts_dtype == ADRT_F32 && n >= 6 && n <= 9)
        return dispatch_os_reg(n, A, nimg, band, st);
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

}  // namespace adrt
