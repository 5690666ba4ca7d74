// Row engine: per offset-frequency row, the butterflies B_m (levels lo..hi), their adjoints and the fused Chebyshev
// filter z = p_k(M) y, M = B^* B (reference: cpp/oblique.cpp:22-104, fastops.RowEngine fastops.py:70-138).
//
// Fast kernel (n <= 8; the compile-time programs also n = 9..11 in FP32). A row of N = 2^n complex values is held in
// registers by a group of T = 2^(n-r) lanes, each holding R = 2^r values, r = ceil(n/2) (r = 4 from n = 9 on, where
// a row spans 1, 2 or 4 warps and the index bits neither layout holds in registers, 4..n-5, are warp-shuffle levels). Butterflies run in place: level m pairs the values whose physical index
// differs in bit m-1, with twiddles z^t, z^(t+1), t = bitrev_{m-1}(p mod 2^(m-1)); in-place forward levels leave the
// row in bit-reversed order and the adjoint levels restore it, so an M = B^* B application needs no permutation.
// Two register layouts cover the index bits:
//   A: p = j + R*u  (register index j = low r bits; levels 1..r run in registers, twiddles shared by all lanes)
//   B: p = u + T*j  (register index j = high r bits; levels r+1..n run in registers, per-lane twiddles)
// and the row moves between them through an XOR-swizzled shared-memory buffer (one per group, conflict free for
// the 16-byte A-side and 8-byte B-side accesses). Work is taken by whole warps from an atomic counter over rows
// sorted by cost, so the groups of a warp normally share a frequency (same degree, no divergence).
//
// Simple kernel (any n <= 11, any lo): one CTA per row, the row in shared memory in natural order, ping-pong
// levels exactly as cpp/oblique.cpp:22-51. Used for op lists the fast kernel does not cover.
#pragma once
#include <type_traits>

#include "common.cuh"
#include "launch.h"

namespace adrt {

template <typename real> struct TwSrc {
    const cplx<real>* roots;  // mode 0: roots of unity, z_k^t = roots[(k t) mod L]
    const cplx<real>* tab;    // mode 1: per-row table of z^t
    int Lmask;
    int tstride;
    __device__ __forceinline__ cplx<real> get(int key, int t) const {
        if (roots) return roots[(key * t) & Lmask];
        return tab[(size_t)key * tstride + t];
    }
};

template <int n> struct FastCfg {
    static constexpr int N = 1 << n;
    // register bits r = ceil(n/2) up to n = 8; from n = 9 on a lane keeps 16 values and a row spans T = 2^(n-4)
    // lanes (1, 2, 4 warps at n = 9, 10, 11), so index bits 4..n-5 are held by neither layout's registers: they run
    // as warp-shuffle levels in the A layout (bit 4 + s is lane bit s, partner lane u ^ 2^s)
    static constexpr int r = n >= 9 ? 4 : (n + 1) / 2;
    static constexpr int R = 1 << r;
    static constexpr int tb = n - r;
    static constexpr int T = 1 << tb;
    static constexpr int WPG = T > 32 ? T / 32 : 1;  // warps per row group (named barrier when > 1)
    static constexpr int BLO = imax(r, tb);  // the B layout's registers hold index bits BLO..n-1
    static constexpr int MID = BLO - r;      // shuffle levels r+1..BLO
    static_assert(MID <= 3 && (MID == 0 || r + MID <= r + 5), "shuffle levels must stay within a warp's lane bits");
    // per-row table z^0..z^(2^(BLO-1)) in shared memory for the lane-dependent shuffle-level twiddles (MID >= 2)
    static constexpr int ZT = MID >= 2 ? (1 << (BLO - 1)) + 1 : 0;
    static constexpr int NB = (n > BLO) ? ((1 << (BLO - tb)) * ((1 << (n - BLO)) - 1)) : 0;
    static constexpr int SW_SHIFT = imax(r, 4);
    static constexpr int SW_MASK = (1 << imin(r - 1, 3)) - 1;
    static constexpr int PAD = (T < 16) ? 8 : 0;
    static constexpr int BUF = N + PAD;
    // shared memory of one row group in complex elements: exchange buffer, filter input, twiddle table, work slot
    static constexpr int GS = BUF + N + ((ZT + 1) & ~1) + (WPG > 1 ? 2 : 0);
    __host__ __device__ static constexpr int phys(int p) { return p ^ (((p >> SW_SHIFT) & SW_MASK) << 1); }
    __host__ __device__ static constexpr int offB(int b) { return (1 << (BLO - tb)) * ((1 << (b - BLO)) - 1); }
};

// pair store/load at an even physical index (16 B for float, 2 x 16 B for double)
__device__ __forceinline__ void st2(float2* p, float2 a, float2 b) {
    *reinterpret_cast<float4*>(p) = make_float4(a.x, a.y, b.x, b.y);
}
__device__ __forceinline__ void st2(double2* p, double2 a, double2 b) { p[0] = a; p[1] = b; }
__device__ __forceinline__ void ld2(const float2* p, float2& a, float2& b) {
    float4 q = *reinterpret_cast<const float4*>(p);
    a = make_float2(q.x, q.y);
    b = make_float2(q.z, q.w);
}
__device__ __forceinline__ void ld2(const double2* p, double2& a, double2& b) { a = p[0]; b = p[1]; }

// logical index of physical slot p after in-place forward levels lo..hi (lo <= 2): bit reversal of the low hi bits
__device__ __forceinline__ int bfly_perm(int p, int hi) {
    const int mask = (1 << hi) - 1;
    return (p & ~mask) | (int)(__brev((unsigned)(p & mask)) >> (32 - hi));
}

template <typename C, int n> struct Lanes {
    using F = FastCfg<n>;
    static constexpr int r = F::r, R = F::R, T = F::T, tb = F::tb, NB = F::NB;

    __device__ __forceinline__ static void fwdA(C (&v)[R], const C (&tA)[R / 2 + 1], int lo, int hi) {
#pragma unroll
        for (int b = 0; b < r; ++b) {
            if (b + 1 >= lo && b + 1 <= hi) {
#pragma unroll
                for (int j = 0; j < R; ++j) {
                    if (j & (1 << b)) continue;
                    const int t = brev(j & ((1 << b) - 1), b);
                    const C f0 = v[j], f1 = v[j | (1 << b)];
                    v[j] = cfma(tA[t], f1, f0);
                    v[j | (1 << b)] = cfma(tA[t + 1], f1, f0);
                }
            }
        }
    }
    __device__ __forceinline__ static void adjA(C (&v)[R], const C (&tA)[R / 2 + 1], int lo, int hi) {
#pragma unroll
        for (int b = r - 1; b >= 0; --b) {
            if (b + 1 >= lo && b + 1 <= hi) {
#pragma unroll
                for (int j = 0; j < R; ++j) {
                    if (j & (1 << b)) continue;
                    const int t = brev(j & ((1 << b) - 1), b);
                    const C g0 = v[j], g1 = v[j | (1 << b)];
                    v[j] = cadd(g0, g1);
                    v[j | (1 << b)] = cdot2c(tA[t], g0, tA[t + 1], g1);
                }
            }
        }
    }
    __device__ __forceinline__ static void fwdB(C (&v)[R], const C (&t0)[NB ? NB : 1], const C (&t1)[NB ? NB : 1], int lo,
                                                int hi) {
#pragma unroll
        for (int b = F::BLO; b < n; ++b) {
            if (b + 1 >= lo && b + 1 <= hi) {
                const int jb = b - tb;
#pragma unroll
                for (int j = 0; j < R; ++j) {
                    if (j & (1 << jb)) continue;
                    const int idx = F::offB(b) + (j & ((1 << jb) - 1));
                    const C f0 = v[j], f1 = v[j | (1 << jb)];
                    v[j] = cfma(t0[idx], f1, f0);
                    v[j | (1 << jb)] = cfma(t1[idx], f1, f0);
                }
            }
        }
    }
    __device__ __forceinline__ static void adjB(C (&v)[R], const C (&t0)[NB ? NB : 1], const C (&t1)[NB ? NB : 1], int lo,
                                                int hi) {
#pragma unroll
        for (int b = n - 1; b >= F::BLO; --b) {
            if (b + 1 >= lo && b + 1 <= hi) {
                const int jb = b - tb;
#pragma unroll
                for (int j = 0; j < R; ++j) {
                    if (j & (1 << jb)) continue;
                    const int idx = F::offB(b) + (j & ((1 << jb) - 1));
                    const C g0 = v[j], g1 = v[j | (1 << jb)];
                    v[j] = cadd(g0, g1);
                    v[j | (1 << jb)] = cdot2c(t0[idx], g0, t1[idx], g1);
                }
            }
        }
    }
    // z^t for t <= R: tA holds t <= R/2, the rest is z^(R/2) z^(t - R/2) (t is a compile-time constant here)
    __device__ __forceinline__ static C twx(const C (&tA)[R / 2 + 1], int t) {
        return t <= R / 2 ? tA[t] : cmul(tA[R / 2], tA[t - R / 2]);
    }
    // the shuffle levels (index bits r + s, s < MID) in the A layout, p = j + R u: the pair partner of slot j is slot j
    // of lane u ^ 2^s, and the twiddle index is t = bitrev_(r+s)(p mod 2^(r+s)) = bitrev_r(j) 2^s + bitrev_s(u mod 2^s)
    // (the same in every lane for s = 0; from the per-row table zt otherwise)
    __device__ __forceinline__ static void mid_tw(const C (&tA)[R / 2 + 1], const C* zt, int s, int j, int ul, C& za,
                                                  C& zb) {
        if (s == 0) {
            za = twx(tA, brev(j, r));
            zb = twx(tA, brev(j, r) + 1);
        } else {
            const int t = (brev(j, r) << s) | ul;
            za = zt[t];
            zb = zt[t + 1];
        }
    }
    __device__ __forceinline__ static void fwdM(C (&v)[R], const C (&tA)[R / 2 + 1], int lo, int hi, int u,
                                                const C* zt = nullptr) {
#pragma unroll
        for (int s = 0; s < F::MID; ++s) {
            if (r + s + 1 >= lo && r + s + 1 <= hi) {
                const bool upper = (u >> s) & 1;
                const int ul = s ? (int)(__brev((unsigned)(u & ((1 << s) - 1))) >> (32 - (s ? s : 1))) : 0;
#pragma unroll
                for (int j = 0; j < R; ++j) {
                    C o, za, zb;
                    o.x = __shfl_xor_sync(0xffffffffu, v[j].x, 1 << s);
                    o.y = __shfl_xor_sync(0xffffffffu, v[j].y, 1 << s);
                    mid_tw(tA, zt, s, j, ul, za, zb);
                    const C f0 = upper ? o : v[j], f1 = upper ? v[j] : o;
                    v[j] = cfma(upper ? zb : za, f1, f0);
                }
            }
        }
    }
    __device__ __forceinline__ static void adjM(C (&v)[R], const C (&tA)[R / 2 + 1], int lo, int hi, int u,
                                                const C* zt = nullptr) {
#pragma unroll
        for (int s = F::MID - 1; s >= 0; --s) {
            if (r + s + 1 >= lo && r + s + 1 <= hi) {
                const bool upper = (u >> s) & 1;
                const int ul = s ? (int)(__brev((unsigned)(u & ((1 << s) - 1))) >> (32 - (s ? s : 1))) : 0;
#pragma unroll
                for (int j = 0; j < R; ++j) {
                    C o, za, zb;
                    o.x = __shfl_xor_sync(0xffffffffu, v[j].x, 1 << s);
                    o.y = __shfl_xor_sync(0xffffffffu, v[j].y, 1 << s);
                    mid_tw(tA, zt, s, j, ul, za, zb);
                    const C g0 = upper ? o : v[j], g1 = upper ? v[j] : o;
                    v[j] = upper ? cdot2c(za, g0, zb, g1) : cadd(g0, g1);
                }
            }
        }
    }
    // barrier of one row group: the warp's lanes, or a named barrier over the group's warps
    __device__ __forceinline__ static void gsync(unsigned gmask) {
        if (F::WPG > 1) {
            asm volatile("bar.sync %0, %1;" ::"r"(1 + (int)(threadIdx.x / T)), "r"(T) : "memory");
        } else {
            __syncwarp(gmask);
        }
    }
    // A layout -> B layout through the group's buffer
    __device__ __forceinline__ static void toB(C (&v)[R], C* buf, int u, unsigned gmask) {
        if (R >= 2) {
#pragma unroll
            for (int j = 0; j < R; j += 2) st2(buf + F::phys(j + R * u), v[j], v[j + 1]);
        }
        gsync(gmask);
#pragma unroll
        for (int j = 0; j < R; ++j) v[j] = buf[F::phys(u + T * j)];
        gsync(gmask);
    }
    __device__ __forceinline__ static void toA(C (&v)[R], C* buf, int u, unsigned gmask) {
#pragma unroll
        for (int j = 0; j < R; ++j) buf[F::phys(u + T * j)] = v[j];
        gsync(gmask);
#pragma unroll
        for (int j = 0; j < R; j += 2) ld2(buf + F::phys(j + R * u), v[j], v[j + 1]);
        gsync(gmask);
    }
    __device__ __forceinline__ static void fwd(C (&v)[R], const C (&tA)[R / 2 + 1], const C (&t0)[NB ? NB : 1],
                                               const C (&t1)[NB ? NB : 1], int lo, int hi, C* buf, int u, unsigned gm,
                                               const C* zt = nullptr) {
        fwdA(v, tA, lo, hi);
        if (hi > r) {
            fwdM(v, tA, lo, hi, u, zt);
            toB(v, buf, u, gm);
            fwdB(v, t0, t1, lo, hi);
            toA(v, buf, u, gm);
        }
    }
    __device__ __forceinline__ static void adj(C (&v)[R], const C (&tA)[R / 2 + 1], const C (&t0)[NB ? NB : 1],
                                               const C (&t1)[NB ? NB : 1], int lo, int hi, C* buf, int u, unsigned gm,
                                               const C* zt = nullptr) {
        if (hi > r) {
            toB(v, buf, u, gm);
            adjB(v, t0, t1, lo, hi);
            toA(v, buf, u, gm);
            adjM(v, tA, lo, hi, u, zt);
        }
        adjA(v, tA, lo, hi);
    }
    __device__ __forceinline__ static void gram(C (&v)[R], const C (&tA)[R / 2 + 1], const C (&t0)[NB ? NB : 1],
                                                const C (&t1)[NB ? NB : 1], int lo, int hi, C* buf, int u, unsigned gm,
                                               const C* zt = nullptr) {
        fwdA(v, tA, lo, hi);
        if (hi > r) {
            fwdM(v, tA, lo, hi, u, zt);
            toB(v, buf, u, gm);
            fwdB(v, t0, t1, lo, hi);
            adjB(v, t0, t1, lo, hi);
            toA(v, buf, u, gm);
            adjM(v, tA, lo, hi, u, zt);
        }
        adjA(v, tA, lo, hi);
    }
};

// ------------------------------------------------------------------ compile-time programs (the hot op lists)
// The four op lists of the packed inverses (fastops.py:277-285, 325-335) with their level ranges fixed at compile
// time: no op interpreter, no runtime level checks, one Gram body in the code (the trailing M of G_h / frame
// reuses the loop body), the first forward level out of place (no copy of z), and the recurrence in momentum form
//     r = y - M z - tau z ;  d = om a r + (om - 1) d ;  z = z + d          (d = z_j - z_{j-1}; z_1 = d_1 = a y)
// which equals z_{j+1} = z_j + om a r + (om - 1)(z_j - z_{j-1}) (cpp/oblique.cpp:93-97) without register rotation.
constexpr int FAST_THREADS = 256;
enum { PROG_GH_HYB = 1, PROG_BP_HYB = 2, PROG_FRAME_LP = 3, PROG_BP_LP = 4 };

template <typename C, int n> struct CtLanes {
    using F = FastCfg<n>;
    using Ln = Lanes<C, n>;
    static constexpr int r = F::r, R = F::R, T = F::T, tb = F::tb, NB = F::NB;
    // forward levels LO..HI; level LO reads src and writes dst, the rest run in place on dst (A layout in and out)
    template <int LO, int HI>
    __device__ __forceinline__ static void fwd_oop(const C (&src)[R], C (&dst)[R], const C (&tA)[R / 2 + 1],
                                                   const C (&t0)[NB ? NB : 1], const C (&t1)[NB ? NB : 1], C* buf, int u,
                                                   unsigned gm, const C* zt) {
#pragma unroll
        for (int b = 0; b < r; ++b) {
            if (b + 1 >= LO && b + 1 <= HI) {
#pragma unroll
                for (int j = 0; j < R; ++j) {
                    if (j & (1 << b)) continue;
                    const int t = brev(j & ((1 << b) - 1), b);
                    const C f0 = (b + 1 == LO) ? src[j] : dst[j];
                    const C f1 = (b + 1 == LO) ? src[j | (1 << b)] : dst[j | (1 << b)];
                    dst[j] = cfma(tA[t], f1, f0);
                    dst[j | (1 << b)] = cfma(tA[t + 1], f1, f0);
                }
            }
        }
        if (HI > r) {
            Ln::fwdM(dst, tA, LO, HI, u, zt);
            Ln::toB(dst, buf, u, gm);
            Ln::fwdB(dst, t0, t1, LO, HI);
        }
    }
    // Gram M = B^* B over LO..HI: src (A layout) -> dst (A layout)
    template <int LO, int HI>
    __device__ __forceinline__ static void gram_oop(const C (&src)[R], C (&dst)[R], const C (&tA)[R / 2 + 1],
                                                    const C (&t0)[NB ? NB : 1], const C (&t1)[NB ? NB : 1], C* buf,
                                                    int u, unsigned gm, const C* zt) {
        fwd_oop<LO, HI>(src, dst, tA, t0, t1, buf, u, gm, zt);
        if (HI > r) {
            Ln::adjB(dst, t0, t1, LO, HI);
            Ln::toA(dst, buf, u, gm);
            Ln::adjM(dst, tA, LO, HI, u, zt);
        }
        Ln::adjA(dst, tA, LO, HI);
    }
};

// one work item (row `item` of the job's selection, all images interleaved) of a compile-time row program, run by
// the T lanes of one row group: buf is the group's shared memory (exchange buffer, filter input, twiddle table)
template <typename real, int n, int PROG>
__device__ __forceinline__ void prog_item(const adrt_row_job& J, const TwSrc<real> tw, const int item,
                                          cplx<real>* buf, const int u, const unsigned gm) {
    using C = cplx<real>;
    using F = FastCfg<n>;
    using Ln = Lanes<C, n>;
    using Ct = CtLanes<C, n>;
    constexpr int N = F::N, R = F::R, T = F::T, tb = F::tb, NB = F::NB;
    constexpr bool HYB = (PROG == PROG_GH_HYB || PROG == PROG_BP_HYB);
    constexpr int LO = HYB ? 2 : 1;  // filter levels LO..n
    constexpr bool BP = (PROG == PROG_BP_HYB || PROG == PROG_BP_LP);
    C* ybuf = buf + F::BUF;
    C* zt = ybuf + F::N;  // shuffle-level twiddles (MID >= 2)
    C* X = reinterpret_cast<C*>(J.X);
    const real tau = (real)J.tau;
    const real* coefs = reinterpret_cast<const real*>(J.coef);
    const int sel = item / J.nimg;
    const int img = item - sel * J.nimg;
    const int row = J.rows ? J.rows[sel] : sel;
    const int k = row % J.freq_mod;
    const int key = tw.roots ? k : row;
    C* ptr = X + (size_t)img * J.img_stride + (size_t)row * N;
    const real* cf = coefs + (size_t)k * J.coef_stride;
    const int d = J.deg[k];
    const real a = cf[0];

    C tA[R / 2 + 1];
#pragma unroll
    for (int t = 0; t <= R / 2; ++t) tA[t] = tw.get(key, t);
    C t0[NB ? NB : 1], t1[NB ? NB : 1];
    if (NB) {
        const int U = tb ? (int)(__brev((unsigned)u) >> (32 - tb)) : 0;
#pragma unroll
        for (int b = F::BLO; b < n; ++b) {
            const int jb = b - tb;
#pragma unroll
            for (int vv = 0; vv < (1 << jb); ++vv) {
                const int t = (U << jb) + brev(vv, jb);
                t0[F::offB(b) + vv] = tw.get(key, t);
                t1[F::offB(b) + vv] = tw.get(key, t + 1);
            }
        }
    }

    if (F::ZT) {
#pragma unroll 1
        for (int t = u; t < F::ZT; t += T) zt[t] = tw.get(key, t);
        Ln::gsync(gm);
    }

    C v[R], w[R], dl[R];
    if (BP) {
        // the back-projections start with the adjoint levels LO..n on rows in natural (slope) order
#pragma unroll
        for (int j = 0; j < R; ++j) v[j] = ptr[bfly_perm(j + R * u, n)];
        Ln::adj(v, tA, t0, t1, LO, n, buf, u, gm, zt);
    } else {
#pragma unroll
        for (int j = 0; j < R; j += 2) ld2(ptr + j + R * u, v[j], v[j + 1]);
        if (PROG == PROG_GH_HYB) Ln::fwdA(v, tA, 1, 1);  // B_1
    }
    // filter input y -> shared memory; z_1 = d_1 = a y
#pragma unroll
    for (int j = 0; j < R; j += 2) st2(ybuf + F::phys(j + R * u), v[j], v[j + 1]);
#pragma unroll
    for (int j = 0; j < R; ++j) {
        v[j] = cscale(a, v[j]);
        dl[j] = v[j];
    }
    // G_h and the frame end with M applied to z_d: one more pass of the loop body without the update
    const int steps = BP ? d - 1 : d;
    real om_a = d > 1 ? cf[2] : (real)0, om_1 = d > 1 ? cf[3] : (real)0;  // step 1
    for (int s = 1; s <= steps; ++s) {
        const real na = (s + 1 < d) ? cf[3 * s + 2] : (real)0, n1 = (s + 1 < d) ? cf[3 * s + 3] : (real)0;
        Ct::template gram_oop<LO, n>(v, w, tA, t0, t1, buf, u, gm, zt);
        if (s == d) break;  // w = M z_d
#pragma unroll
        for (int j = 0; j < R; j += 2) {
            C y0, y1;
            ld2(ybuf + F::phys(j + R * u), y0, y1);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const C yy = h ? y1 : y0;
                C rr = csub(yy, w[j + h]);
                rr.x = fma(-tau, v[j + h].x, rr.x);
                rr.y = fma(-tau, v[j + h].y, rr.y);
                dl[j + h].x = fma(om_1, dl[j + h].x, om_a * rr.x);
                dl[j + h].y = fma(om_1, dl[j + h].y, om_a * rr.y);
                v[j + h] = cadd(v[j + h], dl[j + h]);
            }
        }
        om_a = na;
        om_1 = n1;
    }
    if (BP) {
        if (PROG == PROG_BP_HYB) Ln::adjA(v, tA, 1, 1);  // B_1^*
#pragma unroll
        for (int j = 0; j < R; j += 2) st2(ptr + j + R * u, v[j], v[j + 1]);
    } else {
        if (PROG == PROG_GH_HYB) Ln::adjA(w, tA, 1, 1);  // B_1^*
#pragma unroll
        for (int j = 0; j < R; j += 2) st2(ptr + j + R * u, w[j], w[j + 1]);
    }
}

// the op lists of the packed inverses, recognised for the compile-time kernels (hybrid needs n >= 2)
inline int match_prog(const adrt_row_job& J) {
    const int n = J.n;
    auto is = [&](int o, int op, int lo, int hi) { return J.op[o] == op && J.lo[o] == lo && J.hi[o] == hi; };
    if (n >= 2 && J.nops == 4 && is(0, ADRT_OP_B, 1, 1) && is(1, ADRT_OP_P, 2, n) && is(2, ADRT_OP_M, 2, n) &&
        is(3, ADRT_OP_BT, 1, 1))
        return PROG_GH_HYB;
    if (n >= 2 && J.nops == 3 && is(0, ADRT_OP_BT, 2, n) && is(1, ADRT_OP_P, 2, n) && is(2, ADRT_OP_BT, 1, 1))
        return PROG_BP_HYB;
    if (J.nops == 2 && is(0, ADRT_OP_P, 1, n) && is(1, ADRT_OP_M, 1, n)) return PROG_FRAME_LP;
    if (J.nops == 2 && is(0, ADRT_OP_BT, 1, n) && is(1, ADRT_OP_P, 1, n)) return PROG_BP_LP;
    return 0;
}

}  // namespace adrt
