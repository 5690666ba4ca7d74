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
#include <atomic>
#include <cstdio>
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

#define ADRT_OP_POWER 16  // internal: power iteration (adrt_power_rows)

template <typename real, int n, int THREADS, bool POWER>
__global__ void __launch_bounds__(THREADS, 1)
    rows_fast_kernel(const adrt_row_job J, const TwSrc<real> tw, const int total, const int power_iters,
                     const double power_safety, double* __restrict__ power_out, const int perm_in, const int perm_out) {
    using C = cplx<real>;
    using F = FastCfg<n>;
    using Ln = Lanes<C, n>;
    constexpr int N = F::N, R = F::R, T = F::T, tb = F::tb, NB = F::NB;
    constexpr int GPW = 32 / T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31;
    const int giw = lane / T;
    const int u = lane & (T - 1);
    // per group: exchange buffer (swizzled) then the filter input y (A layout, pairs contiguous)
    C* buf = reinterpret_cast<C*>(smem_raw) + (threadIdx.x / T) * (F::BUF + F::N);
    C* ybuf = buf + F::BUF;
    const unsigned gm = (T == 32) ? 0xffffffffu : (((1u << T) - 1u) << (giw * T));
    C* X = reinterpret_cast<C*>(J.X);
    const real tau = (real)J.tau;
    const real* coefs = reinterpret_cast<const real*>(J.coef);

    for (;;) {
        int base = 0;
        if (lane == 0) base = atomicAdd(J.counter, GPW);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= total) break;
        const bool last = base + GPW >= total;
        const int item = base + giw;
        if (item < total) {
            const int sel = item / J.nimg;
            const int img = item - sel * J.nimg;
            const int row = J.rows ? J.rows[sel] : sel;
            const int k = row % J.freq_mod;
            const int key = tw.roots ? k : row;
            C* ptr = X + (size_t)img * J.img_stride + (size_t)row * N;

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

            C v[R];
            if (perm_in) {
                const int h = J.hi[0];
#pragma unroll
                for (int j = 0; j < R; ++j) v[j] = ptr[bfly_perm(j + R * u, h)];
            } else {
#pragma unroll
                for (int j = 0; j < R; j += 2) ld2(ptr + j + R * u, v[j], v[j + 1]);
            }

            for (int o = 0; o < J.nops; ++o) {
                const int op = J.op[o], lo = J.lo[o], hi = J.hi[o];
                if (op == ADRT_OP_B) {
                    Ln::fwd(v, tA, t0, t1, lo, hi, buf, u, gm);
                } else if (op == ADRT_OP_BT) {
                    Ln::adj(v, tA, t0, t1, lo, hi, buf, u, gm);
                } else if (op == ADRT_OP_M) {
                    Ln::gram(v, tA, t0, t1, lo, hi, buf, u, gm);
                } else if (!POWER && op == ADRT_OP_P) {
                    const real* cf = coefs + (size_t)k * J.coef_stride;
                    const int d = J.deg[k];
                    const real a = cf[0];
                    C zp[R];
#pragma unroll
                    for (int j = 0; j < R; j += 2) st2(ybuf + F::phys(j + R * u), v[j], v[j + 1]);
#pragma unroll
                    for (int j = 0; j < R; ++j) {
                        v[j] = cscale(a, v[j]);
                        zp[j] = mk<real>(0, 0);
                    }
                    for (int s = 1; s < d; ++s) {
                        const real om_a = cf[3 * s - 1], om_1 = cf[3 * s];
                        C w[R];
#pragma unroll
                        for (int j = 0; j < R; ++j) w[j] = v[j];
                        Ln::gram(w, tA, t0, t1, lo, hi, buf, u, gm);
#pragma unroll
                        for (int j = 0; j < R; j += 2) {
                            C y0, y1;
                            ld2(ybuf + F::phys(j + R * u), y0, y1);
                            w[j] = csub(y0, w[j]);
                            w[j + 1] = csub(y1, w[j + 1]);
                        }
#pragma unroll
                        for (int j = 0; j < R; ++j) {
                            // r = y - M z - tau z ; z_new = z + om a r + (om - 1)(z - z_prev)   (cpp/oblique.cpp:93-97)
                            C rr = w[j];
                            rr.x = fma(-tau, v[j].x, rr.x);
                            rr.y = fma(-tau, v[j].y, rr.y);
                            C zn;
                            zn.x = fma(om_1, v[j].x - zp[j].x, fma(om_a, rr.x, v[j].x));
                            zn.y = fma(om_1, v[j].y - zp[j].y, fma(om_a, rr.y, v[j].y));
                            zp[j] = v[j];
                            v[j] = zn;
                        }
                    }
                } else if (POWER && op == ADRT_OP_POWER) {
                    // V <- M V / ||M V|| (power_iters times), then out = safety * Re <V, M V>  (fastcpp.py:109-118)
                    for (int it = 0; it <= power_iters; ++it) {
                        C w[R];
#pragma unroll
                        for (int j = 0; j < R; ++j) w[j] = v[j];
                        Ln::gram(w, tA, t0, t1, lo, hi, buf, u, gm);
                        if (it == power_iters) {
                            double s = 0;
#pragma unroll
                            for (int j = 0; j < R; ++j) s += (double)v[j].x * w[j].x + (double)v[j].y * w[j].y;
#pragma unroll
                            for (int off = T / 2; off > 0; off >>= 1) s += __shfl_xor_sync(gm, s, off);
                            if (u == 0 && img == 0) power_out[row] = power_safety * s;
                            break;
                        }
                        double s = 0;
#pragma unroll
                        for (int j = 0; j < R; ++j) s += (double)w[j].x * w[j].x + (double)w[j].y * w[j].y;
#pragma unroll
                        for (int off = T / 2; off > 0; off >>= 1) s += __shfl_xor_sync(gm, s, off);
                        const real inv = (real)(1.0 / sqrt(s));
#pragma unroll
                        for (int j = 0; j < R; ++j) v[j] = cscale(inv, w[j]);
                    }
                }
            }

            if (perm_out) {
                const int h = J.hi[J.nops - 1];
#pragma unroll
                for (int j = 0; j < R; ++j) ptr[bfly_perm(j + R * u, h)] = v[j];
            } else {
#pragma unroll
                for (int j = 0; j < R; j += 2) st2(ptr + j + R * u, v[j], v[j + 1]);
            }
        }
        if (last) break;
    }
}

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

template <typename real, int n, int THREADS, int PROG>
__global__ void __launch_bounds__(THREADS, 1)
    rows_prog_kernel(const adrt_row_job J, const TwSrc<real> tw, const int total) {
    using C = cplx<real>;
    using F = FastCfg<n>;
    using Ln = Lanes<C, n>;
    using Ct = CtLanes<C, n>;
    constexpr int N = F::N, R = F::R, T = F::T, tb = F::tb, NB = F::NB;
    constexpr int GPW = 32 / T;
    constexpr bool HYB = (PROG == PROG_GH_HYB || PROG == PROG_BP_HYB);
    constexpr int LO = HYB ? 2 : 1;  // filter levels LO..n
    constexpr bool BP = (PROG == PROG_BP_HYB || PROG == PROG_BP_LP);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31;
    const int giw = T >= 32 ? 0 : lane / T;
    const int u = threadIdx.x & (T - 1);
    C* buf = reinterpret_cast<C*>(smem_raw) + (threadIdx.x / T) * F::GS;
    C* ybuf = buf + F::BUF;
    C* zt = ybuf + F::N;  // shuffle-level twiddles (MID >= 2)
    int* slot = reinterpret_cast<int*>(zt + ((F::ZT + 1) & ~1));  // the group's work item (WPG > 1)
    const unsigned gm = (T >= 32) ? 0xffffffffu : (((1u << T) - 1u) << (giw * T));
    C* X = reinterpret_cast<C*>(J.X);
    const real tau = (real)J.tau;
    const real* coefs = reinterpret_cast<const real*>(J.coef);

    for (;;) {
        int item = 0;
        bool last = false;
        if (F::WPG > 1) {
            // a row spans several warps: the group's first thread takes the item, a named barrier shares it (the
            // second barrier keeps the slot until every warp of the group has read it)
            if (u == 0) *slot = atomicAdd(J.counter, 1);
            Ln::gsync(gm);
            item = *slot;
            Ln::gsync(gm);
            if (item >= total) break;
        } else {
            int base = 0;
            if (lane == 0) base = atomicAdd(J.counter, GPW);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= total) break;
            last = base + GPW >= total;
            item = base + giw;
        }
        if (item < total) {
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
        if (last) break;
    }
}

// ------------------------------------------------------------------ simple kernel (natural order, shared memory)
template <typename real>
__device__ void simple_fwd(cplx<real>*& a, cplx<real>*& b, int N, int lo, int hi, const TwSrc<real>& tw, int key) {
    using C = cplx<real>;
    for (int m = lo; m <= hi; ++m) {
        const int w = 1 << (m - 1);
        for (int i = threadIdx.x; i < N / 2; i += blockDim.x) {
            const int l = i / w, t = i - l * w, base = l * 2 * w;
            const C f0 = a[base + t], f1 = a[base + w + t];
            b[base + 2 * t] = cfma(tw.get(key, t), f1, f0);
            b[base + 2 * t + 1] = cfma(tw.get(key, t + 1), f1, f0);
        }
        __syncthreads();
        C* s = a; a = b; b = s;
    }
}

template <typename real>
__device__ void simple_adj(cplx<real>*& a, cplx<real>*& b, int N, int lo, int hi, const TwSrc<real>& tw, int key) {
    using C = cplx<real>;
    for (int m = hi; m >= lo; --m) {
        const int w = 1 << (m - 1);
        for (int i = threadIdx.x; i < N / 2; i += blockDim.x) {
            const int l = i / w, t = i - l * w, base = l * 2 * w;
            const C g0 = a[base + 2 * t], g1 = a[base + 2 * t + 1];
            b[base + t] = cadd(g0, g1);
            b[base + w + t] = cdot2c(tw.get(key, t), g0, tw.get(key, t + 1), g1);
        }
        __syncthreads();
        C* s = a; a = b; b = s;
    }
}

template <typename real>
__global__ void __launch_bounds__(256) rows_simple_kernel(const adrt_row_job J, const TwSrc<real> tw, const int total,
                                                          const int power_iters, const double power_safety,
                                                          double* __restrict__ power_out) {
    using C = cplx<real>;
    const int N = 1 << J.n;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* sm = reinterpret_cast<C*>(smem_raw);
    C* bufs[5] = {sm, sm + N, sm + 2 * N, sm + 3 * N, sm + 4 * N};
    __shared__ double red[256];
    const real tau = (real)J.tau;
    const real* coefs = reinterpret_cast<const real*>(J.coef);
    for (int item = blockIdx.x; item < total; item += gridDim.x) {
        const int sel = item / J.nimg;
        const int img = item - sel * J.nimg;
        const int row = J.rows ? J.rows[sel] : sel;
        const int k = row % J.freq_mod;
        const int key = tw.roots ? k : row;
        C* ptr = reinterpret_cast<C*>(J.X) + (size_t)img * J.img_stride + (size_t)row * N;
        C* cur = bufs[0];
        C* tmp = bufs[1];
        for (int i = threadIdx.x; i < N; i += blockDim.x) cur[i] = ptr[i];
        __syncthreads();
        for (int o = 0; o < J.nops; ++o) {
            const int op = J.op[o], lo = J.lo[o], hi = J.hi[o];
            if (op == ADRT_OP_B) {
                simple_fwd<real>(cur, tmp, N, lo, hi, tw, key);
            } else if (op == ADRT_OP_BT) {
                simple_adj<real>(cur, tmp, N, lo, hi, tw, key);
            } else if (op == ADRT_OP_M) {
                simple_fwd<real>(cur, tmp, N, lo, hi, tw, key);
                simple_adj<real>(cur, tmp, N, lo, hi, tw, key);
            } else {
                // the four buffers other than the current one
                C* oth[4];
                for (int q = 0, no = 0; q < 5; ++q)
                    if (bufs[q] != cur) oth[no++] = bufs[q];
                if (op == ADRT_OP_P) {
                    const real* cf = coefs + (size_t)k * J.coef_stride;
                    const int d = J.deg[k];
                    const real a = cf[0];
                    C* y = cur;
                    C* z = oth[0];
                    C* zp = oth[1];
                    for (int i = threadIdx.x; i < N; i += blockDim.x) {
                        z[i] = cscale(a, y[i]);
                        zp[i] = mk<real>(0, 0);
                    }
                    __syncthreads();
                    for (int s = 1; s < d; ++s) {
                        const real om_a = cf[3 * s - 1], om_1 = cf[3 * s];
                        C* pa = oth[2];
                        C* pb = oth[3];
                        for (int i = threadIdx.x; i < N; i += blockDim.x) pa[i] = z[i];
                        __syncthreads();
                        simple_fwd<real>(pa, pb, N, lo, hi, tw, key);
                        simple_adj<real>(pa, pb, N, lo, hi, tw, key);
                        for (int i = threadIdx.x; i < N; i += blockDim.x) {
                            C rr = csub(y[i], pa[i]);
                            rr.x = fma(-tau, z[i].x, rr.x);
                            rr.y = fma(-tau, z[i].y, rr.y);
                            C zn;
                            zn.x = fma(om_1, z[i].x - zp[i].x, fma(om_a, rr.x, z[i].x));
                            zn.y = fma(om_1, z[i].y - zp[i].y, fma(om_a, rr.y, z[i].y));
                            zp[i] = z[i];
                            z[i] = zn;
                        }
                        __syncthreads();
                    }
                    cur = z;
                    tmp = y;
                } else {  // ADRT_OP_POWER
                    for (int it = 0; it <= power_iters; ++it) {
                        C* pa = oth[0];
                        C* pb = oth[1];
                        for (int i = threadIdx.x; i < N; i += blockDim.x) pa[i] = cur[i];
                        __syncthreads();
                        simple_fwd<real>(pa, pb, N, lo, hi, tw, key);
                        simple_adj<real>(pa, pb, N, lo, hi, tw, key);
                        double s = 0;
                        for (int i = threadIdx.x; i < N; i += blockDim.x)
                            s += (it == power_iters) ? (double)cur[i].x * pa[i].x + (double)cur[i].y * pa[i].y
                                                     : (double)pa[i].x * pa[i].x + (double)pa[i].y * pa[i].y;
                        red[threadIdx.x] = s;
                        __syncthreads();
                        for (int off = blockDim.x / 2; off > 0; off >>= 1) {
                            if ((int)threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
                            __syncthreads();
                        }
                        s = red[0];
                        __syncthreads();
                        if (it == power_iters) {
                            if (threadIdx.x == 0 && img == 0) power_out[row] = power_safety * s;
                            break;
                        }
                        const real inv = (real)(1.0 / sqrt(s));
                        for (int i = threadIdx.x; i < N; i += blockDim.x) cur[i] = cscale(inv, pa[i]);
                        __syncthreads();
                    }
                }
            }
        }
        for (int i = threadIdx.x; i < N; i += blockDim.x) ptr[i] = cur[i];
        __syncthreads();
    }
}

// ------------------------------------------------------------------ twiddle table (binary powering in FP64)
template <typename real>
__global__ void twiddle_table_kernel(int n, int K, const double2* __restrict__ z, cplx<real>* __restrict__ tab) {
    const int H = (1 << n) / 2 + 1;
    const long total = (long)K * H;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int k = (int)(i / H), t = (int)(i - (long)k * H);
        double2 base = z[k], acc = make_double2(1.0, 0.0);
        for (int e = t; e; e >>= 1) {
            if (e & 1) acc = cmul(base, acc);
            base = cmul(base, base);
        }
        tab[i] = mk<real>((real)acc.x, (real)acc.y);
    }
}

// ------------------------------------------------------------------ dispatch
// SM count of the current device, cached per device index (grids are sized for the GPU they run on)
static int num_sms() {
    constexpr int kMaxDev = 64;
    static std::atomic<int> cache[kMaxDev];
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= kMaxDev) dev = 0;
    int sms = cache[dev].load(std::memory_order_relaxed);
    if (sms <= 0) {
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
        cache[dev].store(sms, std::memory_order_relaxed);
    }
    return sms;
}

int device_sm_count() { return num_sms(); }


template <typename real, int n>
static int launch_fast(const adrt_row_job& J, const TwSrc<real>& tw, int total, int iters, double safety, double* pout,
                       cudaStream_t st) {
    using F = FastCfg<n>;
    const size_t smem = (size_t)(FAST_THREADS / F::T) * F::GS * sizeof(cplx<real>);
    auto kern = pout ? rows_fast_kernel<real, n, FAST_THREADS, true> : rows_fast_kernel<real, n, FAST_THREADS, false>;
    if (int rc = ensure_smem((const void*)kern, smem)) return rc;
    const int grid = J.grid > 0 ? J.grid : num_sms();
    // in-place butterflies leave a lone forward op (last) in bit-reversed order and expect a lone adjoint op
    // (first) in that order: fold the permutation into the store / load
    const int last = J.nops - 1;
    const int perm_in = (J.op[0] == ADRT_OP_BT && J.hi[0] >= 2) ? 1 : 0;
    const int perm_out = (J.op[last] == ADRT_OP_B && J.hi[last] >= 2) ? 1 : 0;
    kern<<<grid, FAST_THREADS, smem, st>>>(J, tw, total, iters, safety, pout, perm_in, perm_out);
    return launch_status("rows_fast_kernel");
}

template <typename real>
static int launch_simple(const adrt_row_job& J, const TwSrc<real>& tw, int total, int iters, double safety,
                         double* pout, cudaStream_t st) {
    const int N = 1 << J.n;
    const size_t smem = 5 * (size_t)N * sizeof(cplx<real>);
    auto kern = rows_simple_kernel<real>;
    if (int rc = ensure_smem((const void*)kern, smem)) return rc;
    const int threads = N / 2 >= 256 ? 256 : (N / 2 >= 32 ? N / 2 : 32);
    int grid = num_sms() * 8;
    if (grid > total) grid = total;
    if (grid < 1) grid = 1;
    kern<<<grid, threads, smem, st>>>(J, tw, total, iters, safety, pout);
    return launch_status("rows_simple_kernel");
}

// the register kernel runs in-place levels with lo <= 2 and needs every op but a leading adjoint / trailing forward
// to start and end in natural order (B with hi >= 2 only last, BT with hi >= 2 only first)
static bool fast_levels_ok(const adrt_row_job& J) {
    for (int o = 0; o < J.nops; ++o) {
        if (J.lo[o] > 2) return false;
        if (J.op[o] == ADRT_OP_B && J.hi[o] >= 2 && o != J.nops - 1) return false;
        if (J.op[o] == ADRT_OP_BT && J.hi[o] >= 2 && o != 0) return false;
    }
    return true;
}

static bool fast_ok(const adrt_row_job& J) { return J.n >= 1 && J.n <= 8 && fast_levels_ok(J); }

template <typename real, int n>
static int launch_prog(const adrt_row_job& J, const TwSrc<real>& tw, int total, int prog, cudaStream_t st) {
    using F = FastCfg<n>;
    const size_t smem = (size_t)(FAST_THREADS / F::T) * F::GS * sizeof(cplx<real>);
    void (*kern)(const adrt_row_job, const TwSrc<real>, const int) = nullptr;
    switch (prog) {
        case PROG_GH_HYB: kern = rows_prog_kernel<real, n, FAST_THREADS, PROG_GH_HYB>; break;
        case PROG_BP_HYB: kern = rows_prog_kernel<real, n, FAST_THREADS, PROG_BP_HYB>; break;
        case PROG_FRAME_LP: kern = rows_prog_kernel<real, n, FAST_THREADS, PROG_FRAME_LP>; break;
        default: kern = rows_prog_kernel<real, n, FAST_THREADS, PROG_BP_LP>; break;
    }
    if (int rc = ensure_smem((const void*)kern, smem)) return rc;
    const int grid = J.grid > 0 ? J.grid : num_sms();
    kern<<<grid, FAST_THREADS, smem, st>>>(J, tw, total);
    return launch_status("rows_prog_kernel");
}

// the op lists of the packed inverses, recognised for the compile-time kernels (hybrid needs n >= 2)
static int match_prog(const adrt_row_job& J) {
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

template <typename real>
static int rows_dispatch(const adrt_row_job& J, int iters, double safety, double* pout, cudaStream_t st) {
    TwSrc<real> tw;
    tw.roots = reinterpret_cast<const cplx<real>*>(J.roots);
    tw.tab = reinterpret_cast<const cplx<real>*>(J.twtab);
    tw.Lmask = (2 << J.n) - 1;
    tw.tstride = (1 << J.n) / 2 + 1;
    const long total_l = (long)J.nimg * J.nsel;
    if (total_l <= 0) return ADRT_OK;
    if (total_l > 0x7fffff00L) {
        set_error("rows: %ld work items exceed the 32-bit item index", total_l);
        return ADRT_EINVAL;
    }
    const int total = (int)total_l;
    // compile-time programs: n <= 8 in both precisions, n = 9..11 (shuffle levels) in FP32
    const bool prog_n = (J.n >= 1 && J.n <= 8) || (J.n <= 11 && std::is_same<real, float>::value);
    const int prog = (!pout && prog_n && fast_levels_ok(J)) ? match_prog(J) : 0;
    if (prog) {
        switch (J.n) {
            case 1: return launch_prog<real, 1>(J, tw, total, prog, st);
            case 2: return launch_prog<real, 2>(J, tw, total, prog, st);
            case 3: return launch_prog<real, 3>(J, tw, total, prog, st);
            case 4: return launch_prog<real, 4>(J, tw, total, prog, st);
            case 5: return launch_prog<real, 5>(J, tw, total, prog, st);
            case 6: return launch_prog<real, 6>(J, tw, total, prog, st);
            case 7: return launch_prog<real, 7>(J, tw, total, prog, st);
            case 8: return launch_prog<real, 8>(J, tw, total, prog, st);
            case 9:
                if constexpr (std::is_same<real, float>::value) return launch_prog<real, 9>(J, tw, total, prog, st);
                break;
            case 10:
                if constexpr (std::is_same<real, float>::value) return launch_prog<real, 10>(J, tw, total, prog, st);
                break;
            case 11:
                if constexpr (std::is_same<real, float>::value) return launch_prog<real, 11>(J, tw, total, prog, st);
                break;
        }
    }
    if (fast_ok(J)) {
        switch (J.n) {
            case 1: return launch_fast<real, 1>(J, tw, total, iters, safety, pout, st);
            case 2: return launch_fast<real, 2>(J, tw, total, iters, safety, pout, st);
            case 3: return launch_fast<real, 3>(J, tw, total, iters, safety, pout, st);
            case 4: return launch_fast<real, 4>(J, tw, total, iters, safety, pout, st);
            case 5: return launch_fast<real, 5>(J, tw, total, iters, safety, pout, st);
            case 6: return launch_fast<real, 6>(J, tw, total, iters, safety, pout, st);
            case 7: return launch_fast<real, 7>(J, tw, total, iters, safety, pout, st);
            case 8: return launch_fast<real, 8>(J, tw, total, iters, safety, pout, st);
        }
    }
    return launch_simple<real>(J, tw, total, iters, safety, pout, st);
}

static int validate_job(const adrt_row_job* J) {
    if (!J) { set_error("rows: null job"); return ADRT_EINVAL; }
    if (J->dtype != ADRT_F32 && J->dtype != ADRT_F64) { set_error("rows: dtype must be F32 or F64"); return ADRT_EINVAL; }
    if (J->n < 1 || J->n > 11) { set_error("rows: n=%d out of range 1..11", J->n); return ADRT_EINVAL; }
    if (J->nops < 1 || J->nops > ADRT_MAX_OPS) { set_error("rows: nops=%d out of range", J->nops); return ADRT_EINVAL; }
    if (!J->X || !J->counter) { set_error("rows: null X or counter"); return ADRT_EINVAL; }
    if (!J->roots && !J->twtab) { set_error("rows: need roots or twtab"); return ADRT_EINVAL; }
    if (J->freq_mod < 1) { set_error("rows: freq_mod must be >= 1"); return ADRT_EINVAL; }
    if (J->nimg < 0 || J->nsel < 0) { set_error("rows: negative counts"); return ADRT_EINVAL; }
    for (int o = 0; o < J->nops; ++o) {
        const int op = J->op[o];
        if (op != ADRT_OP_B && op != ADRT_OP_BT && op != ADRT_OP_M && op != ADRT_OP_P && op != ADRT_OP_POWER) {
            set_error("rows: bad op %d", op);
            return ADRT_EINVAL;
        }
        if (J->lo[o] < 1 || J->hi[o] > J->n || J->lo[o] > J->hi[o]) {
            set_error("rows: op %d levels [%d, %d] outside 1..%d", o, J->lo[o], J->hi[o], J->n);
            return ADRT_EINVAL;
        }
        if (op == ADRT_OP_P && (!J->deg || !J->coef)) { set_error("rows: P op needs deg and coef"); return ADRT_EINVAL; }
    }
    if ((reinterpret_cast<uintptr_t>(J->X) & 15) || (J->img_stride & 1)) {
        set_error("rows: X must be 16-byte aligned with an even image stride");
        return ADRT_EINVAL;
    }
    return ADRT_OK;
}

int rows_run(const adrt_row_job* J, int iters, double safety, double* pout, cudaStream_t st) {
    int rc = validate_job(J);
    if (rc) return rc;
    // the persistent warps take work from *counter: reset it on the stream first
    if ((rc = cuda_status(cudaMemsetAsync(J->counter, 0, sizeof(int32_t), st), "work counter reset"))) return rc;
    if (J->dtype == ADRT_F32) return rows_dispatch<float>(*J, iters, safety, pout, st);
    return rows_dispatch<double>(*J, iters, safety, pout, st);
}

int twiddle_table(int dtype, int n, int K, const double* z, void* tab, cudaStream_t st) {
    if (n < 1 || n > 11 || K < 0 || (K && (!z || !tab))) { set_error("twiddle_table: bad arguments"); return ADRT_EINVAL; }
    if (!K) return ADRT_OK;
    const long total = (long)K * ((1 << n) / 2 + 1);
    int grid = (int)((total + 255) / 256);
    if (grid > 4096) grid = 4096;
    if (dtype == ADRT_F32)
        twiddle_table_kernel<float><<<grid, 256, 0, st>>>(n, K, reinterpret_cast<const double2*>(z),
                                                           reinterpret_cast<float2*>(tab));
    else
        twiddle_table_kernel<double><<<grid, 256, 0, st>>>(n, K, reinterpret_cast<const double2*>(z),
                                                            reinterpret_cast<double2*>(tab));
    return launch_status("twiddle_table_kernel");
}

}  // namespace adrt
