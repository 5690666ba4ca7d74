// Row engine kernels and dispatch; the register layouts, lane programs and the per-item body of the compile-time
// programs are in rows_core.cuh.
#include <atomic>
#include <cstdio>

#include "rows_core.cuh"

namespace adrt {

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

template <typename real, int n, int THREADS, int PROG>
__global__ void __launch_bounds__(THREADS, 1)
    rows_prog_kernel(const adrt_row_job J, const TwSrc<real> tw, const int total) {
    using C = cplx<real>;
    using F = FastCfg<n>;
    using Ln = Lanes<C, n>;
    constexpr int T = F::T;
    constexpr int GPW = 32 / T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31;
    const int giw = T >= 32 ? 0 : lane / T;
    const int u = threadIdx.x & (T - 1);
    C* buf = reinterpret_cast<C*>(smem_raw) + (threadIdx.x / T) * F::GS;
    C* zt = buf + F::BUF + F::N;
    int* slot = reinterpret_cast<int*>(zt + ((F::ZT + 1) & ~1));  // the group's work item (WPG > 1)
    const unsigned gm = (T >= 32) ? 0xffffffffu : (((1u << T) - 1u) << (giw * T));

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
        if (item < total) prog_item<real, n, PROG>(J, tw, item, buf, u, gm);
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
