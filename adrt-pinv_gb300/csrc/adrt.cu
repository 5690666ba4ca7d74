// Spatial ADRT levels in the reference's layout (adrtcore.py:29-137). Level m maps data on E^n_{m-1}
// (stored (N + 2^(m-1) - 1) x N, row = h + 2^(m-1) - 1) to E^n_m ((N + 2^m - 1) x N):
//   g(h, l*2w + 2t + b) = f(h, l*2w + t) [h >= -t] + f(h + t + b, l*2w + w + t) [h + t + b in [-t, N)],  w = 2^(m-1).
// Forward: one pass per level over all images and quadrants, the quadrant permutation T_q folded into level 1.
// Adjoint: the scatter-add of S_m^T is evaluated as a gather (two terms per output), and the last level also applies
// T_q^T and sums the four quadrants. Additions only, so integer dtypes are exact.
#include "common.cuh"
#include "launch.h"

namespace adrt {

static int grid_of(size_t total) {
    size_t g = (total + 255) / 256;
    if (g > 65535u * 16) g = 65535u * 16;
    return (int)(g ? g : 1);
}

// (T_q x)(i, j) (adrtcore.py:29-39)
template <typename T> __device__ __forceinline__ T tq_read(const T* x, int N, int q, int i, int j) {
    switch (q) {
        case 0: return x[(size_t)j * N + (N - 1 - i)];
        case 1: return x[(size_t)(N - 1 - i) * N + j];
        case 2: return x[(size_t)i * N + j];
        default: return x[(size_t)(N - 1 - j) * N + (N - 1 - i)];
    }
}

// one forward level for every (image, quadrant); level 1 reads T_q x, later levels read src; slot stride S elements.
// active (nullable): images with active[img] == 0 are skipped (their output is left as it was)
template <typename T>
__global__ void adrt_fwd_level(int n, int m, int nimg, const T* __restrict__ src, T* __restrict__ dst, size_t S,
                               const int* __restrict__ active) {
    const int N = 1 << n, w = 1 << (m - 1);
    const int Hout = N + 2 * w - 1;
    const size_t per = (size_t)Hout * N;
    const size_t total = per * 4 * nimg;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const size_t slot = e / per;
        if (active && !active[slot >> 2]) continue;
        const size_t rem = e - slot * per;
        const int row = (int)(rem >> n), s = (int)(rem & (N - 1));
        const int h = row - (2 * w - 1);
        const int l = s / (2 * w), rr = s - l * 2 * w, t = rr >> 1, b = rr & 1;
        const int c0 = l * 2 * w + t, c1 = c0 + w;
        T acc = 0;
        if (m == 1) {
            const int q = (int)(slot & 3);
            const T* x = src + (slot >> 2) * (size_t)N * N;
            if (h >= 0 && h < N) acc += tq_read(x, N, q, h, c0);
            const int h1 = h + b;
            if (h1 >= 0 && h1 < N) acc += tq_read(x, N, q, h1, c1);
        } else {
            const T* f = src + slot * S;
            const int off = w - 1;
            if (h >= -t && h < N) acc += f[(size_t)(h + off) * N + c0];
            const int h1 = h + t + b;
            if (h1 >= -t && h1 < N) acc += f[(size_t)(h1 + off) * N + c1];
        }
        dst[slot * S + rem] = acc;
    }
}

// adjoint value of level m at input position (h, col) from level-m data g (rows h_out + 2w - 1)
template <typename T> __device__ __forceinline__ T adj_at(const T* g, int N, int m, int h, int col) {
    const int w = 1 << (m - 1);
    const int l = col / (2 * w), r = col - l * 2 * w, c = r / w, t = r - c * w;
    if (h < -t || h >= N) return 0;
    const int base = l * 2 * w + 2 * t, off = 2 * w - 1;
    if (c == 0) return g[(size_t)(h + off) * N + base] + g[(size_t)(h + off) * N + base + 1];
    return g[(size_t)(h - t + off) * N + base] + g[(size_t)(h - t - 1 + off) * N + base + 1];
}

template <typename T>
__global__ void adrt_adj_level(int n, int m, int nimg, const T* __restrict__ src, T* __restrict__ dst, size_t S,
                               const int* __restrict__ active) {
    const int N = 1 << n, w = 1 << (m - 1);
    const int Hin = N + w - 1;
    const size_t per = (size_t)Hin * N;
    const size_t total = per * 4 * nimg;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const size_t slot = e / per;
        if (active && !active[slot >> 2]) continue;
        const size_t rem = e - slot * per;
        const int row = (int)(rem >> n), col = (int)(rem & (N - 1));
        dst[slot * S + rem] = adj_at(src + slot * S, N, m, row - (w - 1), col);
    }
}

// ------------------------------------------------------------------ tiled level passes (N >= 32, level m >= 2)
// The per-element kernels above read the second term f(h + t + b, c1) along a shear: neighbouring output columns
// read different rows, so a warp's loads touch many rows. The tiled passes stage the input rows a tile of 32 output
// columns x ADRT_TR output rows needs in shared memory with row-contiguous (coalesced) loads, then gather from there;
// the arithmetic and the guards are those of adrt_fwd_level / adj_at.
constexpr int ADRT_TR = 32;  // output rows per tile

template <typename T>
__global__ void __launch_bounds__(256) adrt_fwd_level_tiled(int n, int m, const T* __restrict__ src,
                                                            T* __restrict__ dst, size_t S,
                                                            const int* __restrict__ active) {
    const int N = 1 << n, w = 1 << (m - 1);
    const int Hout = N + 2 * w - 1, off = w - 1;
    const int s0 = blockIdx.x * 32, row0 = blockIdx.y * ADRT_TR;
    const size_t slot = blockIdx.z;
    if (active && !active[slot >> 2]) return;
    const T* f = src + slot * S;
    T* g = dst + slot * S;
    const int h0 = row0 - (2 * w - 1);  // h of the tile's first output row
    __shared__ T tA[ADRT_TR + 16][33];
    __shared__ T tB[ADRT_TR + 16][17];
    const int lane = threadIdx.x & 31, grp = threadIdx.x >> 5;
    auto ld = [&](int h, int c) -> T { return (h >= -(w - 1) && h < N) ? f[(size_t)(h + off) * N + c] : (T)0; };
    const bool small = 2 * w <= 32;
    int cA = s0, cB = 0, hB = h0, t0 = 0;
    if (small) {
        // the 32 output columns read input columns of the same window, rows h0 .. h0 + TR + w - 1
        for (int e = threadIdx.x; e < (ADRT_TR + w) * 32; e += 256) {
            const int r = e >> 5, c = e & 31;
            tA[r][c] = ld(h0 + r, s0 + c);
        }
    } else {
        const int l = s0 / (2 * w);
        t0 = (s0 - l * 2 * w) >> 1;
        cA = l * 2 * w + t0;  // c0 columns cA .. cA + 15
        cB = cA + w;          // c1 columns cB .. cB + 15
        hB = h0 + t0;         // c1 rows h + t + b start at h0 + t0
        for (int e = threadIdx.x; e < ADRT_TR * 16; e += 256) {
            const int r = e >> 4, c = e & 15;
            tA[r][c] = ld(h0 + r, cA + c);
        }
        for (int e = threadIdx.x; e < (ADRT_TR + 16) * 16; e += 256) {
            const int r = e >> 4, c = e & 15;
            tB[r][c] = ld(hB + r, cB + c);
        }
    }
    __syncthreads();
    const int s = s0 + lane;
    const int l = s / (2 * w), rr = s - l * 2 * w, t = rr >> 1, b = rr & 1;
    const int c0 = l * 2 * w + t, c1 = c0 + w;
    for (int i = grp; i < ADRT_TR; i += 8) {
        const int row = row0 + i;
        if (row >= Hout) break;
        const int h = h0 + i;
        T acc = 0;
        if (h >= -t && h < N) acc += small ? tA[i][c0 - s0] : tA[i][c0 - cA];
        const int h1 = h + t + b;
        if (h1 >= -t && h1 < N) acc += small ? tA[h1 - h0][c1 - s0] : tB[h1 - hB][c1 - cB];
        g[(size_t)row * N + s] = acc;
    }
}

template <typename T>
__global__ void __launch_bounds__(256) adrt_adj_level_tiled(int n, int m, const T* __restrict__ src,
                                                            T* __restrict__ dst, size_t S,
                                                            const int* __restrict__ active) {
    const int N = 1 << n, w = 1 << (m - 1);
    const int Hin = N + w - 1, off = 2 * w - 1;  // output rows (level m-1 layout); input row offset (level m)
    const int col0 = blockIdx.x * 32, row0 = blockIdx.y * ADRT_TR;
    const size_t slot = blockIdx.z;
    if (active && !active[slot >> 2]) return;
    const T* g = src + slot * S;
    T* o = dst + slot * S;
    const int h0 = row0 - (w - 1);
    __shared__ T tg[ADRT_TR + 32][65];
    const int lane = threadIdx.x & 31, grp = threadIdx.x >> 5;
    const int Hg = N + 2 * w - 1;
    auto ld = [&](int h, int c) -> T {
        const int r = h + off;
        return (r >= 0 && r < Hg) ? g[(size_t)r * N + c] : (T)0;
    };
    const bool small = 2 * w <= 32;
    const int l = col0 / (2 * w), r0 = col0 - l * 2 * w, half = small ? 0 : r0 / w;
    const int t0 = small ? 0 : r0 - half * w;
    int gc0, gh0, ncols;
    if (small) {
        gc0 = col0;      // the window's own columns
        gh0 = h0 - w;    // rows h - t - 1 >= h0 - w
        ncols = 32;
    } else {
        gc0 = l * 2 * w + 2 * t0;                // base columns of t0 .. t0 + 31, and base + 1
        gh0 = half == 0 ? h0 : h0 - t0 - 32;     // second half reads rows h - t, h - t - 1
        ncols = 64;
    }
    const int nrows = small ? ADRT_TR + w : (half == 0 ? ADRT_TR : ADRT_TR + 32);
    for (int e = threadIdx.x; e < nrows * ncols; e += 256) {
        const int r = e / ncols, c = e - r * ncols;
        tg[r][c] = ld(gh0 + r, gc0 + c);
    }
    __syncthreads();
    const int col = col0 + lane;
    const int cl = col / (2 * w), r = col - cl * 2 * w, c = r / w, t = r - c * w;
    const int base = cl * 2 * w + 2 * t - gc0;
    for (int i = grp; i < ADRT_TR; i += 8) {
        const int row = row0 + i;
        if (row >= Hin) break;
        const int h = h0 + i;
        T v = 0;
        if (h >= -t && h < N) {
            if (c == 0) v = tg[h - gh0][base] + tg[h - gh0][base + 1];
            else v = tg[h - t - gh0][base] + tg[h - t - 1 - gh0][base + 1];
        }
        o[(size_t)row * N + col] = v;
    }
}

// ------------------------------------------------------------------ the first four levels in shared memory
// Levels 1..4 only combine columns within blocks of 16 (level m pairs the halves of blocks of 2^m columns), so a CTA
// can take one 16-column block of one quadrant through all four levels in shared memory: the forward pass reads the
// T_q strip once and writes level 4; the adjoint reads level 4 and writes level 1 (the quadrant sum stays with
// adrt_adj_final). Rows in shared memory have a stride of 17 elements (conflict-free column walks).
constexpr int F4_SP = 17;

template <typename T> static size_t f4_smem(int N) { return 2 * (size_t)(N + 15) * F4_SP * sizeof(T); }

template <typename T>
__global__ void __launch_bounds__(256) adrt_fwd_levels14(int n, const T* __restrict__ x, T* __restrict__ dst, size_t S,
                                                         const int* __restrict__ active) {
    const int N = 1 << n;
    const int c0 = blockIdx.x * 16, q = blockIdx.y, img = blockIdx.z;
    if (active && !active[img]) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* a = reinterpret_cast<T*>(smem_raw);
    T* b = a + (size_t)(N + 15) * F4_SP;
    const T* xi = x + (size_t)img * N * N;
    // level 0: the T_q strip (rows h = 0..N-1); quadrants 0 and 3 read image rows, so there consecutive threads take
    // consecutive h, the others consecutive columns
    for (int e = threadIdx.x; e < N * 16; e += 256) {
        int h, c;
        if (q == 1 || q == 2) {
            h = e >> 4;
            c = e & 15;
        } else {
            c = e >> n;
            h = e & (N - 1);
        }
        a[h * F4_SP + c] = tq_read(xi, N, q, h, c0 + c);
    }
    __syncthreads();
    int off = 0;  // row offset of the level held in a (level m-1 data: 2^(m-1) - 1)
    for (int m = 1; m <= 4; ++m) {
        const int w = 1 << (m - 1), Hout = N + 2 * w - 1;
        for (int e = threadIdx.x; e < Hout * 16; e += 256) {
            const int row = e >> 4, cc = e & 15;
            const int h = row - (2 * w - 1);
            const int l = cc / (2 * w), rr = cc - l * 2 * w, t = rr >> 1, bb = rr & 1;
            const int ca = l * 2 * w + t, cb = ca + w;
            T acc = 0;
            if (h >= -t && h < N) acc += a[(h + off) * F4_SP + ca];
            const int h1 = h + t + bb;
            if (h1 >= -t && h1 < N) acc += a[(h1 + off) * F4_SP + cb];
            b[row * F4_SP + cc] = acc;
        }
        __syncthreads();
        T* tmp = a;
        a = b;
        b = tmp;
        off = 2 * w - 1;
    }
    T* g = dst + ((size_t)img * 4 + q) * S;
    for (int e = threadIdx.x; e < (N + 15) * 16; e += 256) {
        const int row = e >> 4, cc = e & 15;
        g[(size_t)row * N + c0 + cc] = a[row * F4_SP + cc];
    }
}

template <typename T>
__global__ void __launch_bounds__(256) adrt_adj_levels42(int n, const T* __restrict__ src, T* __restrict__ dst,
                                                         size_t S, const int* __restrict__ active) {
    const int N = 1 << n;
    const int c0 = blockIdx.x * 16;
    const size_t slot = blockIdx.y;
    if (active && !active[slot >> 2]) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* a = reinterpret_cast<T*>(smem_raw);
    T* b = a + (size_t)(N + 15) * F4_SP;
    const T* g = src + slot * S;
    for (int e = threadIdx.x; e < (N + 15) * 16; e += 256) {
        const int row = e >> 4, cc = e & 15;
        a[row * F4_SP + cc] = g[(size_t)row * N + c0 + cc];
    }
    __syncthreads();
    for (int m = 4; m >= 2; --m) {
        // level-m data in a (rows h + 2w - 1) -> level m-1 data in b (rows h + w - 1), as adj_at
        const int w = 1 << (m - 1), Hin = N + w - 1, goff = 2 * w - 1;
        for (int e = threadIdx.x; e < Hin * 16; e += 256) {
            const int row = e >> 4, col = e & 15;
            const int h = row - (w - 1);
            const int l = col / (2 * w), r = col - l * 2 * w, c = r / w, t = r - c * w;
            T v = 0;
            if (h >= -t && h < N) {
                const int base = l * 2 * w + 2 * t;
                if (c == 0) v = a[(h + goff) * F4_SP + base] + a[(h + goff) * F4_SP + base + 1];
                else v = a[(h - t + goff) * F4_SP + base] + a[(h - t - 1 + goff) * F4_SP + base + 1];
            }
            b[row * F4_SP + col] = v;
        }
        __syncthreads();
        T* tmp = a;
        a = b;
        b = tmp;
    }
    T* o = dst + slot * S;
    for (int e = threadIdx.x; e < (N + 1) * 16; e += 256) {  // level 1: N + 1 rows
        const int row = e >> 4, cc = e & 15;
        o[(size_t)row * N + c0 + cc] = a[row * F4_SP + cc];
    }
}

// level-1 adjoint of the four quadrants, T_q^T and the quadrant sum (adrtcore.py:131-137)
template <typename T>
__global__ void adrt_adj_final(int n, int nimg, const T* __restrict__ src, T* __restrict__ x, size_t S,
                               const int* __restrict__ active) {
    const int N = 1 << n;
    const size_t per = (size_t)N * N;
    const size_t total = per * nimg;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const size_t img = e / per;
        if (active && !active[img]) continue;
        const size_t rem = e - img * per;
        const int a = (int)(rem >> n), b = (int)(rem & (N - 1));
        const T* g = src + img * 4 * S;
        // x[a, b] = sum_q (T_q^T f_q)[a, b]: q0 f(N-1-b, a); q1 f(N-1-a, b); q2 f(a, b); q3 f(N-1-b, N-1-a)
        T acc = adj_at(g + 0 * S, N, 1, N - 1 - b, a);
        acc += adj_at(g + 1 * S, N, 1, N - 1 - a, b);
        acc += adj_at(g + 2 * S, N, 1, a, b);
        acc += adj_at(g + 3 * S, N, 1, N - 1 - b, N - 1 - a);
        x[e] = acc;
    }
}

template <typename T>
static int fwd_t(int n, int nimg, const void* x, void* b, void* scratch, const int* active, cudaStream_t st) {
    const int N = 1 << n;
    const size_t S = (size_t)(2 * N - 1) * N;
    T* bufs[2] = {reinterpret_cast<T*>(scratch), reinterpret_cast<T*>(scratch) + S * 4 * nimg};
    const T* src = reinterpret_cast<const T*>(x);
    int m0 = 1;
    if (n >= 4 && f4_smem<T>(N) <= 200 * 1024 && nimg <= 65535) {
        // levels 1..4 in one pass per 16-column block and quadrant
        T* dst = (n == 4) ? reinterpret_cast<T*>(b) : bufs[0];
        const size_t smem = f4_smem<T>(N);
        if (int rc = ensure_smem((const void*)adrt_fwd_levels14<T>, smem)) return rc;
        adrt_fwd_levels14<T><<<dim3(N / 16, 4, nimg), 256, smem, st>>>(n, src, dst, S, active);
        if (int rc = launch_status("adrt_fwd_levels14")) return rc;
        src = dst;
        m0 = 5;
    }
    for (int m = m0; m <= n; ++m) {
        T* dst = (m == n) ? reinterpret_cast<T*>(b) : bufs[m & 1];
        const int Hout = N + (1 << m) - 1;
        const size_t total = (size_t)Hout * N * 4 * nimg;
        if (m >= 2 && N >= 32 && 4L * nimg <= 65535) {
            dim3 grid(N / 32, (Hout + ADRT_TR - 1) / ADRT_TR, 4 * nimg);
            adrt_fwd_level_tiled<T><<<grid, 256, 0, st>>>(n, m, src, dst, S, active);
        } else {
            adrt_fwd_level<T><<<grid_of(total), 256, 0, st>>>(n, m, nimg, src, dst, S, active);
        }
        int rc = launch_status("adrt_fwd_level");
        if (rc) return rc;
        src = dst;
    }
    return ADRT_OK;
}

template <typename T>
static int adj_t(int n, int nimg, const void* b, void* x, void* scratch, const int* active, cudaStream_t st) {
    const int N = 1 << n;
    const size_t S = (size_t)(2 * N - 1) * N;
    T* bufs[2] = {reinterpret_cast<T*>(scratch), reinterpret_cast<T*>(scratch) + S * 4 * nimg};
    const T* src = reinterpret_cast<const T*>(b);
    const bool fuse = n >= 4 && f4_smem<T>(N) <= 200 * 1024 && 4L * nimg <= 65535;
    for (int m = n; m >= (fuse ? 5 : 2); --m) {
        T* dst = bufs[m & 1];
        const int Hin = N + (1 << (m - 1)) - 1;
        const size_t total = (size_t)Hin * N * 4 * nimg;
        if (N >= 32 && 4L * nimg <= 65535) {
            dim3 grid(N / 32, (Hin + ADRT_TR - 1) / ADRT_TR, 4 * nimg);
            adrt_adj_level_tiled<T><<<grid, 256, 0, st>>>(n, m, src, dst, S, active);
        } else {
            adrt_adj_level<T><<<grid_of(total), 256, 0, st>>>(n, m, nimg, src, dst, S, active);
        }
        int rc = launch_status("adrt_adj_level");
        if (rc) return rc;
        src = dst;
    }
    if (fuse) {
        // levels 4..2 in one pass per 16-column block and quadrant: level 4 in, level 1 out
        T* dst = (src == bufs[0]) ? bufs[1] : bufs[0];
        const size_t smem = f4_smem<T>(N);
        if (int rc = ensure_smem((const void*)adrt_adj_levels42<T>, smem)) return rc;
        adrt_adj_levels42<T><<<dim3(N / 16, 4 * nimg), 256, smem, st>>>(n, src, dst, S, active);
        if (int rc = launch_status("adrt_adj_levels42")) return rc;
        src = dst;
    }
    adrt_adj_final<T><<<grid_of((size_t)N * N * nimg), 256, 0, st>>>(n, nimg, src, reinterpret_cast<T*>(x), S, active);
    return launch_status("adrt_adj_final");
}

int adrt_fwd(int dtype, int n, int nimg, const void* x, void* b, void* scratch, cudaStream_t st, const int* active) {
    if (n < 1 || n > 12 || nimg < 0) { set_error("adrt_forward: bad n=%d nimg=%d", n, nimg); return ADRT_EINVAL; }
    if (!nimg) return ADRT_OK;
    if (!x || !b || (!scratch && n > 1)) { set_error("adrt_forward: null pointer"); return ADRT_EINVAL; }
    switch (dtype) {
        case ADRT_F32: return fwd_t<float>(n, nimg, x, b, scratch, active, st);
        case ADRT_F64: return fwd_t<double>(n, nimg, x, b, scratch, active, st);
        case ADRT_I32: return fwd_t<int32_t>(n, nimg, x, b, scratch, active, st);
        case ADRT_I64: return fwd_t<long long>(n, nimg, x, b, scratch, active, st);
    }
    set_error("adrt_forward: bad dtype %d", dtype);
    return ADRT_EINVAL;
}

int adrt_adj(int dtype, int n, int nimg, const void* b, void* x, void* scratch, cudaStream_t st, const int* active) {
    if (n < 1 || n > 12 || nimg < 0) { set_error("adrt_transpose: bad n=%d nimg=%d", n, nimg); return ADRT_EINVAL; }
    if (!nimg) return ADRT_OK;
    if (!x || !b || (!scratch && n > 1)) { set_error("adrt_transpose: null pointer"); return ADRT_EINVAL; }
    switch (dtype) {
        case ADRT_F32: return adj_t<float>(n, nimg, b, x, scratch, active, st);
        case ADRT_F64: return adj_t<double>(n, nimg, b, x, scratch, active, st);
        case ADRT_I32: return adj_t<int32_t>(n, nimg, b, x, scratch, active, st);
        case ADRT_I64: return adj_t<long long>(n, nimg, b, x, scratch, active, st);
    }
    set_error("adrt_transpose: bad dtype %d", dtype);
    return ADRT_EINVAL;
}

}  // namespace adrt
