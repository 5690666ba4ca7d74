// Offset-axis DFTs with the quadrant packing folded into the loads and stores (reference: fastops._packed,
// fastops.py:209-220; Tq / TqT / iota, fastspec.py:142-174).
//
// One CTA handles a block of C strip columns of one image. The length-L (L = 2N) DFT of each column runs as an
// in-place radix-2 decimation-in-time transform on bit-reversed input: each thread holds 8 points of its column,
// does three stages in registers per pass and exchanges through a padded shared-memory tile between passes.
// Twiddles come from an FP64-accurate table of L roots of unity staged in shared memory.
//
// pack:   strips s_qa + i s_qb of each quadrant pair are gathered (coalesced, through the tile) from the image
//         (Tq of the zero-padded image) or the sinogram (iota), transformed forward, and written as rows of Y.
// unpack: both pairs of a column block are transformed back (1/L), only the first N offsets are kept, and the
//         four quadrant strips are scattered with TqT and cropped into three image-space partial sums:
//         colpart (quadrants II+III: out columns), rowpart0 (quadrant I: out rows), rowpart3 (quadrant IV).
#include <type_traits>

#include "common.cuh"
#include "launch.h"

namespace adrt {

template <int l> struct FftCfg {
    static constexpr int L = 1 << l;
    static constexpr int e = (l >= 3) ? 3 : l;  // log2 of points per thread
    static constexpr int E = 1 << e;
    static constexpr int TPC = L / E;           // threads per column
    static constexpr int NPASS = (l + 2) / 3;
    __host__ __device__ static constexpr int s0(int q) { return 3 * q; }
    __host__ __device__ static constexpr int nb(int q) { return imin(3, l - 3 * q); }
    // physical position of register j in pass q for column-thread t
    __device__ static __forceinline__ int pos(int q, int t, int j) {
        if (l < 3) return j;
        const int b = nb(q), s = s0(q);
        if (b == 3) return (t & ((1 << s) - 1)) | (j << s) | ((t >> s) << (s + 3));
        const int x = 3 - b;
        return (t & ((1 << (s - x)) - 1)) | ((j >> b) << (s - x)) | ((j & ((1 << b) - 1)) << s);
    }
};

template <typename real> struct FftMax;
template <> struct FftMax<float> { static constexpr int C = 16; };
template <> struct FftMax<double> { static constexpr int C = 8; };

// columns per CTA: the largest power of two <= Cmax, <= 1024 / threads-per-column and <= N whose unpack tiles
// (roots L + exchange tile L x CP + pair-(0,1) result N x CP, CP = C + 1 padding for C > 1) fit in 227 KB
constexpr int kSmemBudget = 227 * 1024;
__host__ __device__ constexpr int fft_pad(int c) { return c > 1 ? c + 1 : 1; }
template <int l> __host__ __device__ constexpr int fft_cols(int Cmax, int elem_bytes) {
    int c = imax(1, imin(imin(Cmax, 1024 / FftCfg<l>::TPC), (1 << l) / 2));
    while (c > 1 && ((1 << l) + ((1 << l) + (1 << (l - 1))) * fft_pad(c)) * elem_bytes > kSmemBudget) c >>= 1;
    return c;
}

// all passes of the in-place DIT transform on the registers x[] of (column c, column-thread t)
template <typename real, int l, bool INV>
__device__ __forceinline__ void dit_passes(cplx<real> (&x)[FftCfg<l>::E], const cplx<real>* __restrict__ roots,
                                           cplx<real>* tile, int CP, int c, int t) {
    using F = FftCfg<l>;
    using C = cplx<real>;
#pragma unroll
    for (int q = 0; q < F::NPASS; ++q) {
        if (q > 0) {
            __syncthreads();
#pragma unroll
            for (int j = 0; j < F::E; ++j) tile[F::pos(q - 1, t, j) * CP + c] = x[j];
            __syncthreads();
#pragma unroll
            for (int j = 0; j < F::E; ++j) x[j] = tile[F::pos(q, t, j) * CP + c];
        }
        const int s = F::s0(q), b = F::nb(q);
#pragma unroll
        for (int rb = 0; rb < b; ++rb) {
            const int sg = s + rb;  // stage bit
#pragma unroll
            for (int j = 0; j < F::E; ++j) {
                if (j & (1 << rb)) continue;
                const int p = F::pos(q, t, j);
                C w = roots[(p & ((1 << sg) - 1)) * (F::L >> (sg + 1))];
                if (!INV) w.y = -w.y;
                const C u = x[j];
                const C v = cmul(w, x[j | (1 << rb)]);
                x[j] = cadd(u, v);
                x[j | (1 << rb)] = csub(u, v);
            }
        }
    }
}

// threads of a CTA and the CTAs per SM the register budget is sized for (the whole SM's 2048 threads in FP32)
template <typename real, int l, int CB> struct FftLaunch {
    static constexpr int threads = CB * FftCfg<l>::TPC;
    static constexpr int pack_min = sizeof(real) == 4 ? imax(1, 2048 / threads) : imax(1, 1024 / threads);
    static constexpr int unpack_min = imax(1, 1024 / threads);
};

template <typename real, int l, int CB, typename SRC>
__global__ void __launch_bounds__(FftLaunch<real, l, CB>::threads, FftLaunch<real, l, CB>::pack_min)
    pack_fft_kernel(int nimg, int src_kind, const SRC* __restrict__ src, long long src_stride, cplx<real>* __restrict__ Y,
                    const cplx<real>* __restrict__ roots_g) {
    using F = FftCfg<l>;
    using C = cplx<real>;
    constexpr int L = F::L, N = L / 2;
    constexpr int CP = fft_pad(CB);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* roots = reinterpret_cast<C*>(smem_raw);
    C* tile = roots + L;
    const int c0 = blockIdx.x * CB;
    const int pair = blockIdx.y;
    const int img = blockIdx.z;
    constexpr int nthr = CB * F::TPC;  // L * CB elements per gather = E per thread
    for (int i = threadIdx.x; i < L; i += nthr) roots[i] = roots_g[i];

    // ---- gather the packed strips of columns c0..c0+CB-1 into tile[i][c]; every thread issues its E loads before
    // its shared-memory stores (E independent loads in flight)
    if (src_kind == 0 && CB % 2 == 0) {
        // two neighbouring elements per load: column pairs of the column reads, offset pairs of the row reads
        using S2 = typename std::conditional<sizeof(SRC) == 8, double2, float2>::type;
        constexpr int HC = CB / 2, HE = F::E / 2, HL = L / 2;
        const size_t ib = (size_t)img * src_stride;
        // column reads: pair 0 imag = x[N-1-i, c] (quadrant II), pair 1 real = x[i, c] (quadrant III)
        real va[HE], vb[HE];
#pragma unroll
        for (int k = 0; k < HE; ++k) {
            const int e = threadIdx.x + k * nthr;
            const int c = 2 * (e % HC), i = e / HC;
            va[k] = 0;
            vb[k] = 0;
            if (i < N) {
                const S2 w = *reinterpret_cast<const S2*>(src + ib + (size_t)(pair == 0 ? N - 1 - i : i) * N + c0 + c);
                va[k] = (real)w.x;
                vb[k] = (real)w.y;
            }
        }
#pragma unroll
        for (int k = 0; k < HE; ++k) {
            const int e = threadIdx.x + k * nthr;
            const int c = 2 * (e % HC), i = e / HC;
            if (pair == 0) {
                tile[i * CP + c].y = va[k];
                tile[i * CP + c + 1].y = vb[k];
            } else {
                tile[i * CP + c].x = va[k];
                tile[i * CP + c + 1].x = vb[k];
            }
        }
        // row reads: pair 0 real = x[c, N-1-i] (quadrant I), pair 1 imag = x[N-1-c, N-1-i] (quadrant IV); the pair
        // (i, i+1) is the element pair (N-2-i, N-1-i) of the image row
#pragma unroll
        for (int k = 0; k < HE; ++k) {
            const int e = threadIdx.x + k * nthr;
            const int i = 2 * (e % HL), c = e / HL;
            va[k] = 0;
            vb[k] = 0;
            if (i < N) {
                const int rowx = (pair == 0) ? (c0 + c) : (N - 1 - c0 - c);
                const S2 w = *reinterpret_cast<const S2*>(src + ib + (size_t)rowx * N + (N - 2 - i));
                va[k] = (real)w.y;  // offset i
                vb[k] = (real)w.x;  // offset i + 1
            }
        }
#pragma unroll
        for (int k = 0; k < HE; ++k) {
            const int e = threadIdx.x + k * nthr;
            const int i = 2 * (e % HL), c = e / HL;
            if (pair == 0) {
                tile[i * CP + c].x = va[k];
                tile[(i + 1) * CP + c].x = vb[k];
            } else {
                tile[i * CP + c].y = va[k];
                tile[(i + 1) * CP + c].y = vb[k];
            }
        }
    } else if (src_kind == 0) {
        const size_t ib = (size_t)img * src_stride;
        // column reads: pair 0 imag = x[N-1-i, c] (quadrant II), pair 1 real = x[i, c] (quadrant III)
        real v[F::E];
#pragma unroll
        for (int k = 0; k < F::E; ++k) {
            const int e = threadIdx.x + k * nthr;
            const int c = e % CB, i = e / CB;
            v[k] = 0;
            if (i < N) v[k] = (real)src[ib + (size_t)(pair == 0 ? N - 1 - i : i) * N + c0 + c];
        }
#pragma unroll
        for (int k = 0; k < F::E; ++k) {
            const int e = threadIdx.x + k * nthr;
            const int c = e % CB, i = e / CB;
            if (pair == 0) tile[i * CP + c].y = v[k]; else tile[i * CP + c].x = v[k];
        }
        // row reads: pair 0 real = x[c, N-1-i] (quadrant I), pair 1 imag = x[N-1-c, N-1-i] (quadrant IV)
#pragma unroll
        for (int k = 0; k < F::E; ++k) {
            const int e = threadIdx.x + k * nthr;
            const int i = e % L, c = e / L;
            v[k] = 0;
            if (i < N) {
                const int rowx = (pair == 0) ? (c0 + c) : (N - 1 - c0 - c);
                v[k] = (real)src[ib + (size_t)rowx * N + (N - 1 - i)];
            }
        }
#pragma unroll
        for (int k = 0; k < F::E; ++k) {
            const int e = threadIdx.x + k * nthr;
            const int i = e % L, c = e / L;
            if (pair == 0) tile[i * CP + c].x = v[k]; else tile[i * CP + c].y = v[k];
        }
    } else {
        // iota of the sinogram quadrants qa = 2*pair, qb = 2*pair+1: S[i] = b[i+N-1] (i < N), 0 (i = N), b[i-N-1]
        const size_t H = 2 * (size_t)N - 1;
        const size_t ba = ((size_t)img * 4 + 2 * pair) * H * N, bb = ba + H * N;
        real va[F::E], vb[F::E];
#pragma unroll
        for (int k = 0; k < F::E; ++k) {
            const int e = threadIdx.x + k * nthr;
            const int c = e % CB, i = e / CB;
            va[k] = 0;
            vb[k] = 0;
            if (i != N) {
                const size_t h = (i < N) ? (size_t)(i + N - 1) : (size_t)(i - N - 1);
                va[k] = (real)src[ba + h * N + c0 + c];
                vb[k] = (real)src[bb + h * N + c0 + c];
            }
        }
#pragma unroll
        for (int k = 0; k < F::E; ++k) {
            const int e = threadIdx.x + k * nthr;
            const int c = e % CB, i = e / CB;
            tile[i * CP + c] = mk<real>(va[k], vb[k]);
        }
    }
    __syncthreads();

    const int c = threadIdx.x % CB, t = threadIdx.x / CB;
    C x[F::E];
#pragma unroll
    for (int j = 0; j < F::E; ++j) x[j] = tile[(__brev((unsigned)F::pos(0, t, j)) >> (32 - l)) * CP + c];
    dit_passes<real, l, false>(x, roots, tile, CP, c, t);
    C* out = Y + ((size_t)img * 2 * L + (size_t)pair * L) * N + c0 + c;
#pragma unroll
    for (int j = 0; j < F::E; ++j) out[(size_t)F::pos(F::NPASS - 1, t, j) * N] = x[j];
}

template <typename real, int l, int CB>
__global__ void __launch_bounds__(FftLaunch<real, l, CB>::threads, FftLaunch<real, l, CB>::unpack_min)
    ifft_unpack_kernel(int nimg, const cplx<real>* __restrict__ Z, real* __restrict__ colpart, real* __restrict__ row0,
                       real* __restrict__ row3, const cplx<real>* __restrict__ roots_g) {
    using F = FftCfg<l>;
    using C = cplx<real>;
    constexpr int L = F::L, N = L / 2;
    constexpr int CP = fft_pad(CB);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* roots = reinterpret_cast<C*>(smem_raw);
    C* tile = roots + L;          // L x CP exchange tile
    C* s01 = tile + L * CP;       // N x CP: pair (0,1) result, re = quadrant I strip, im = quadrant II strip
    const int c0 = blockIdx.x * CB;
    const int img = blockIdx.y;
    const int nthr = CB * F::TPC;
    for (int i = threadIdx.x; i < L; i += nthr) roots[i] = roots_g[i];
    __syncthreads();
    const int c = threadIdx.x % CB, t = threadIdx.x / CB;
    const real scale = (real)1 / (real)L;
#pragma unroll 1
    for (int pair = 0; pair < 2; ++pair) {
        const C* in = Z + ((size_t)img * 2 * L + (size_t)pair * L) * N + c0 + c;
        C x[F::E];
#pragma unroll
        for (int j = 0; j < F::E; ++j) x[j] = in[(size_t)(__brev((unsigned)F::pos(0, t, j)) >> (32 - l)) * N];
        dit_passes<real, l, true>(x, roots, tile, CP, c, t);
        C* dst = pair == 0 ? s01 : tile;  // pair (2,3) lands in the first N rows of the exchange tile
        __syncthreads();
#pragma unroll
        for (int j = 0; j < F::E; ++j) {
            const int p = F::pos(F::NPASS - 1, t, j);
            if (p < N) dst[p * CP + c] = cscale(scale, x[j]);
        }
    }
    __syncthreads();
    // colpart[i][c0+c] = S_III[i][c] + S_II[N-1-i][c]
    const size_t ib = (size_t)img * N * N;
    for (int e = threadIdx.x; e < N * CB; e += nthr) {
        const int cc = e % CB, i = e / CB;
        colpart[ib + (size_t)i * N + c0 + cc] = tile[i * CP + cc].x + s01[(N - 1 - i) * CP + cc].y;
    }
    // rowpart0[c0+c][N-1-r] = S_I[r][c] ; rowpart3[N-1-c0-c][N-1-r] = S_IV[r][c]
    for (int e = threadIdx.x; e < N * CB; e += nthr) {
        const int r = e % N, cc = e / N;
        row0[ib + (size_t)(c0 + cc) * N + (N - 1 - r)] = s01[r * CP + cc].x;
        row3[ib + (size_t)(N - 1 - c0 - cc) * N + (N - 1 - r)] = tile[r * CP + cc].y;
    }
}

template <typename real, int l, int CB> static size_t pack_smem() {
    return ((size_t)(1 << l) + (size_t)(1 << l) * fft_pad(CB)) * sizeof(cplx<real>);
}
template <typename real, int l, int CB> static size_t unpack_smem() {
    return ((size_t)(1 << l) + ((size_t)(1 << l) + (size_t)(1 << (l - 1))) * fft_pad(CB)) * sizeof(cplx<real>);
}

// columns per CTA: the default (as many as fit, up to 16 FP32 / 8 FP64) or a quarter of it (narrower CTAs, more of
// them per SM, so the load, transform and store phases of different CTAs overlap); cols = 0 picks the default
template <typename real, int l> constexpr int cols_wide() { return fft_cols<l>(FftMax<real>::C, sizeof(cplx<real>)); }
template <typename real, int l> constexpr int cols_narrow() { return imax(1, cols_wide<real, l>() / 4); }

template <typename real, int l, int CB, typename SRC>
static int launch_pack_cb(int nimg, int src_kind, const void* src, long long src_stride, void* Y, const void* roots,
                          cudaStream_t st) {
    constexpr int N = 1 << (l - 1);
    const size_t smem = pack_smem<real, l, CB>();
    auto kern = pack_fft_kernel<real, l, CB, SRC>;
    if (int rc = ensure_smem((const void*)kern, smem)) return rc;
    dim3 grid(N / CB, 2, nimg);
    kern<<<grid, CB * FftCfg<l>::TPC, smem, st>>>(nimg, src_kind, reinterpret_cast<const SRC*>(src),
                                                   src_stride ? src_stride : (long long)N * N,
                                                   reinterpret_cast<cplx<real>*>(Y),
                                                   reinterpret_cast<const cplx<real>*>(roots));
    return launch_status("pack_fft_kernel");
}

template <typename real, int l, typename SRC>
static int launch_pack_src(int nimg, int src_kind, const void* src, long long src_stride, void* Y, const void* roots,
                           int cols, cudaStream_t st) {
    constexpr int W = cols_wide<real, l>(), NW = cols_narrow<real, l>();
    if (cols == 0 || cols == W) return launch_pack_cb<real, l, W, SRC>(nimg, src_kind, src, src_stride, Y, roots, st);
    if (NW != W && cols == NW) return launch_pack_cb<real, l, NW, SRC>(nimg, src_kind, src, src_stride, Y, roots, st);
    set_error("pack_fft: %d columns per CTA unsupported (%d or %d at n=%d)", cols, W, NW, l - 1);
    return ADRT_EINVAL;
}

template <typename real, int l>
static int launch_pack(int nimg, int src_kind, int src_dtype, const void* src, long long src_stride, void* Y,
                       const void* roots, int cols, cudaStream_t st) {
    if (src_dtype == ADRT_F64)
        return launch_pack_src<real, l, double>(nimg, src_kind, src, src_stride, Y, roots, cols, st);
    return launch_pack_src<real, l, float>(nimg, src_kind, src, src_stride, Y, roots, cols, st);
}

template <typename real, int l, int CB>
static int launch_unpack_cb(int nimg, const void* Z, void* colpart, void* row0, void* row3, const void* roots,
                            cudaStream_t st) {
    constexpr int N = 1 << (l - 1);
    const size_t smem = unpack_smem<real, l, CB>();
    auto kern = ifft_unpack_kernel<real, l, CB>;
    if (int rc = ensure_smem((const void*)kern, smem)) return rc;
    dim3 grid(N / CB, nimg);
    kern<<<grid, CB * FftCfg<l>::TPC, smem, st>>>(nimg, reinterpret_cast<const cplx<real>*>(Z), reinterpret_cast<real*>(colpart),
                                                   reinterpret_cast<real*>(row0), reinterpret_cast<real*>(row3),
                                                   reinterpret_cast<const cplx<real>*>(roots));
    return launch_status("ifft_unpack_kernel");
}

template <typename real, int l>
static int launch_unpack(int nimg, const void* Z, void* colpart, void* row0, void* row3, const void* roots, int cols,
                         cudaStream_t st) {
    constexpr int W = cols_wide<real, l>(), NW = cols_narrow<real, l>();
    if (cols == 0 || cols == W) return launch_unpack_cb<real, l, W>(nimg, Z, colpart, row0, row3, roots, st);
    if (NW != W && cols == NW) return launch_unpack_cb<real, l, NW>(nimg, Z, colpart, row0, row3, roots, st);
    set_error("ifft_unpack: %d columns per CTA unsupported (%d or %d at n=%d)", cols, W, NW, l - 1);
    return ADRT_EINVAL;
}

#define ADRT_FFT_CASES(F, ...)                     \
    switch (n) {                                   \
        case 1: return F<real, 2>(__VA_ARGS__);    \
        case 2: return F<real, 3>(__VA_ARGS__);    \
        case 3: return F<real, 4>(__VA_ARGS__);    \
        case 4: return F<real, 5>(__VA_ARGS__);    \
        case 5: return F<real, 6>(__VA_ARGS__);    \
        case 6: return F<real, 7>(__VA_ARGS__);    \
        case 7: return F<real, 8>(__VA_ARGS__);    \
        case 8: return F<real, 9>(__VA_ARGS__);    \
        case 9: return F<real, 10>(__VA_ARGS__);   \
        case 10: return F<real, 11>(__VA_ARGS__);  \
        case 11: return F<real, 12>(__VA_ARGS__);  \
    }

template <typename real>
static int pack_t(int n, int nimg, int src_kind, int src_dtype, const void* src, long long src_stride, void* Y,
                  const void* roots, int cols, cudaStream_t st) {
    ADRT_FFT_CASES(launch_pack, nimg, src_kind, src_dtype, src, src_stride, Y, roots, cols, st)
    set_error("pack_fft: n=%d unsupported", n);
    return ADRT_EUNSUPPORTED;
}
template <typename real>
static int unpack_t(int n, int nimg, const void* Z, void* colpart, void* row0, void* row3, const void* roots, int cols,
                    cudaStream_t st) {
    ADRT_FFT_CASES(launch_unpack, nimg, Z, colpart, row0, row3, roots, cols, st)
    set_error("ifft_unpack: n=%d unsupported", n);
    return ADRT_EUNSUPPORTED;
}

int pack_fft(int dtype, int n, int nimg, int src_kind, int src_dtype, const void* src, long long src_stride, void* Y,
             const void* roots, int cols, cudaStream_t st) {
    const long long NN = n >= 1 && n <= 11 ? 1ll << (2 * n) : 0;
    if (n < 1 || n > 11 || nimg < 0 || (src_kind != 0 && src_kind != 1) ||
        (src_dtype != ADRT_F32 && src_dtype != ADRT_F64) || (nimg && (!src || !Y || !roots)) ||
        (src_stride != 0 && (src_kind != 0 || src_stride < NN || src_stride % 4 != 0))) {
        set_error("pack_fft: bad arguments (n=%d nimg=%d src_kind=%d src_dtype=%d src_stride=%lld)", n, nimg, src_kind,
                  src_dtype, src_stride);
        return ADRT_EINVAL;
    }
    if (!nimg) return ADRT_OK;
    if (dtype == ADRT_F32) return pack_t<float>(n, nimg, src_kind, src_dtype, src, src_stride, Y, roots, cols, st);
    if (dtype == ADRT_F64) return pack_t<double>(n, nimg, src_kind, src_dtype, src, src_stride, Y, roots, cols, st);
    set_error("pack_fft: dtype must be F32 or F64");
    return ADRT_EINVAL;
}

int ifft_unpack(int dtype, int n, int nimg, const void* Z, void* colpart, void* row0, void* row3, const void* roots,
                int cols, cudaStream_t st) {
    if (n < 1 || n > 11 || nimg < 0 || (nimg && (!Z || !colpart || !row0 || !row3 || !roots))) {
        set_error("ifft_unpack: bad arguments (n=%d nimg=%d)", n, nimg);
        return ADRT_EINVAL;
    }
    if (!nimg) return ADRT_OK;
    if (dtype == ADRT_F32) return unpack_t<float>(n, nimg, Z, colpart, row0, row3, roots, cols, st);
    if (dtype == ADRT_F64) return unpack_t<double>(n, nimg, Z, colpart, row0, row3, roots, cols, st);
    set_error("ifft_unpack: dtype must be F32 or F64");
    return ADRT_EINVAL;
}

}  // namespace adrt
