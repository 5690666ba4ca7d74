// Dense low-frequency rows: for every dense row r of the packed rows and every image b,
//     Z[r, b] = W_r Y[b, row_r]        (W_r: N x N complex, the row's exact operator; reference: fastops.py:28-40,
//                                       100-117, with the butterflies around the filter folded into W_r on the host)
// computed out of place into Zd (nrows x nimg x N) and scattered back into Y.
//
// Tensor-core kernel (N >= 64, FP32 data): the complex product in real form,
//     [Re z; Im z] (2N x B) = [[Re W, -Im W], [Im W, Re W]] (2N x 2N) . [Re y; Im y] (2N x B),
// on tcgen05.mma kind::tf32 with the 3xTF32 split (a = a_hi + a_lo, products hi.hi + hi.lo + lo.hi, FP32 accumulation
// in tensor memory): about FP32 accuracy, which these rows need (they carry most of the image energy). One CTA per
// (dense row, 128 real output rows, batch tile of <= 64 images); K in chunks of 32 through two stages: the threads
// convert and store the A / X tiles of chunk k+1 into shared memory (canonical K-major layout without swizzle:
// 8-row x 16-byte core matrices, 128 B apart along K, 1024 B apart along M / N) while the tensor cores run chunk k;
// one thread issues 12 MMAs per chunk into one of two tensor-memory accumulators and commits them to that stage's
// mbarrier, on which every thread waits (bounded) before reusing the stage. Each accumulator holds one chunk only:
// the warps read it back (tcgen05.ld) and add it into FP32 registers, because accumulating all of K in tensor memory
// measured 2e-6..7e-6 relative error growing with K (truncating accumulation), against 1e-7 this way.
//
// CUDA-core kernel: the same product for any N and for FP64.
#include "common.cuh"
#include "launch.h"

namespace adrt {

// ------------------------------------------------------------------ scatter and CUDA-core product
template <typename C>
__global__ void dense_scatter_kernel(int N, int nimg, int nrows, const int* __restrict__ rows, const C* __restrict__ Zd,
                                     C* __restrict__ Y, long long img_stride) {
    const long long total = (long long)nrows * nimg * N;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const long long rb = e / N;
        const int o = (int)(e - rb * N);
        const int r = (int)(rb / nimg), b = (int)(rb - (long long)r * nimg);
        Y[b * img_stride + (long long)rows[r] * N + o] = Zd[e];
    }
}

template <typename real>
__global__ void __launch_bounds__(256) dense_simt_kernel(int N, int nimg, const int* __restrict__ rows,
                                                         const cplx<real>* __restrict__ W, const cplx<real>* __restrict__ Y,
                                                         long long img_stride, cplx<real>* __restrict__ Zd) {
    using C = cplx<real>;
    __shared__ C Wt[32][33];
    __shared__ C Yt[8][33];
    const int r = blockIdx.x, o0 = blockIdx.y * 32;
    const int oi = threadIdx.x & 31, bi = threadIdx.x >> 5;
    const C* Wr = W + (size_t)r * N * N;
    const long long row = rows[r];
    for (int b0 = 0; b0 < nimg; b0 += 8) {
        C acc = mk<real>(0, 0);
        for (int i0 = 0; i0 < N; i0 += 32) {
            for (int e = threadIdx.x; e < 32 * 32; e += 256) {
                const int a = e >> 5, c = e & 31;
                Wt[a][c] = (o0 + a < N && i0 + c < N) ? Wr[(size_t)(o0 + a) * N + i0 + c] : mk<real>(0, 0);
            }
            {
                const int c = threadIdx.x & 31, bb = threadIdx.x >> 5;
                Yt[bb][c] = (b0 + bb < nimg && i0 + c < N) ? Y[(b0 + bb) * img_stride + row * N + i0 + c] : mk<real>(0, 0);
            }
            __syncthreads();
#pragma unroll 8
            for (int c = 0; c < 32; ++c) acc = cfma(Wt[oi][c], Yt[bi][c], acc);
            __syncthreads();
        }
        if (o0 + oi < N && b0 + bi < nimg) Zd[((size_t)r * nimg + b0 + bi) * N + o0 + oi] = acc;
    }
}

// Small batches (nimg <= 16, FP32): the product streams each operator from HBM once per group of up to 8 images, so
// the kernel is built for that stream. The operator comes transposed, WT_r[i][o] = W_r[o][i], each thread owns one output row o and walks i, so
// a warp reads 32 consecutive complex values per i (coalesced), with eight loads in flight per thread; the images'
// input rows are staged in shared memory in chunks of DS_IC and read as broadcasts. FP32 FMA accumulation in two levels.
constexpr int DS_THREADS = 256;
constexpr int DS_IC = 512;
constexpr int DS_SUB = 128;
template <int NB>
__global__ void __launch_bounds__(DS_THREADS) dense_stream_kernel(int N, int nimg, const int* __restrict__ rows,
                                                                  const float2* __restrict__ WT,
                                                                  const float2* __restrict__ Y, long long img_stride,
                                                                  float2* __restrict__ Zd) {
    __shared__ float2 ys[NB][DS_IC];
    const int r = blockIdx.x;
    const int o = blockIdx.y * DS_THREADS + threadIdx.x;
    const int b0 = blockIdx.z * NB;  // images b0 .. b0 + NB - 1 (one pass over the operators per group of NB)
    const long long yrow = (long long)rows[r] * N;
    const bool live = o < N;
    float2 acc[NB];
#pragma unroll
    for (int b = 0; b < NB; ++b) acc[b] = make_float2(0.f, 0.f);
    for (int i0 = 0; i0 < N; i0 += DS_IC) {
        const int ic = N - i0 < DS_IC ? N - i0 : DS_IC;
        __syncthreads();
        for (int e = threadIdx.x; e < NB * ic; e += DS_THREADS) {
            const int b = e / ic, i = e - (e / ic) * ic;
            ys[b][i] = b0 + b < nimg ? Y[(b0 + b) * img_stride + yrow + i0 + i] : make_float2(0.f, 0.f);
        }
        __syncthreads();
        if (live) {
            const float2* w = WT + ((size_t)r * N + i0) * N + o;
            // two-level sum: a fresh partial every DS_SUB terms, added into the total (round-off grows with
            // sqrt(DS_SUB) + sqrt(N / DS_SUB) instead of sqrt(N))
            for (int ib = 0; ib < ic; ib += DS_SUB) {
                const int ie = ic - ib < DS_SUB ? ic : ib + DS_SUB;
                float2 part[NB];
#pragma unroll
                for (int b = 0; b < NB; ++b) part[b] = make_float2(0.f, 0.f);
#pragma unroll 8
                for (int i = ib; i < ie; ++i) {
                    const float2 wv = w[(size_t)i * N];
#pragma unroll
                    for (int b = 0; b < NB; ++b) part[b] = cfma(wv, ys[b][i], part[b]);
                }
#pragma unroll
                for (int b = 0; b < NB; ++b) acc[b] = cadd(acc[b], part[b]);
            }
        }
    }
    if (live) {
#pragma unroll
        for (int b = 0; b < NB; ++b)
            if (b0 + b < nimg) Zd[((size_t)r * nimg + b0 + b) * N + o] = acc[b];
    }
}

// ------------------------------------------------------------------ tcgen05 (sm_100 family) helpers
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: K-major, no swizzle; LBO = byte step between core matrices along K,
// SBO = byte step between 8-row groups along M / N; bits 46-47 = 1 (descriptor version of tcgen05)
__device__ __forceinline__ uint64_t desc_kmajor(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}

// bounded wait on an mbarrier phase; returns false if the limit ran out
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    for (long it = 0; it < (1L << 24); ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

constexpr int TC_M = 128;   // real output rows per CTA (TMEM lanes)
constexpr int TC_KC = 32;   // real K per chunk (16 complex columns of W)
constexpr int TC_THREADS = 256;

// Tiles in the canonical K-major no-swizzle layout of a TC_KC-wide chunk: element (row, k) at byte
// ((row/8) * (TC_KC/4) + k/4) * 128 + (row%8) * 16 + (k%4) * 4. K is interleaved by complex column:
// k = 2 (i - i0) + c multiplies Re y_i (c = 0) or Im y_i (c = 1), so A row m reads whole complex entries of W.
// Warps fill one core matrix per instruction: lane -> (row%8 = lane/4, k%4 = lane%4), 128 contiguous bytes.
template <int BP>
__global__ void __launch_bounds__(TC_THREADS) dense_tc_kernel(int N, int nimg, const int* __restrict__ rows,
                                                              const float2* __restrict__ W, const float2* __restrict__ Y,
                                                              long long img_stride, float2* __restrict__ Zd,
                                                              int* __restrict__ err) {
    constexpr int A_BYTES = TC_M * TC_KC * 4;  // 16 KB
    constexpr int X_BYTES = BP * TC_KC * 4;
    constexpr int STAGE = 2 * A_BYTES + 2 * X_BYTES;
    constexpr int NCOLS = 2 * BP <= 32 ? 32 : (2 * BP <= 64 ? 64 : 128);  // two accumulators of BP columns
    constexpr int HB = BP / 2;                                             // columns promoted per warp
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smem_raw + 2 * STAGE);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mbar + 3);  // mbar[2]: the drain barrier of the give-up path

    const int r = blockIdx.x;
    const int m0 = blockIdx.y * TC_M;  // first real output row of this CTA (0 .. 2N)
    const int b0 = blockIdx.z * BP;    // first image of this CTA
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const float2* Wr = W + (size_t)r * N * N;
    const long long yrow = (long long)rows[r] * N;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                     "r"(NCOLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&mbar[0])));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&mbar[1])));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&mbar[2])));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    // instruction descriptor: D f32 (bits 4-5 = 1), A and B tf32 (bits 7-9, 10-12 = 2), both K-major,
    // N >> 3 at bits 17-22, M >> 4 at bits 24-28
    const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BP >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);
    const int kchunks = (2 * N) / TC_KC;
    // warps w and w + 4 read the same 32 accumulator lanes (rows), each half of the columns
    const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
    const int col0 = (warp >> 2) * HB;
    float acc[HB];
#pragma unroll
    for (int q = 0; q < HB; ++q) acc[q] = 0.f;
    bool ok = true;

    // add one chunk's partial sums (accumulator s) into the FP32 registers
    auto promote = [&](int s) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
        for (int c = 0; c < HB; c += 8) {
            uint32_t v[8];
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                         : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
                         : "r"(tmem + lane_base + (uint32_t)(s * BP + col0 + c)));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int q = 0; q < 8; ++q) acc[c + q] += __uint_as_float(v[q]);
        }
    };

    // operand tiles: every thread issues all its loads of a chunk at once (AIT + XIT independent loads in flight),
    // one chunk ahead: the loads of chunk kc + 1 are issued right after the MMAs of chunk kc and land while the
    // MMAs of chunk kc - 1 are awaited and folded in; core matrix cm = warp + it * 8
    constexpr int AIT = (TC_M / 8) * (TC_KC / 4) / (TC_THREADS / 32);
    constexpr int XIT = (BP / 8) * (TC_KC / 4) / (TC_THREADS / 32);
    float2 wv[AIT], yv[XIT];
    auto load_chunk = [&](int kc) {
        const int i0 = kc * (TC_KC / 2);
#pragma unroll
        for (int it = 0; it < AIT; ++it) {
            const int cm = warp + it * (TC_THREADS / 32);
            const int rg = cm / (TC_KC / 4), kg = cm % (TC_KC / 4);
            const int m = m0 + rg * 8 + (lane >> 2), k = kg * 4 + (lane & 3);
            const int outhalf = m >= N ? 1 : 0;
            wv[it] = Wr[(size_t)(m - outhalf * N) * N + i0 + (k >> 1)];
        }
#pragma unroll
        for (int it = 0; it < XIT; ++it) {
            const int cm = warp + it * (TC_THREADS / 32);
            const int rg = cm / (TC_KC / 4), kg = cm % (TC_KC / 4);
            const int b = b0 + rg * 8 + (lane >> 2), k = kg * 4 + (lane & 3);
            yv[it] = b < nimg ? Y[b * img_stride + yrow + i0 + (k >> 1)] : make_float2(0.f, 0.f);
        }
    };
    load_chunk(0);

    for (int kc = 0; kc < kchunks; ++kc) {
        const int s = kc & 1;
        unsigned char* a_hi = smem_raw + s * STAGE;
        unsigned char* a_lo = a_hi + A_BYTES;
        unsigned char* x_hi = a_lo + A_BYTES;
        unsigned char* x_lo = x_hi + X_BYTES;
        if (kc >= 2) {
            // chunk kc-2 used this stage and accumulator: wait for its MMAs, fold its partial in
            const int waited = mbar_wait(smem_addr(&mbar[s]), (uint32_t)(((kc - 2) >> 1) & 1)) ? 1 : 0;
            ok = __syncthreads_and(waited) != 0;
            if (!ok) break;
            promote(s);
        }
#pragma unroll
        for (int it = 0; it < AIT; ++it) {
            const int cm = warp + it * (TC_THREADS / 32);
            const int rg = cm / (TC_KC / 4);
            const int m = m0 + rg * 8 + (lane >> 2), k = (cm % (TC_KC / 4)) * 4 + (lane & 3);
            const int outhalf = m >= N ? 1 : 0;
            const int c = k & 1;
            const float2 w = wv[it];
            const float v = outhalf == 0 ? (c == 0 ? w.x : -w.y) : (c == 0 ? w.y : w.x);
            const uint32_t hi = to_tf32(v);
            const uint32_t lo = to_tf32(v - __uint_as_float(hi));
            const int off = cm * 128 + lane * 4;
            *reinterpret_cast<uint32_t*>(a_hi + off) = hi;
            *reinterpret_cast<uint32_t*>(a_lo + off) = lo;
        }
#pragma unroll
        for (int it = 0; it < XIT; ++it) {
            const int cm = warp + it * (TC_THREADS / 32);
            const int k = (cm % (TC_KC / 4)) * 4 + (lane & 3);
            const float v = (k & 1) ? yv[it].y : yv[it].x;
            const uint32_t hi = to_tf32(v);
            const uint32_t lo = to_tf32(v - __uint_as_float(hi));
            const int off = cm * 128 + lane * 4;
            *reinterpret_cast<uint32_t*>(x_hi + off) = hi;
            *reinterpret_cast<uint32_t*>(x_lo + off) = lo;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (threadIdx.x == 0) {
            const uint32_t d = tmem + (uint32_t)(s * BP);
#pragma unroll
            for (int k8 = 0; k8 < TC_KC / 8; ++k8) {
                const uint32_t koff = k8 * 256;  // two core matrices along K
                const uint64_t ah = desc_kmajor(smem_addr(a_hi) + koff, 128, (TC_KC / 4) * 128);
                const uint64_t al = desc_kmajor(smem_addr(a_lo) + koff, 128, (TC_KC / 4) * 128);
                const uint64_t xh = desc_kmajor(smem_addr(x_hi) + koff, 128, (TC_KC / 4) * 128);
                const uint64_t xl = desc_kmajor(smem_addr(x_lo) + koff, 128, (TC_KC / 4) * 128);
                mma_tf32(d, ah, xh, idesc, k8 > 0 ? 1u : 0u);
                mma_tf32(d, ah, xl, idesc, 1u);
                mma_tf32(d, al, xh, idesc, 1u);
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_addr(&mbar[s]))
                         : "memory");
        }
        if (kc + 1 < kchunks) load_chunk(kc + 1);
    }
    // drain: the last two chunks
    if (ok) {
        for (int kc = kchunks - 2 > 0 ? kchunks - 2 : 0; kc < kchunks; ++kc) {
            const int s = kc & 1;
            const int waited = mbar_wait(smem_addr(&mbar[s]), (uint32_t)((kc >> 1) & 1)) ? 1 : 0;
            ok = __syncthreads_and(waited) != 0;
            if (!ok) break;
            promote(s);
        }
    }
    if (!ok && threadIdx.x == 0) {
        // a wait gave up while MMAs of this CTA may still be writing its TMEM columns: before the columns are freed
        // (and possibly handed to the next CTA on this SM), one more commit of every tcgen05 operation this thread
        // issued goes to the spare barrier, awaited with the same bound. Flag 1: the launch's dense rows were not
        // written; flag 2: even the drain ran out, so the stream's later device results cannot be trusted either.
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_addr(&mbar[2]))
                     : "memory");
        const bool drained = mbar_wait(smem_addr(&mbar[2]), 0u);
        atomicMax(err, drained ? 1 : 2);
    }
    if (ok) {
        const int mrow = m0 + (warp & 3) * 32 + lane;
        const int outhalf = mrow >= N ? 1 : 0;
        const int o = mrow - outhalf * N;
        float* zf = reinterpret_cast<float*>(Zd);
#pragma unroll
        for (int q = 0; q < HB; ++q) {
            const int b = b0 + col0 + q;
            if (b < nimg) zf[(((size_t)r * nimg + b) * N + o) * 2 + outhalf] = acc[q];
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(NCOLS));
}

// ------------------------------------------------------------------ complex-blocked tensor-core kernel on pre-split
// operators (N >= 128, FP32 data). The operators are constant, so they are split once (dense_split) into TF32 tiles in
// the MMA's K-major layout: per (dense row, block of 128 output rows, chunk of 16 input columns) four 8 KB tiles
// Re W hi, Re W lo, Im W hi, Im W lo, stored contiguously (32 KB per chunk, one bulk copy). With the images' rows split
// the same way per chunk, three TMEM accumulators hold
//     P1 = Re W Re y,   P2 = Im W Im y,   P3 = Im W Re y + Re W Im y     (each term 3xTF32: hi hi + hi lo + lo hi)
// and z = (P1 - P2) + i P3: half the operator bytes of the real 2N x 2N form for the same products. Pipeline: a ring
// of CX_S stages; one thread issues the bulk copy of a chunk's operator tiles two chunks ahead (mbarrier with a byte
// count), every thread converts its share of the image rows of the current chunk into the stage, one thread issues
// the chunk's 24 MMAs into one of two accumulator sets and commits them to the stage's mbarrier, and the chunk two
// back is folded into FP32 registers (its MMAs complete by then) while the tensor cores run the current one.
constexpr int CX_M = 128;            // complex output rows per CTA (TMEM lanes)
constexpr int CX_KC = 16;            // complex input columns per chunk
constexpr int CX_S = 4;              // pipeline stages
constexpr int CX_TILE = CX_M * CX_KC;  // floats per operator tile
constexpr int CX_THREADS = 256;
// after the stages: 3 CX_S + 5 mbarriers, then the TMEM slot and three flags
constexpr int CX_BAR_BYTES = 256;
static_assert((3 * CX_S + 5) * 8 + 4 * 4 <= CX_BAR_BYTES, "barrier area too small");

// W (nrows x N x N complex FP32, [row][out][in]) -> Ws (nrows x N/128 x N/16 x 4 tiles x CX_TILE floats); element
// (o, i) of a tile at float ((o%128)/8 * (CX_KC/4) + (i%16)/4) * 32 + (o%8) * 4 + i%4 (core matrices of 8 rows x 16 B)
__global__ void dense_split_kernel(int N, long long total, const float2* __restrict__ W, float* __restrict__ Ws) {
    const int MT = N / CX_M, NC = N / CX_KC;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const long long ro = e / N;
        const int i = (int)(e - ro * N);
        const long long r = ro / N;
        const int o = (int)(ro - r * N);
        const float2 w = W[e];
        const int mt = o / CX_M, om = o % CX_M, c = i / CX_KC, k = i % CX_KC;
        float* t = Ws + (((size_t)r * MT + mt) * NC + c) * 4 * CX_TILE + ((om / 8) * (CX_KC / 4) + k / 4) * 32 +
                   (om % 8) * 4 + (k % 4);
        const uint32_t reh = to_tf32(w.x), imh = to_tf32(w.y);
        t[0] = __uint_as_float(reh);
        t[CX_TILE] = __uint_as_float(to_tf32(w.x - __uint_as_float(reh)));
        t[2 * CX_TILE] = __uint_as_float(imh);
        t[3 * CX_TILE] = __uint_as_float(to_tf32(w.y - __uint_as_float(imh)));
    }
}

__device__ __forceinline__ void mbar_expect_bulk(uint32_t mbar, uint32_t dst, const void* src, uint32_t bytes) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}\n" ::"r"(mbar),
                 "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(mbar)
                 : "memory");
}

// bounded wait that also gives up when another role of the CTA has set the abort flag
__device__ __forceinline__ bool mbar_wait_or_abort(uint32_t mbar, uint32_t parity, const volatile int* abort_flag) {
    for (long it = 0; it < (1L << 24); ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
        if ((it & 255) == 255 && *abort_flag) return false;
    }
    return false;
}
// the same, polled by lane 0 of a converged warp and broadcast, so that every lane takes the same branch
__device__ __forceinline__ bool warp_wait(uint32_t mbar, uint32_t parity, const volatile int* abort_flag) {
    int okv = 0;
    if ((threadIdx.x & 31) == 0) okv = mbar_wait_or_abort(mbar, parity, abort_flag) ? 1 : 0;
    return __shfl_sync(0xffffffffu, okv, 0) != 0;
}
__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}\n" ::"r"(mbar) : "memory");
}

// Warp-specialised: warp 0 (one thread) streams the operator tiles of chunk after chunk into the ring, warps 2-3 build
// the image tiles, warp 1 (one thread) issues the MMAs, warps 4-7 fold each chunk's accumulator set into FP32
// registers and write the result. Per stage: a_full (operator bytes landed), x_full (64 image-tile arrivals),
// stage_free (commit of the chunk's MMAs); per accumulator set: acc_full (commit), acc_free (128 fold arrivals).
// The CTAs of one row (its N / 128 blocks of output rows) form a thread-block cluster: each reads the whole input row
// while it runs, so the results are written in place only after a cluster barrier at the end, when every CTA of the
// row has finished reading (no staging buffer, no scatter).
template <int BP>
__global__ void __launch_bounds__(CX_THREADS, 1) dense_cx_kernel(int N, int nimg, const int* __restrict__ rows,
                                                                 const float* __restrict__ Ws, float2* Y,
                                                                 long long img_stride, int* __restrict__ err) {
    constexpr int A_BYTES = 4 * CX_TILE * 4;  // 32 KB
    constexpr int XT = BP * CX_KC;            // floats per image tile
    constexpr int STAGE = A_BYTES + 6 * XT * 4;  // image tiles: Re hi, Re lo, Im hi, Im lo, -Im hi, -Im lo
    constexpr int NACC = 2 * BP;                 // columns of one accumulator set (Re z, Im z)
    constexpr int NCOLS = 2 * NACC <= 64 ? 64 : (2 * NACC <= 128 ? 128 : 256);
    constexpr int XW = 64;  // image-tile threads (warps 2-3)
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    uint64_t* a_full = reinterpret_cast<uint64_t*>(smem_raw + CX_S * STAGE);
    uint64_t* x_full = a_full + CX_S;
    uint64_t* stage_free = x_full + CX_S;
    uint64_t* acc_full = stage_free + CX_S;
    uint64_t* acc_free = acc_full + 2;
    uint64_t* drain = acc_free + 2;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    volatile int* s_issued = abort_flag + 1;    // operator chunks whose copy was issued (warp 0)
    volatile int* s_consumed = abort_flag + 2;  // operator chunks seen landed (warp 1)

    const int r = blockIdx.x, mt = blockIdx.y, b0 = blockIdx.z * BP;
    const int MT = N / CX_M, NC = N / CX_KC;
    const float* Wr = Ws + ((size_t)r * MT + mt) * NC * 4 * CX_TILE;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long yrow = (long long)rows[r] * N;
    float zr[BP], zi[BP];  // the fold warps' results (warps 4-7), written after the cluster barrier
    bool folded = false;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                     "r"(NCOLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (threadIdx.x == 32) {
        for (int q = 0; q < CX_S; ++q) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&a_full[q])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&x_full[q])), "r"(XW));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&stage_free[q])));
        }
        for (int q = 0; q < 2; ++q) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&acc_full[q])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 128;" ::"r"(smem_addr(&acc_free[q])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(drain)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *abort_flag = 0;
        *s_issued = 0;
        *s_consumed = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    // every role runs its loop on whole warps (lane 0 issues; waits are polled by lane 0 and broadcast), so the warps
    // stay converged for the CTA barrier at the end
    if (warp == 0) {  // operator tiles, chunk after chunk, as soon as a stage is free
        for (int kc = 0; kc < NC; ++kc) {
            const int s = kc % CX_S, u = kc / CX_S;
            if (u > 0 && !warp_wait(smem_addr(&stage_free[s]), (uint32_t)((u - 1) & 1), abort_flag)) {
                if (lane == 0) *abort_flag = 1;
                break;
            }
            if (lane == 0) {
                mbar_expect_bulk(smem_addr(&a_full[s]), smem_addr(smem_raw + s * STAGE), Wr + (size_t)kc * 4 * CX_TILE,
                                 A_BYTES);
                *s_issued = kc + 1;
            }
            __syncwarp();
        }
    } else if (warp == 1) {
        {  // the MMAs of chunk after chunk
            const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BP >> 3) << 17) |
                                   ((uint32_t)(CX_M >> 4) << 24);
            constexpr uint32_t SBO = (CX_KC / 4) * 128;
            for (int kc = 0; kc < NC; ++kc) {
                // accumulator set of chunk kc: kc % 2 (its v-th use, v = kc / 2); every chunk is folded into FP32
                // registers on its own (accumulating two chunks in tensor memory measured a larger error)
                const int s = kc % CX_S, u = kc / CX_S, be = kc & 1, v = kc >> 1;
                if (!warp_wait(smem_addr(&a_full[s]), (uint32_t)(u & 1), abort_flag)) {
                    if (lane == 0) *abort_flag = 1;
                    break;
                }
                if (lane == 0) *s_consumed = kc + 1;
                if (!warp_wait(smem_addr(&x_full[s]), (uint32_t)(u & 1), abort_flag) ||
                    (v > 0 && !warp_wait(smem_addr(&acc_free[be]), (uint32_t)((v - 1) & 1), abort_flag))) {
                    if (lane == 0) *abort_flag = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                if (lane == 0) {
                    const uint32_t d = tmem + (uint32_t)(be * NACC);
                    const uint32_t a0 = smem_addr(smem_raw + s * STAGE), x0 = a0 + A_BYTES;
#pragma unroll
                    for (int k8 = 0; k8 < CX_KC / 8; ++k8) {
                        const uint32_t ko = k8 * 256;
                        const uint64_t reh = desc_kmajor(a0 + ko, 128, SBO), rel = desc_kmajor(a0 + CX_TILE * 4 + ko, 128, SBO);
                        const uint64_t imh = desc_kmajor(a0 + 2 * CX_TILE * 4 + ko, 128, SBO);
                        const uint64_t iml = desc_kmajor(a0 + 3 * CX_TILE * 4 + ko, 128, SBO);
                        const uint64_t xrh = desc_kmajor(x0 + ko, 128, SBO), xrl = desc_kmajor(x0 + XT * 4 + ko, 128, SBO);
                        const uint64_t xih = desc_kmajor(x0 + 2 * XT * 4 + ko, 128, SBO);
                        const uint64_t xil = desc_kmajor(x0 + 3 * XT * 4 + ko, 128, SBO);
                        const uint64_t xnh = desc_kmajor(x0 + 4 * XT * 4 + ko, 128, SBO);
                        const uint64_t xnl = desc_kmajor(x0 + 5 * XT * 4 + ko, 128, SBO);
                        const uint32_t acc = k8 == 0 ? 0u : 1u;
                        mma_tf32(d, reh, xrh, idesc, acc);  // Re z = Re W Re y + Im W (-Im y)
                        mma_tf32(d, reh, xrl, idesc, 1u);
                        mma_tf32(d, rel, xrh, idesc, 1u);
                        mma_tf32(d, imh, xnh, idesc, 1u);
                        mma_tf32(d, imh, xnl, idesc, 1u);
                        mma_tf32(d, iml, xnh, idesc, 1u);
                        mma_tf32(d + BP, imh, xrh, idesc, acc);  // Im z = Im W Re y + Re W Im y
                        mma_tf32(d + BP, imh, xrl, idesc, 1u);
                        mma_tf32(d + BP, iml, xrh, idesc, 1u);
                        mma_tf32(d + BP, reh, xih, idesc, 1u);
                        mma_tf32(d + BP, reh, xil, idesc, 1u);
                        mma_tf32(d + BP, rel, xih, idesc, 1u);
                    }
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                     smem_addr(&stage_free[s]))
                                 : "memory");
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                     smem_addr(&acc_full[be]))
                                 : "memory");
                }
                __syncwarp();
            }
        }
    } else if (warp < 4) {  // image tiles: item e = (image e / 4, quad e % 4 of the chunk's 16 columns)
        const int t = threadIdx.x - 64;
        constexpr int ITEMS = BP * (CX_KC / 4);
        constexpr int PER = (ITEMS + XW - 1) / XW;
        // three chunks of image values in flight: the loads of chunk kc + 3 are issued once chunk kc is stored
        float4 ya0[PER], yb0[PER], ya1[PER], yb1[PER], ya2[PER], yb2[PER];
        auto load = [&](int kc, float4 (&ya)[PER], float4 (&yb)[PER]) {
#pragma unroll
            for (int j = 0; j < PER; ++j) {
                const int e = t + j * XW, xb = e / (CX_KC / 4), xq = e % (CX_KC / 4);
                ya[j] = yb[j] = make_float4(0.f, 0.f, 0.f, 0.f);
                if (kc < NC && e < ITEMS && b0 + xb < nimg) {
                    const float4* src = reinterpret_cast<const float4*>(Y + (long long)(b0 + xb) * img_stride + yrow +
                                                                        kc * CX_KC + 4 * xq);
                    ya[j] = src[0];
                    yb[j] = src[1];
                }
            }
        };
        // store chunk kc (values in ya, yb) into its stage, then load chunk kc + 3 into the same registers
        auto step = [&](int kc, float4 (&ya)[PER], float4 (&yb)[PER]) -> bool {
            const int s = kc % CX_S, u = kc / CX_S;
            if (u > 0 && !warp_wait(smem_addr(&stage_free[s]), (uint32_t)((u - 1) & 1), abort_flag)) {
                if (lane == 0) *abort_flag = 1;
                return false;
            }
            unsigned char* xt = smem_raw + s * STAGE + A_BYTES;
#pragma unroll
            for (int j = 0; j < PER; ++j) {
                const int e = t + j * XW, xb = e / (CX_KC / 4), xq = e % (CX_KC / 4);
                if (e >= ITEMS) continue;
                const float re[4] = {ya[j].x, ya[j].z, yb[j].x, yb[j].z}, im[4] = {ya[j].y, ya[j].w, yb[j].y, yb[j].w};
                uint32_t rh[4], rl[4], ih[4], il[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    rh[q] = to_tf32(re[q]);
                    rl[q] = to_tf32(re[q] - __uint_as_float(rh[q]));
                    ih[q] = to_tf32(im[q]);
                    il[q] = to_tf32(im[q] - __uint_as_float(ih[q]));
                }
                const int off = ((xb / 8) * (CX_KC / 4) + xq) * 128 + (xb % 8) * 16;
                *reinterpret_cast<uint4*>(xt + off) = make_uint4(rh[0], rh[1], rh[2], rh[3]);
                *reinterpret_cast<uint4*>(xt + XT * 4 + off) = make_uint4(rl[0], rl[1], rl[2], rl[3]);
                *reinterpret_cast<uint4*>(xt + 2 * XT * 4 + off) = make_uint4(ih[0], ih[1], ih[2], ih[3]);
                *reinterpret_cast<uint4*>(xt + 3 * XT * 4 + off) = make_uint4(il[0], il[1], il[2], il[3]);
                constexpr uint32_t SG = 0x80000000u;  // -Im y: the sign flipped, exactly
                *reinterpret_cast<uint4*>(xt + 4 * XT * 4 + off) = make_uint4(ih[0] ^ SG, ih[1] ^ SG, ih[2] ^ SG, ih[3] ^ SG);
                *reinterpret_cast<uint4*>(xt + 5 * XT * 4 + off) = make_uint4(il[0] ^ SG, il[1] ^ SG, il[2] ^ SG, il[3] ^ SG);
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_arrive(smem_addr(&x_full[s]));
            load(kc + 3, ya, yb);
            return true;
        };
        load(0, ya0, yb0);
        load(1, ya1, yb1);
        load(2, ya2, yb2);
        for (int kc = 0; kc < NC; kc += 3) {
            if (!step(kc, ya0, yb0)) break;
            if (kc + 1 < NC && !step(kc + 1, ya1, yb1)) break;
            if (kc + 2 < NC && !step(kc + 2, ya2, yb2)) break;
        }
    } else {  // warps 4-7: fold every accumulator set (TMEM lanes 32 (warp % 4) ..) into FP32 registers
        const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
#pragma unroll
        for (int q = 0; q < BP; ++q) zr[q] = zi[q] = 0.f;
        bool ok = true;
        // all of one accumulator's columns are loaded before the single wait for them
        auto fold = [&](uint32_t addr, float (&z)[BP]) {
            uint32_t t[BP];
#pragma unroll
            for (int c = 0; c < BP; c += 16)
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                    "[%16];"
                    : "=r"(t[c]), "=r"(t[c + 1]), "=r"(t[c + 2]), "=r"(t[c + 3]), "=r"(t[c + 4]), "=r"(t[c + 5]),
                      "=r"(t[c + 6]), "=r"(t[c + 7]), "=r"(t[c + 8]), "=r"(t[c + 9]), "=r"(t[c + 10]), "=r"(t[c + 11]),
                      "=r"(t[c + 12]), "=r"(t[c + 13]), "=r"(t[c + 14]), "=r"(t[c + 15])
                    : "r"(addr + c));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int q = 0; q < BP; ++q) z[q] += __uint_as_float(t[q]);
        };
        for (int kc = 0; kc < NC; ++kc) {
            const int be = kc & 1, v = kc >> 1;
            if (!warp_wait(smem_addr(&acc_full[be]), (uint32_t)(v & 1), abort_flag)) {
                if (lane == 0) *abort_flag = 1;
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t base = tmem + lane_base + (uint32_t)(be * NACC);
            fold(base, zr);
            fold(base + BP, zi);
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            mbar_arrive(smem_addr(&acc_free[be]));
        }
        folded = ok;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (*abort_flag && threadIdx.x == 32) {
        // a wait gave up: before the tensor memory is freed and the CTA leaves, every MMA issued (one more commit to
        // the spare barrier) and every operator copy issued (the stages' byte counts) must have completed; the waits
        // are bounded. Flag 1: this launch's dense rows were not written; 2: even the drain ran out.
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_addr(drain))
                     : "memory");
        bool drained = mbar_wait(smem_addr(drain), 0u);
        for (int kc = *s_consumed; kc < *s_issued; ++kc)  // at most CX_S outstanding copies, in distinct stages
            drained = mbar_wait(smem_addr(&a_full[kc % CX_S]), (uint32_t)((kc / CX_S) & 1)) && drained;
        atomicMax(err, drained ? 1 : 2);
    }
    __syncthreads();
    // every CTA of the row has read its inputs: the results go in place (none if any role of this CTA gave up)
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
    if (folded && !*abort_flag) {
        const int o = mt * CX_M + (warp & 3) * 32 + lane;
#pragma unroll
        for (int q = 0; q < BP; ++q) {
            const int b = b0 + q;
            if (b < nimg) Y[(long long)b * img_stride + yrow + o] = make_float2(zr[q], zi[q]);
        }
    }
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(NCOLS));
}

template <int BP>
static int launch_cx(int n, int nimg, int nrows, const int* rows, const void* Ws, void* Y, long long img_stride, int* err,
                     cudaStream_t st) {
    const int N = 1 << n;
    const size_t smem = (size_t)CX_S * (4 * CX_TILE * 4 + 6 * BP * CX_KC * 4) + CX_BAR_BYTES;  // stages, barriers
    auto kern = dense_cx_kernel<BP>;
    if (int rc = ensure_smem((const void*)kern, smem)) return rc;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nrows, N / CX_M, (nimg + BP - 1) / BP);
    cfg.blockDim = dim3(CX_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;  // the N / 128 CTAs of a row (at most 8 for N <= 1024)
    attr[0].val.clusterDim.x = 1;
    attr[0].val.clusterDim.y = N / CX_M;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return launch_ex_status(cudaLaunchKernelEx(&cfg, kern, N, nimg, rows, reinterpret_cast<const float*>(Ws),
                                               reinterpret_cast<float2*>(Y), img_stride, err),
                            "dense_cx_kernel");
}

int dense_split(int n, int nrows, const void* W, void* Ws, cudaStream_t st) {
    if (n < 7 || n > 10 || nrows < 0 || (nrows && (!W || !Ws))) {
        set_error("dense_split: bad arguments (n=%d nrows=%d; n must be 7..10)", n, nrows);
        return ADRT_EINVAL;
    }
    const long long total = (long long)nrows << (2 * n);
    if (!total) return ADRT_OK;
    long long g = (total + 255) / 256;
    if (g > 65535LL * 16) g = 65535LL * 16;
    dense_split_kernel<<<(int)g, 256, 0, st>>>(1 << n, total, reinterpret_cast<const float2*>(W),
                                               reinterpret_cast<float*>(Ws));
    return launch_status("dense_split_kernel");
}

template <int BP>
static int launch_tc(int n, int nimg, int nrows, const int* rows, const void* W, const void* Y, long long img_stride,
                     void* Zd, int* err, cudaStream_t st) {
    const int N = 1 << n;
    const size_t smem = 2 * (2 * (size_t)TC_M * TC_KC * 4 + 2 * (size_t)BP * TC_KC * 4) + 64;
    auto kern = dense_tc_kernel<BP>;
    if (int rc = ensure_smem((const void*)kern, smem)) return rc;
    dim3 grid(nrows, (2 * N) / TC_M, (nimg + BP - 1) / BP);
    kern<<<grid, TC_THREADS, smem, st>>>(N, nimg, rows, reinterpret_cast<const float2*>(W),
                                         reinterpret_cast<const float2*>(Y), img_stride, reinterpret_cast<float2*>(Zd), err);
    return launch_status("dense_tc_kernel");
}

int dense_rows(int dtype, int n, int nimg, int nrows, const int* rows, const void* W, void* Y, long long img_stride,
               void* Zd, int* err, int use_tc, int tile, cudaStream_t st) {
    if (tile != 0 && tile != 16 && tile != 32 && tile != 64) {
        set_error("dense_rows: tile must be 0 (auto), 16, 32 or 64 images per CTA");
        return ADRT_EINVAL;
    }
    if ((dtype != ADRT_F32 && dtype != ADRT_F64) || n < 1 || n > 11 || nimg < 0 || nrows < 0 ||
        (nimg && nrows && (!rows || !W || !Y || (!Zd && use_tc != 3)))) {
        set_error("dense_rows: bad arguments (dtype=%d n=%d nimg=%d nrows=%d)", dtype, n, nimg, nrows);
        return ADRT_EINVAL;
    }
    if (!nimg || !nrows) return ADRT_OK;
    const int N = 1 << n;
    int rc;
    if (use_tc == 3) {
        if (dtype != ADRT_F32 || n < 7 || n > 10 || !err) {
            set_error("dense_rows: the pre-split tensor-core kernel (use_tc = 3) takes FP32, 7 <= n <= 10 and an error "
                      "flag");
            return ADRT_EINVAL;
        }
        const int bp = tile ? tile : (nimg <= 16 ? 16 : (nimg <= 32 ? 32 : 64));
        if (bp == 16) return launch_cx<16>(n, nimg, nrows, rows, W, Y, img_stride, err, st);
        if (bp == 32) return launch_cx<32>(n, nimg, nrows, rows, W, Y, img_stride, err, st);
        return launch_cx<64>(n, nimg, nrows, rows, W, Y, img_stride, err, st);  // in place: no Zd, no scatter
    } else if (use_tc == 2) {
        if (dtype != ADRT_F32 || nimg > 16) {
            set_error("dense_rows: the streaming kernel (use_tc = 2) takes FP32 and at most 16 images (nimg=%d)", nimg);
            return ADRT_EINVAL;
        }
        dim3 grid(nrows, (N + DS_THREADS - 1) / DS_THREADS, nimg > 8 ? (nimg + 7) / 8 : 1);
        const float2* Wt = reinterpret_cast<const float2*>(W);
        const float2* Yf = reinterpret_cast<const float2*>(Y);
        float2* Zf = reinterpret_cast<float2*>(Zd);
        if (nimg <= 1) dense_stream_kernel<1><<<grid, DS_THREADS, 0, st>>>(N, nimg, rows, Wt, Yf, img_stride, Zf);
        else if (nimg <= 2) dense_stream_kernel<2><<<grid, DS_THREADS, 0, st>>>(N, nimg, rows, Wt, Yf, img_stride, Zf);
        else if (nimg <= 4) dense_stream_kernel<4><<<grid, DS_THREADS, 0, st>>>(N, nimg, rows, Wt, Yf, img_stride, Zf);
        else dense_stream_kernel<8><<<grid, DS_THREADS, 0, st>>>(N, nimg, rows, Wt, Yf, img_stride, Zf);
        rc = launch_status("dense_stream_kernel");
    } else if (dtype == ADRT_F32 && use_tc && n >= 6) {
        if (!err) { set_error("dense_rows: the tensor-core path needs an error flag"); return ADRT_EINVAL; }
        const int bp = tile ? tile : (nimg <= 16 ? 16 : (nimg <= 32 ? 32 : 64));  // images per CTA
        if (bp == 16) rc = launch_tc<16>(n, nimg, nrows, rows, W, Y, img_stride, Zd, err, st);
        else if (bp == 32) rc = launch_tc<32>(n, nimg, nrows, rows, W, Y, img_stride, Zd, err, st);
        else rc = launch_tc<64>(n, nimg, nrows, rows, W, Y, img_stride, Zd, err, st);
    } else {
        dim3 grid(nrows, (N + 31) / 32);
        if (dtype == ADRT_F32)
            dense_simt_kernel<float><<<grid, 256, 0, st>>>(N, nimg, rows, reinterpret_cast<const float2*>(W),
                                                           reinterpret_cast<const float2*>(Y), img_stride,
                                                           reinterpret_cast<float2*>(Zd));
        else
            dense_simt_kernel<double><<<grid, 256, 0, st>>>(N, nimg, rows, reinterpret_cast<const double2*>(W),
                                                            reinterpret_cast<const double2*>(Y), img_stride,
                                                            reinterpret_cast<double2*>(Zd));
        rc = launch_status("dense_simt_kernel");
    }
    if (rc) return rc;
    const long long total = (long long)nrows * nimg * N;
    int grid = (int)((total + 255) / 256);
    if (grid > 65535 * 4) grid = 65535 * 4;
    if (dtype == ADRT_F32)
        dense_scatter_kernel<float2><<<grid, 256, 0, st>>>(N, nimg, nrows, rows, reinterpret_cast<const float2*>(Zd),
                                                           reinterpret_cast<float2*>(Y), img_stride);
    else
        dense_scatter_kernel<double2><<<grid, 256, 0, st>>>(N, nimg, nrows, rows, reinterpret_cast<const double2*>(Zd),
                                                            reinterpret_cast<double2*>(Y), img_stride);
    return launch_status("dense_scatter_kernel");
}

}  // namespace adrt
