// Compensated rows: the row engine's op lists (butterflies B, adjoints B^*, Grams M = B^* B, the Chebyshev filter
// p_k(M) of cpp/oblique.cpp:74-104 / fastops.py:100-138) on selected FP32 rows in float-float arithmetic (about 48
// significant bits on the FP32 pipe, ff.cuh), for the high-condition rows where FP32 loses accuracy.
//
// Why: the filter approximates (M + tau)^-1 and the G_h / frame op lists end with M applied to its output. On a
// low-frequency row M_k has a near-null space while (Lambda_k + tau)/tau reaches several hundred, so every FP32
// evaluation of M z (inside the recurrence's residual and at the end) carries an error of about eps Lambda ||z||,
// kappa eps relative to the result (measured in emulation: 8e-5 at N=256, k = 0). Compensating only the update of
// z does not help; the products with M must be carried in extended precision. Here the whole op list of such a row
// runs in float-float: twiddles from the FP64 roots of unity, the filter constants from the FP64 table, the row read
// from and written back to the FP32 packed rows.
//
// One CTA per work item (row, image), the row in shared memory in natural order, levels ping-ponged between two
// buffers (the level arithmetic of cpp/oblique.cpp:22-51); the filter keeps y, z and the step delta in shared memory.
#include "common.cuh"
#include "ff.cuh"
#include "launch.h"

namespace adrt {

constexpr int FF_THREADS = 512;  // the largest CTA; N <= 512 rows take 256 threads

// forward levels lo..hi: o[2t] = f0[t] + z^t f1[t], o[2t+1] = f0[t] + z^(t+1) f1[t]
__device__ void ff_fwd(ffc*& a, ffc*& b, int N, int lo, int hi, const ffc* tw) {
    for (int m = lo; m <= hi; ++m) {
        const int w = 1 << (m - 1);
        for (int i = threadIdx.x; i < N / 2; i += blockDim.x) {
            const int l = i / w, t = i - l * w, base = l * 2 * w;
            const ffc f0 = a[base + t], f1 = a[base + w + t];
            b[base + 2 * t] = ffc_add(f0, ffc_mul(tw[t], f1));
            b[base + 2 * t + 1] = ffc_add(f0, ffc_mul(tw[t + 1], f1));
        }
        __syncthreads();
        ffc* s = a; a = b; b = s;
    }
}

// adjoint levels hi..lo: o0[t] = g0 + g1, o1[t] = conj(z^t) g0 + conj(z^(t+1)) g1
__device__ void ff_adj(ffc*& a, ffc*& b, int N, int lo, int hi, const ffc* tw) {
    for (int m = hi; m >= lo; --m) {
        const int w = 1 << (m - 1);
        for (int i = threadIdx.x; i < N / 2; i += blockDim.x) {
            const int l = i / w, t = i - l * w, base = l * 2 * w;
            const ffc g0 = a[base + 2 * t], g1 = a[base + 2 * t + 1];
            b[base + t] = ffc_add(g0, g1);
            b[base + w + t] = ffc_add(ffc_mulc(tw[t], g0), ffc_mulc(tw[t + 1], g1));
        }
        __syncthreads();
        ffc* s = a; a = b; b = s;
    }
}

// J.X: FP32 complex rows; J.roots: the L roots of unity in FP64 (complex128); J.coef: the filter table in FP64
__global__ void __launch_bounds__(FF_THREADS) rows_ff_kernel(const adrt_row_job J, const int total) {
    const int N = 1 << J.n;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ffc* sm = reinterpret_cast<ffc*>(smem_raw);
    ffc* tw = sm;                        // z^t, t = 0 .. N/2
    ffc* bufs[5];
    for (int q = 0; q < 5; ++q) bufs[q] = sm + (N / 2 + 1) + (size_t)q * N;
    const double2* roots = reinterpret_cast<const double2*>(J.roots);
    const double* coefs = reinterpret_cast<const double*>(J.coef);
    const int Lmask = (2 << J.n) - 1;
    const ff tau = ff_from_d(J.tau);
    for (int item = blockIdx.x; item < total; item += gridDim.x) {
        const int sel = item / J.nimg;
        const int img = item - sel * J.nimg;
        const int row = J.rows ? J.rows[sel] : sel;
        const int k = row % J.freq_mod;
        float2* ptr = reinterpret_cast<float2*>(J.X) + (size_t)img * J.img_stride + (size_t)row * N;
        for (int t = threadIdx.x; t <= N / 2; t += blockDim.x) tw[t] = ffc_from_d2(roots[((long)k * t) & Lmask]);
        ffc* cur = bufs[0];
        ffc* tmp = bufs[1];
        for (int i = threadIdx.x; i < N; i += blockDim.x) cur[i] = ffc_from_f2(ptr[i]);
        __syncthreads();
        for (int o = 0; o < J.nops; ++o) {
            const int op = J.op[o], lo = J.lo[o], hi = J.hi[o];
            if (op == ADRT_OP_B) {
                ff_fwd(cur, tmp, N, lo, hi, tw);
            } else if (op == ADRT_OP_BT) {
                ff_adj(cur, tmp, N, lo, hi, tw);
            } else if (op == ADRT_OP_M) {
                ff_fwd(cur, tmp, N, lo, hi, tw);
                ff_adj(cur, tmp, N, lo, hi, tw);
            } else {  // ADRT_OP_P: z_1 = a y; z_{s+1} = z_s + om_a (y - (M + tau) z_s) + om_1 (z_s - z_{s-1})
                ffc* oth[4];
                for (int q = 0, no = 0; q < 5; ++q)
                    if (bufs[q] != cur) oth[no++] = bufs[q];
                const double* cf = coefs + (size_t)k * J.coef_stride;
                const int d = J.deg[k];
                const ff a = ff_from_d(cf[0]);
                ffc* y = cur;
                ffc* z = oth[0];
                ffc* dl = oth[1];  // z_s - z_{s-1}
                for (int i = threadIdx.x; i < N; i += blockDim.x) {
                    z[i] = ffc_scale(a, y[i]);
                    dl[i] = z[i];
                }
                __syncthreads();
                for (int s = 1; s < d; ++s) {
                    const ff om_a = ff_from_d(cf[3 * s - 1]), om_1 = ff_from_d(cf[3 * s]);
                    ffc* pa = oth[2];
                    ffc* pb = oth[3];
                    for (int i = threadIdx.x; i < N; i += blockDim.x) pa[i] = z[i];
                    __syncthreads();
                    ff_fwd(pa, pb, N, lo, hi, tw);
                    ff_adj(pa, pb, N, lo, hi, tw);
                    for (int i = threadIdx.x; i < N; i += blockDim.x) {
                        const ffc r = ffc_sub(ffc_sub(y[i], pa[i]), ffc_scale(tau, z[i]));
                        const ffc dn = ffc_add(ffc_scale(om_1, dl[i]), ffc_scale(om_a, r));
                        dl[i] = dn;
                        z[i] = ffc_add(z[i], dn);
                    }
                    __syncthreads();
                }
                cur = z;
                tmp = dl;
            }
        }
        for (int i = threadIdx.x; i < N; i += blockDim.x) ptr[i] = ffc_to_f2(cur[i]);
        __syncthreads();
    }
}

int rows_ff_run(const adrt_row_job* J, cudaStream_t st) {
    if (!J || J->dtype != ADRT_F32 || J->n < 1 || J->n > 11 || J->nops < 1 || J->nops > ADRT_MAX_OPS || !J->X ||
        !J->roots || J->freq_mod < 1 || J->nimg < 0 || J->nsel < 0) {
        set_error("rows_ff: bad job (FP32 rows, FP64 roots of unity and coefficients required)");
        return ADRT_EINVAL;
    }
    for (int o = 0; o < J->nops; ++o) {
        const int op = J->op[o];
        if (op != ADRT_OP_B && op != ADRT_OP_BT && op != ADRT_OP_M && op != ADRT_OP_P) {
            set_error("rows_ff: bad op %d", op);
            return ADRT_EINVAL;
        }
        if (J->lo[o] < 1 || J->hi[o] > J->n || J->lo[o] > J->hi[o]) {
            set_error("rows_ff: op %d levels [%d, %d] outside 1..%d", o, J->lo[o], J->hi[o], J->n);
            return ADRT_EINVAL;
        }
        if (op == ADRT_OP_P && (!J->deg || !J->coef)) { set_error("rows_ff: P op needs deg and coef"); return ADRT_EINVAL; }
    }
    const long total_l = (long)J->nimg * J->nsel;
    if (total_l <= 0) return ADRT_OK;
    if (total_l > 0x7fffff00L) { set_error("rows_ff: too many work items"); return ADRT_EINVAL; }
    const int N = 1 << J->n;
    const size_t smem = ((size_t)N / 2 + 1 + 5 * (size_t)N) * sizeof(ffc);
    if (int rc = ensure_smem((const void*)rows_ff_kernel, smem)) return rc;
    int per_sm = (int)((227u * 1024u) / smem);
    if (per_sm < 1) per_sm = 1;
    if (per_sm > 8) per_sm = 8;
    long grid = (long)device_sm_count() * per_sm;
    if (grid > total_l) grid = total_l;
    const int threads = N >= 1024 ? FF_THREADS : 256;  // at least two butterflies per thread and level
    rows_ff_kernel<<<(int)grid, threads, smem, st>>>(*J, (int)total_l);
    return launch_status("rows_ff_kernel");
}

}  // namespace adrt

extern "C" int adrt_rows_ff_run(const adrt_row_job* J, void* stream) {
    return adrt::rows_ff_run(J, adrt::as_stream(stream));
}
