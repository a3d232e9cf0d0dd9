// mlp_kernels.cu -- BF16 tensor-core kernels of the chemistry surrogate, a multilayer perceptron
// that predicts a cell's mass-fraction and temperature increments over an update interval.
// There is no counterpart in the reference; the network, its training and its use are this
// engine's own.
//
//   gemm:  D = alpha * op(A) * op(B) (+ bias) (+ beta * D), BF16 operands, FP32 accumulation,
//          mma.sync.m16n8k16 on 128x64x32 block tiles fed by a 3-stage cp.async pipeline, fragments
//          by ldmatrix (.trans for row-contiguous operands); epilogues: GELU (keeping the
//          pre-activation), GELU backward; split-K with a fixed-order reduction for the weight
//          gradients (K = batch).
//   column sums (bias gradients), weighted squared-error gradient, AdamW, row gather, casts.
//
// The network's GEMMs are small (K, N <= 256): a training step over 8192 samples is about
// 10 GFLOP, and inference over a million cells about 0.4 TFLOP, far below the FP64 cost of
// the integrations it replaces.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "mlp_launch.h"

namespace gdtk {
namespace {

constexpr int BM = 128, BN = 64, BK = 32, STAGES = 3, THREADS = 256;
constexpr int PADH = 8;   // bf16 padding per shared-memory row: rows of 80 or 272 bytes, conflict-free ldmatrix

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// 16-byte global -> shared copy; src_bytes = 0 fills the destination with zeros (out-of-range chunks)
__device__ __forceinline__ void cp_async16(void* dst, const void* src, int src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_addr(dst)), "l"(src), "r"(src_bytes));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void* p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(smem_addr(p)));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], const void* p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(smem_addr(p)));
}

// GELU, tanh form: 0.5 x (1 + tanh(u)), u = sqrt(2/pi) (x + 0.044715 x^3), evaluated as
// x / (1 + exp(-2u)) (the tcgen05 kernel's epilogue uses the same expression), and its derivative.
__device__ __forceinline__ float gelu_f(float x) {
    const float m2c_log2e = -2.0f * 0.7978845608028654f * 1.4426950408889634f;
    const float e = exp2f(m2c_log2e * (x + 0.044715f * x * x * x));
    return __fdividef(x, 1.0f + e);
}
__device__ __forceinline__ float gelu_grad(float x) {
    const float c = 0.7978845608028654f;
    const float x2 = x * x;
    const float t = tanhf(c * (x + 0.044715f * x2 * x));
    return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * c * (1.0f + 3.0f * 0.044715f * x2);
}

// One pipeline stage of an operand tile: ROWS (M or N) x BK (k).  K-contiguous operands are kept
// [ROWS][BK + PADH]; row-contiguous ones [BK][ROWS + PADH] and read back with ldmatrix.trans.
template <int ROWS, bool KCONTIG>
struct Tile {
    static constexpr int ELEMS = KCONTIG ? ROWS * (BK + PADH) : BK * (ROWS + PADH);
};

// Issue the cp.async copies of one operand tile: rows [r0, r0 + ROWS) of op(X), k in [k0, k0 + BK)
// clipped to kend.  Chunks of 8 bf16 along the contiguous dimension; out-of-range chunks read zeros.
template <int ROWS, bool KCONTIG>
__device__ __forceinline__ void load_tile(__nv_bfloat16* S, const __nv_bfloat16* X, int ld, int r0, int rows, int k0,
                                          int kend, int tid) {
    constexpr int CHUNKS = ROWS * BK / 8;
#pragma unroll
    for (int it = 0; it < (CHUNKS + THREADS - 1) / THREADS; ++it) {
        const int idx = tid + it * THREADS;
        if (idx >= CHUNKS) break;
        if (KCONTIG) {   // X[r][k]
            const int rr = idx / (BK / 8), kc = (idx % (BK / 8)) * 8;
            const int r = r0 + rr, k = k0 + kc;
            const bool in = r < rows && k < kend;
            cp_async16(S + rr * (BK + PADH) + kc, in ? X + (size_t)r * ld + k : X, in ? 16 : 0);
        } else {         // X[k][r]
            const int kk = idx / (ROWS / 8), rc = (idx % (ROWS / 8)) * 8;
            const int k = k0 + kk, r = r0 + rc;
            const bool in = k < kend && r < rows;
            cp_async16(S + kk * (ROWS + PADH) + rc, in ? X + (size_t)k * ld + r : X, in ? 16 : 0);
        }
    }
}

// 256 threads = 8 warps in 4 (M) x 2 (N); each warp computes 32 x 32 (2 m16 x 4 n8 mma tiles).
// A 3-stage cp.async pipeline feeds shared memory; fragments are loaded with ldmatrix (.trans for
// row-contiguous operands).
template <bool AK, bool BKC>
__global__ void __launch_bounds__(THREADS) gemm_bf16_kernel(const GemmArgs g) {
    __shared__ __align__(128) __nv_bfloat16 As[STAGES][Tile<BM, AK>::ELEMS];
    __shared__ __align__(128) __nv_bfloat16 Bs[STAGES][Tile<BN, BKC>::ELEMS];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const int gid = lane >> 2, tig = lane & 3;
    const int q = lane >> 3, r8 = lane & 7;
    // this block's K range (split-K over blockIdx.z, in BK multiples)
    const int kper = ((g.K + g.splits - 1) / g.splits + BK - 1) / BK * BK;
    const int kbeg = blockIdx.z * kper;
    const int kend = min(g.K, kbeg + kper);
    const int nk = kend > kbeg ? (kend - kbeg + BK - 1) / BK : 0;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;

#pragma unroll
    for (int st = 0; st < STAGES - 1; ++st) {
        if (st < nk) {
            load_tile<BM, AK>(As[st], g.A, g.lda, m0, g.M, kbeg + st * BK, kend, tid);
            load_tile<BN, BKC>(Bs[st], g.B, g.ldb, n0, g.N, kbeg + st * BK, kend, tid);
        }
        cp_async_commit();
    }
    for (int kt = 0; kt < nk; ++kt) {
        cp_async_wait<STAGES - 2>();
        __syncthreads();
        const __nv_bfloat16* A_ = As[kt % STAGES];
        const __nv_bfloat16* B_ = Bs[kt % STAGES];
#pragma unroll
        for (int ks = 0; ks < BK; ks += 16) {
            uint32_t a[2][4], b[4][2];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int mb = wm + i * 16;
                if (AK) ldsm_x4(a[i], A_ + (mb + (lane & 15)) * (BK + PADH) + ks + ((lane >> 4) << 3));
                else ldsm_x4_t(a[i], A_ + (ks + r8 + ((q >> 1) << 3)) * (BM + PADH) + mb + ((q & 1) << 3));
            }
#pragma unroll
            for (int j = 0; j < 4; j += 2) {
                const int nb = wn + j * 8;
                uint32_t t[4];
                if (BKC) ldsm_x4(t, B_ + (nb + r8 + ((q >> 1) << 3)) * (BK + PADH) + ks + ((q & 1) << 3));
                else ldsm_x4_t(t, B_ + (ks + r8 + ((q & 1) << 3)) * (BN + PADH) + nb + ((q >> 1) << 3));
                b[j][0] = t[0]; b[j][1] = t[1]; b[j + 1][0] = t[2]; b[j + 1][1] = t[3];
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], a[i], b[j]);
        }
        const int nxt = kt + STAGES - 1;
        if (nxt < nk) {
            load_tile<BM, AK>(As[nxt % STAGES], g.A, g.lda, m0, g.M, kbeg + nxt * BK, kend, tid);
            load_tile<BN, BKC>(Bs[nxt % STAGES], g.B, g.ldb, n0, g.N, kbeg + nxt * BK, kend, tid);
        }
        cp_async_commit();
    }
    cp_async_wait<0>();

#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int m = m0 + wm + i * 16 + gid + (r >= 2 ? 8 : 0);
                const int n = n0 + wn + j * 8 + 2 * tig + (r & 1);
                if (m >= g.M || n >= g.N) continue;
                if (g.splits > 1) {   // raw partial; the reduction applies alpha and beta
                    g.work[((size_t)blockIdx.z * g.M + m) * g.N + n] = acc[i][j][r];
                    continue;
                }
                const size_t o = (size_t)m * g.ldd + n;
                float v = g.alpha * acc[i][j][r];
                if (g.bias) v += g.bias[n];
                if (g.beta != 0.f) v += g.beta * g.D[o];
                if (g.act == ACT_GELU) {
                    if (g.pre) g.pre[o] = v;
                    v = gelu_f(v);
                } else if (g.act == ACT_GELU_BWD) {
                    v *= gelu_grad(g.pre_in[o]);
                }
                if (g.D) g.D[o] = v;
                if (g.Dh) g.Dh[o] = __float2bfloat16(v);
            }
}

// D[m][n] = alpha * sum_z work[z][m][n] (+ beta * D), z ascending.
__global__ void splitk_reduce_kernel(int M, int N, int splits, const float* work, float alpha, float beta, float* D,
                                     int ldd) {
    const size_t MN = (size_t)M * N;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < MN; i += (size_t)gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int z = 0; z < splits; ++z) s += work[z * MN + i];
        const size_t o = (i / N) * ldd + i % N;
        float v = alpha * s;
        if (beta != 0.f) v += beta * D[o];
        D[o] = v;
    }
}

// Column sums of x[M][N]: block b sums rows [b*CH, (b+1)*CH) into partial[b][n]; then a single
// pass adds the partials in ascending b (fixed order).
constexpr int COLSUM_ROWS = 256;

__global__ void column_partial_kernel(int M, int N, const float* x, float* partial) {
    const int r0 = blockIdx.x * COLSUM_ROWS, r1 = min(M, r0 + COLSUM_ROWS);
    for (int n = threadIdx.x; n < N; n += blockDim.x) {
        float s = 0.f;
        for (int r = r0; r < r1; ++r) s += x[(size_t)r * N + n];
        partial[(size_t)blockIdx.x * N + n] = s;
    }
}

__global__ void column_final_kernel(int chunks, int N, const float* partial, float* out) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0.f;
    for (int b = 0; b < chunks; ++b) s += partial[(size_t)b * N + n];
    out[n] = s;
}

// Weighted squared error over M rows: loss_sum += sum_n w[n] (pred - y)^2 and
// grad = 2 w[n] (pred - y) / M (fp32 and bf16 copies).
__global__ void mse_grad_kernel(int M, int N, const float* pred, const float* y, const float* w, float* grad,
                                __nv_bfloat16* gradh, float* loss_sum) {
    float local = 0.f;
    const size_t total = (size_t)M * N;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int n = (int)(i % N);
        const float wt = w ? w[n] : 1.f;
        const float d = pred[i] - y[i];
        const float gv = 2.f * wt * d / (float)M;
        if (grad) grad[i] = gv;
        if (gradh) gradh[i] = __float2bfloat16(gv);
        local += wt * d * d;
    }
    if (loss_sum) {
        for (int off = 16; off > 0; off >>= 1) local += __shfl_down_sync(0xffffffffu, local, off);
        if ((threadIdx.x & 31) == 0) atomicAdd(loss_sum, local);
    }
}

// AdamW (decoupled weight decay) on fp32 master weights; refreshes the bf16 copy.
__global__ void adamw_kernel(int count, float* w, const float* g, float* m, float* v, __nv_bfloat16* wh, float lr,
                             float beta1, float beta2, float eps, float wd, float bc1, float bc2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = beta1 * m[i] + (1.f - beta1) * gi;
        const float vi = beta2 * v[i] + (1.f - beta2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        float wi = w[i] * (1.f - lr * wd);
        wi -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
        w[i] = wi;
        if (wh) wh[i] = __float2bfloat16(wi);
    }
}

__global__ void cast_bf16_kernel(int count, const float* x, __nv_bfloat16* y) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
        y[i] = __float2bfloat16(x[i]);
}

// Row idx[r] of X and Y, standardised: Xh[r][c] = bf16((X - xs) / xd), Yg[r][c] = (Y - ys) / yd.
__global__ void gather_rows_kernel(int n, const int* idx, const float* X, int ldx, const float* xs, const float* xd,
                                   __nv_bfloat16* Xh, const float* Y, int ldy, const float* ys, const float* yd,
                                   float* Yg) {
    const int w = ldx + ldy;
    const size_t total = (size_t)n * w;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(i / w), c = (int)(i % w);
        const size_t src = idx ? (size_t)idx[r] : (size_t)r;
        if (c < ldx) {
            Xh[(size_t)r * ldx + c] = __float2bfloat16((X[src * ldx + c] - xs[c]) / xd[c]);
        } else if (Y) {
            const int k = c - ldx;
            Yg[(size_t)r * ldy + k] = (Y[src * ldy + k] - ys[k]) / yd[k];
        }
    }
}

__global__ void affine_columns_kernel(int n, int w, const float* shift, const float* scale, float* x) {
    const size_t total = (size_t)n * w;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(i % w);
        x[i] = x[i] * scale[k] + shift[k];
    }
}

// feat[r] = [xh[r][0..nin), bf16(out[r][0..nout))]: the error network's input
__global__ void error_features_kernel(int B, const __nv_bfloat16* xh, int nin, const float* out, int nout,
                                      __nv_bfloat16* feat) {
    const int w = nin + nout;
    const size_t total = (size_t)B * w;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const size_t r = i / w;
        const int c = (int)(i % w);
        feat[i] = c < nin ? xh[r * nin + c] : __float2bfloat16(out[r * nout + (c - nin)]);
    }
}

// tgt[r][0] = log10(e + 1e-12), e = max(max_s |(out[r][s] - y[r][s]) y_scale[s]|, T_weight |dT error| / T):
// the raw-unit error of the standardised prediction out against the target y over the nsp mass
// fractions, and the temperature increment's error (output nsp) relative to the sample's T =
// exp(X[rows[r]][0]) weighted by T_weight (0.1 makes a relative T error of 1e-3 count as a mass-
// fraction error of 1e-4).  Other columns of the w-wide row are zero.
__global__ void error_targets_kernel(int B, const float* out, const float* y, int ld, const float* y_scale, int nsp,
                                     const float* X, const int* rows, int xld, float T_weight, float* tgt, int w) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < B; r += gridDim.x * blockDim.x) {
        float e = 0.f;
        for (int k = 0; k < nsp; ++k) e = fmaxf(e, fabsf((out[(size_t)r * ld + k] - y[(size_t)r * ld + k]) * y_scale[k]));
        const size_t row = rows ? (size_t)rows[r] : (size_t)r;
        const float T = expf(X[row * xld]);
        const float eT = fabsf((out[(size_t)r * ld + nsp] - y[(size_t)r * ld + nsp]) * y_scale[nsp]) / T;
        e = fmaxf(e, T_weight * eT);
        tgt[(size_t)r * w] = log10f(e + 1e-12f);
        for (int c = 1; c < w; ++c) tgt[(size_t)r * w + c] = 0.f;
    }
}

// Pinball (quantile) loss of column 0 of pred[B][w] against tgt: loss_sum += max(tau r, (tau - 1) r),
// r = tgt - pred; grad = d(mean loss)/d pred = (r > 0 ? -tau : 1 - tau) / B (other columns 0).
__global__ void pinball_grad_kernel(int B, int w, const float* pred, const float* tgt, float tau, float* grad,
                                    __nv_bfloat16* gradh, float* loss_sum) {
    float local = 0.f;
    const size_t total = (size_t)B * w;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        float gv = 0.f;
        if (i % w == 0) {
            const float r = tgt[i] - pred[i];
            local += r > 0.f ? tau * r : (tau - 1.f) * r;
            gv = (r > 0.f ? -tau : 1.f - tau) / (float)B;
        }
        grad[i] = gv;
        gradh[i] = __float2bfloat16(gv);
    }
    if (loss_sum) {
        for (int off = 16; off > 0; off >>= 1) local += __shfl_down_sync(0xffffffffu, local, off);
        if ((threadIdx.x & 31) == 0) atomicAdd(loss_sum, local);
    }
}

__global__ void copy_column_kernel(int n, const float* x, int ld, int col, float* out) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) out[r] = x[(size_t)r * ld + col];
}

int grid_for(size_t count) {
    size_t g = (count + 255) / 256;
    return (int)(g > 8192 ? 8192 : (g < 1 ? 1 : g));
}

bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

}  // namespace

cudaError_t launch_gemm_bf16(const GemmArgs& g, cudaStream_t s) {
    if (g.M <= 0 || g.N <= 0 || g.K <= 0) return cudaSuccess;
    if (tcgen05_gemm_eligible(g)) {   // the forward shapes: fifth-generation tensor cores
        const cudaError_t e = launch_gemm_bf16_tcgen05(g, s);
        if (e != cudaErrorNotSupported) return e;
    }
    // 16-byte chunks along the contiguous dimension of each operand
    const int a_inner = g.trans_a ? g.M : g.K, b_inner = g.trans_b ? g.K : g.N;
    if (g.K % 8 || a_inner % 8 || b_inner % 8 || g.lda % 8 || g.ldb % 8 || !aligned16(g.A) || !aligned16(g.B))
        return cudaErrorInvalidValue;
    if (g.splits < 1 || (g.splits > 1 && (!g.work || g.bias || g.act != ACT_NONE || !g.D || g.Dh)))
        return cudaErrorInvalidValue;
    if ((g.act == ACT_GELU_BWD && !g.pre_in) || (g.beta != 0.f && !g.D))
        return cudaErrorInvalidValue;
    dim3 grid((g.N + BN - 1) / BN, (g.M + BM - 1) / BM, g.splits);
    if (grid.y > 65535u || grid.z > 65535u) return cudaErrorInvalidConfiguration;
    const bool ak = !g.trans_a, bk = g.trans_b != 0;   // K-contiguous operands
    if (ak && bk) gemm_bf16_kernel<true, true><<<grid, THREADS, 0, s>>>(g);
    else if (ak) gemm_bf16_kernel<true, false><<<grid, THREADS, 0, s>>>(g);
    else if (bk) gemm_bf16_kernel<false, true><<<grid, THREADS, 0, s>>>(g);
    else gemm_bf16_kernel<false, false><<<grid, THREADS, 0, s>>>(g);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || g.splits == 1) return e;
    splitk_reduce_kernel<<<grid_for((size_t)g.M * g.N), 256, 0, s>>>(g.M, g.N, g.splits, g.work, g.alpha, g.beta, g.D,
                                                                      g.ldd);
    return cudaGetLastError();
}

int column_sum_partials(int M) { return (M + COLSUM_ROWS - 1) / COLSUM_ROWS; }

cudaError_t launch_column_sum(int M, int N, const float* x, float* partial, float* out, cudaStream_t s) {
    if (M <= 0 || N <= 0) return cudaSuccess;
    const int chunks = column_sum_partials(M);
    column_partial_kernel<<<chunks, N < 256 ? ((N + 31) / 32) * 32 : 256, 0, s>>>(M, N, x, partial);
    column_final_kernel<<<(N + 127) / 128, 128, 0, s>>>(chunks, N, partial, out);
    return cudaGetLastError();
}

cudaError_t launch_mse_grad(int M, int N, const float* pred, const float* y, const float* w, float* grad,
                            __nv_bfloat16* gradh, float* loss_sum, cudaStream_t s) {
    if (M <= 0 || N <= 0) return cudaSuccess;
    mse_grad_kernel<<<grid_for((size_t)M * N), 256, 0, s>>>(M, N, pred, y, w, grad, gradh, loss_sum);
    return cudaGetLastError();
}

cudaError_t launch_adamw(int count, float* w, const float* g, float* m, float* v, __nv_bfloat16* wh, float lr,
                         float beta1, float beta2, float eps, float wd, int step, cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    const float bc1 = 1.f - powf(beta1, (float)step), bc2 = 1.f - powf(beta2, (float)step);
    adamw_kernel<<<grid_for((size_t)count), 256, 0, s>>>(count, w, g, m, v, wh, lr, beta1, beta2, eps, wd, bc1, bc2);
    return cudaGetLastError();
}

cudaError_t launch_cast_bf16(int count, const float* x, __nv_bfloat16* y, cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    cast_bf16_kernel<<<grid_for((size_t)count), 256, 0, s>>>(count, x, y);
    return cudaGetLastError();
}

cudaError_t launch_gather_rows(int n, const int* idx, const float* X, int ldx, const float* xs, const float* xd,
                               __nv_bfloat16* Xh, const float* Y, int ldy, const float* ys, const float* yd, float* Yg,
                               cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int w = ldx + (Y ? ldy : 0);
    gather_rows_kernel<<<grid_for((size_t)n * w), 256, 0, s>>>(n, idx, X, ldx, xs, xd, Xh, Y, Y ? ldy : 0, ys, yd,
                                                               Yg);
    return cudaGetLastError();
}

cudaError_t launch_affine_columns(int n, int w, const float* shift, const float* scale, float* x, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    affine_columns_kernel<<<grid_for((size_t)n * w), 256, 0, s>>>(n, w, shift, scale, x);
    return cudaGetLastError();
}

cudaError_t launch_error_features(int B, const __nv_bfloat16* xh, int nin, const float* out, int nout,
                                  __nv_bfloat16* feat, cudaStream_t s) {
    if (B <= 0) return cudaSuccess;
    error_features_kernel<<<grid_for((size_t)B * (nin + nout)), 256, 0, s>>>(B, xh, nin, out, nout, feat);
    return cudaGetLastError();
}

cudaError_t launch_error_targets(int B, const float* out, const float* y, int ld, const float* y_scale, int nsp,
                                 const float* X, const int* rows, int xld, float T_weight, float* tgt, int w,
                                 cudaStream_t s) {
    if (B <= 0) return cudaSuccess;
    error_targets_kernel<<<grid_for((size_t)B), 256, 0, s>>>(B, out, y, ld, y_scale, nsp, X, rows, xld, T_weight, tgt,
                                                             w);
    return cudaGetLastError();
}

cudaError_t launch_pinball_grad(int B, int w, const float* pred, const float* tgt, float tau, float* grad,
                                __nv_bfloat16* gradh, float* loss_sum, cudaStream_t s) {
    if (B <= 0) return cudaSuccess;
    pinball_grad_kernel<<<grid_for((size_t)B * w), 256, 0, s>>>(B, w, pred, tgt, tau, grad, gradh, loss_sum);
    return cudaGetLastError();
}

cudaError_t launch_copy_column(int n, const float* x, int ld, int col, float* out, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    copy_column_kernel<<<grid_for((size_t)n), 256, 0, s>>>(n, x, ld, col, out);
    return cudaGetLastError();
}

}  // namespace gdtk
