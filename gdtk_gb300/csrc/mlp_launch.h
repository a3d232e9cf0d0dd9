// mlp_launch.h -- host launchers of the surrogate network's BF16 tensor-core kernels (mlp_kernels.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace gdtk {

enum { ACT_NONE = 0, ACT_GELU = 1, ACT_GELU_BWD = 2 };

// D[M][N] = alpha * op(A)[M][K] * op(B)[K][N] (+ bias[n]) (+ beta * D), epilogue act:
//   ACT_GELU:     pre <- value (when pre is set), value <- gelu(value)
//   ACT_GELU_BWD: value <- value * gelu'(pre_in)
// op(A) = A[M][lda] row-major (trans_a = 0) or A stored as [K][lda] (trans_a = 1); likewise
// op(B) = B[K][ldb] (trans_b = 0) or B stored as [N][ldb] (trans_b = 1).
// Requirements (checked by the launcher): K % 8 == 0, the feature dimension of every operand a
// multiple of 8 (16-byte vector loads), 16-byte aligned base pointers and leading dimensions.
// splits > 1 partitions K over blockIdx.z; partial tiles go to work[splits][M][N] and a second
// kernel sums them in a fixed order (deterministic), applying alpha/beta (no bias or act).
struct GemmArgs {
    int M = 0, N = 0, K = 0;
    const __nv_bfloat16* A = nullptr;
    int lda = 0, trans_a = 0;
    const __nv_bfloat16* B = nullptr;
    int ldb = 0, trans_b = 0;
    float alpha = 1.f, beta = 0.f;
    const float* bias = nullptr;
    int act = ACT_NONE;
    const float* pre_in = nullptr;   // ACT_GELU_BWD
    float* pre = nullptr;            // ACT_GELU: pre-activation out
    float* D = nullptr;              // fp32 out (may be null)
    __nv_bfloat16* Dh = nullptr;     // bf16 out (may be null)
    int ldd = 0;
    int splits = 1;
    float* work = nullptr;
};

cudaError_t launch_gemm_bf16(const GemmArgs& g, cudaStream_t s);

// The tcgen05 (TMEM-accumulator) form, mlp_tcgen05.cu: taken by launch_gemm_bf16 for D = A W^T (+ bias)
// (GELU) with A [M][K] and W [N][K] K-contiguous, K and N multiples of 16 in 16..256, alpha 1, beta 0,
// no split; cudaErrorNotSupported when those do not hold or it is switched off (GDTK_MLP_TCGEN05=0 in the
// environment, or tcgen05_gemm_set(0)).
bool tcgen05_gemm_eligible(const GemmArgs& g);
bool tcgen05_gemm_enabled();
int tcgen05_gemm_set(int enable);                   // -1 leaves it; returns the previous setting
unsigned long long tcgen05_gemm_launches();         // launches so far in this process
cudaError_t tcgen05_gemm_error(int* error);         // 1/2: a load/MMA wait gave up (read and cleared)
cudaError_t launch_gemm_bf16_tcgen05(const GemmArgs& g, cudaStream_t s);
cudaError_t launch_column_sum(int M, int N, const float* x, float* partial, float* out, cudaStream_t s);
cudaError_t launch_mse_grad(int M, int N, const float* pred, const float* y, const float* w, float* grad,
                            __nv_bfloat16* gradh, float* loss_sum, cudaStream_t s);
cudaError_t launch_adamw(int count, float* w, const float* g, float* m, float* v, __nv_bfloat16* wh, float lr,
                         float beta1, float beta2, float eps, float wd, int step, cudaStream_t s);
cudaError_t launch_cast_bf16(int count, const float* x, __nv_bfloat16* y, cudaStream_t s);
// rows idx[i] (or i when idx is null) of X (fp32 [.][ldx]) -> Xh[i] = bf16((X - xs) / xd), and
// of Y (may be null) -> Yg[i] = (Y - ys) / yd (fp32, width ldy)
cudaError_t launch_gather_rows(int n, const int* idx, const float* X, int ldx, const float* xs, const float* xd,
                               __nv_bfloat16* Xh, const float* Y, int ldy, const float* ys, const float* yd, float* Yg,
                               cudaStream_t s);

// x[i][k] = x[i][k] * scale[k] + shift[k] over n rows of width w
cudaError_t launch_affine_columns(int n, int w, const float* shift, const float* scale, float* x, cudaStream_t s);

// The surrogate's error network: input rows [xh (nin bf16), out (nout fp32 -> bf16)]; targets
// log10 of the larger of the largest raw |dY| error of out against y over the nsp mass fractions
// and T_weight times the relative error of the temperature increment (T = exp(X[rows[r]][0]));
// pinball (quantile tau) loss gradient of column 0; column copy.
cudaError_t launch_error_features(int B, const __nv_bfloat16* xh, int nin, const float* out, int nout,
                                  __nv_bfloat16* feat, cudaStream_t s);
cudaError_t launch_error_targets(int B, const float* out, const float* y, int ld, const float* y_scale, int nsp,
                                 const float* X, const int* rows, int xld, float T_weight, float* tgt, int w,
                                 cudaStream_t s);
cudaError_t launch_pinball_grad(int B, int w, const float* pred, const float* tgt, float tau, float* grad,
                                __nv_bfloat16* gradh, float* loss_sum, cudaStream_t s);
cudaError_t launch_copy_column(int n, const float* x, int ld, int col, float* out, cudaStream_t s);

int column_sum_partials(int M);   // row chunks used by launch_column_sum (partial holds chunks * N floats)

}  // namespace gdtk
