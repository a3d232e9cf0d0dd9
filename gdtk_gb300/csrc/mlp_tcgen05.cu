// mlp_tcgen05.cu -- the surrogate network's forward GEMM on the fifth-generation tensor cores:
//   D[M][N] = A[M][K] W[N][K]^T + bias, then GELU (keeping the pre-activation) or nothing,
// BF16 operands, FP32 accumulation in tensor memory (TMEM), K and N multiples of 16 up to 256.
//
// One persistent CTA of 128 threads per SM.  The CTA loads W once with TMA and keeps it in shared
// memory; for each 128-row tile of A it
//   1. loads the tile with TMA (2-D boxes of 8 elements x rows, which land as the K-major,
//      no-swizzle canonical layout: 8-row x 16-byte core matrices, rows 16 bytes apart, K-groups
//      rows x 16 bytes apart), completion counted in bytes on an mbarrier;
//   2. one thread issues K/16 tcgen05.mma (M = 128, N, K = 16) into an N-column FP32 accumulator
//      and tcgen05.commit arrives on a second mbarrier when they are done;
//   3. each warp reads its 32 TMEM lanes (= rows) with tcgen05.ld 32x32b, adds the bias, applies the
//      activation and stores FP32 and/or BF16 rows.
// Every mbarrier wait is bounded: on timeout the CTA records an error flag, waits (bounded) for
// what it has in flight, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <atomic>
#include <cstdlib>
#include <cstring>

#include "mlp_launch.h"

namespace gdtk {
namespace {

constexpr int TC_M = 128;                           // rows per tile = TMEM lanes
constexpr int EPI_WARPS = 16;                       // epilogue warps: 4 lane quarters x 4 column slices
constexpr int TC_THREADS = 32 * (1 + EPI_WARPS);
constexpr unsigned long long SPIN_LIMIT = 1ull << 22;   // mbarrier polls before a wait gives up

__device__ int g_tc_error;

struct TcArgs {
    int M, N, K;
    int a_bytes, w_bytes;   // shared-memory bytes of one A tile and of W
    unsigned tmem_cols;
    const float* bias;
    int act;
    float* pre;
    float* D;
    __nv_bfloat16* Dh;
    int ldd;
};

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// Waits for the phase of parity `parity` to complete; false if it has not after SPIN_LIMIT polls.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
    const unsigned a = smem_u32(bar);
    for (unsigned long long i = 0; i < SPIN_LIMIT; ++i) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: start address, leading-dimension (K-direction) and stride-dimension
// (M/N-direction) byte offsets between core matrices, descriptor version 1, no swizzle.
__device__ __forceinline__ unsigned long long smem_desc(unsigned addr, unsigned lbo, unsigned sbo) {
    return (unsigned long long)((addr & 0x3FFFFu) >> 4) | (unsigned long long)((lbo >> 4) & 0x3FFFu) << 16 |
           (unsigned long long)((sbo >> 4) & 0x3FFFu) << 32 | 1ull << 46;
}

__device__ __forceinline__ void mma_bf16(unsigned tmem_d, unsigned long long adesc, unsigned long long bdesc,
                                         unsigned idesc, unsigned accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(unsigned long long* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// Starts loading 16 consecutive FP32 columns of this thread's TMEM lane; the values are valid after
// tmem_ld_wait.
__device__ __forceinline__ void tmem_ld16(unsigned taddr, unsigned (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}

// Waits for this thread's TMEM loads; the empty statements after it make every later use of r depend on
// the wait.
template <int Q>
__device__ __forceinline__ void tmem_ld_wait(unsigned (&r)[Q][16]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int q = 0; q < Q; ++q)
#pragma unroll
        for (int i = 0; i < 16; ++i) asm volatile("" : "+r"(r[q][i])::"memory");
}

// GELU, tanh form, as the mma.sync kernel's epilogue: 0.5 x (1 + tanh(u)) = x / (1 + exp(-2u)),
// u = sqrt(2/pi) (x + 0.044715 x^3), with exp2f and __fdividef (each within 2 ulp); exp(-2u) -> inf gives
// -0, exp(-2u) -> 0 gives x.
__device__ __forceinline__ float gelu_tc(float x) {
    const float m2c_log2e = -2.0f * 0.7978845608028654f * 1.4426950408889634f;
    const float e = exp2f(m2c_log2e * (x + 0.044715f * x * x * x));
    return __fdividef(x, 1.0f + e);
}

__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Warp 0 (one lane) loads and issues the MMAs; warps 1..EPI_WARPS drain the accumulators.  Two TMEM
// accumulators alternate between tiles, so that the MMAs of tile i+1 (and the load of its A) run while
// the epilogue warps drain tile i.  Epilogue warp w reads TMEM lanes 32 (w % 4) .. + 31 (the lanes a warp
// may access) and the column slice (w - 1) / 4 of EPI_WARPS / 4 slices.
// Barriers: load (A tile, + W the first time), full[b] (tcgen05.commit of accumulator b), empty[b]
// (every epilogue warp has read accumulator b).
__global__ void __launch_bounds__(TC_THREADS, 1)
    gemm_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmW, const TcArgs g) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* sA = smem;
    unsigned char* sW = smem + g.a_bytes;
    unsigned long long* bars = reinterpret_cast<unsigned long long*>(smem + g.a_bytes + g.w_bytes);
    unsigned long long* bar_load = bars;
    unsigned long long* bar_full = bars + 1;    // [2]
    unsigned long long* bar_empty = bars + 3;   // [2]
    unsigned* tmem_slot = reinterpret_cast<unsigned*>(bars + 5);
    int* s_state = reinterpret_cast<int*>(tmem_slot + 1);   // [0] failed, [1] commits issued
    float* s_bias = reinterpret_cast<float*>(bars + 8);       // [N]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int k = threadIdx.x; k < g.N; k += blockDim.x) s_bias[k] = g.bias ? g.bias[k] : 0.f;

    if (threadIdx.x == 0) {
        mbar_init(bar_load, 1);
        mbar_init(&bar_full[0], 1);
        mbar_init(&bar_full[1], 1);
        mbar_init(&bar_empty[0], EPI_WARPS);
        mbar_init(&bar_empty[1], EPI_WARPS);
        s_state[0] = 0;
        s_state[1] = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(2 * g.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = *tmem_slot;
    const int ntiles = (g.M + TC_M - 1) / TC_M;
    const int my_tiles = blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;

    if (warp == 0) {
        if (lane == 0) {
            // instruction descriptor: FP32 accumulator, BF16 A and B, both K-major, N >> 3, M >> 4
            const unsigned idesc =
                (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(g.N >> 3) << 17) | ((unsigned)(TC_M >> 4) << 24);
            const unsigned a_lbo = TC_M * 16, w_lbo = (unsigned)g.N * 16;   // bytes between K-groups
            const int kgroups = g.K / 8;
            int failed = 0, commits = 0;
            unsigned load_parity = 0;
            for (int i = 0; i < my_tiles && !failed; ++i) {
                const int tile = blockIdx.x + i * gridDim.x, b = i & 1;
                // A is free once the previous tile's MMAs are done (its commit)
                if (i > 0 && !mbar_wait(&bar_full[(i - 1) & 1], ((i - 1) >> 1) & 1)) { failed = 2; break; }
                mbar_expect_tx(bar_load, (unsigned)(g.a_bytes + (i == 0 ? g.w_bytes : 0)));
                for (int kg = 0; kg < kgroups; ++kg) tma_load_2d(sA + kg * a_lbo, &tmA, kg * 8, tile * TC_M, bar_load);
                if (i == 0)
                    for (int kg = 0; kg < kgroups; ++kg) tma_load_2d(sW + kg * w_lbo, &tmW, kg * 8, 0, bar_load);
                load_parity = i & 1;
                if (!mbar_wait(bar_load, load_parity)) { failed = 1; break; }
                // accumulator b is free once the epilogue has drained its previous tile
                if (i >= 2 && !mbar_wait(&bar_empty[b], ((i >> 1) - 1) & 1)) { failed = 3; break; }
                tc_fence_after();
                const unsigned acc = tmem + (unsigned)b * g.tmem_cols;
                for (int ks = 0; ks < g.K / 16; ++ks) {   // one K = 16 step covers two K-groups
                    const unsigned long long ad = smem_desc(smem_u32(sA) + 2u * ks * a_lbo, a_lbo, 128);
                    const unsigned long long bd = smem_desc(smem_u32(sW) + 2u * ks * w_lbo, w_lbo, 128);
                    mma_bf16(acc, ad, bd, idesc, ks > 0 ? 1u : 0u);
                }
                mma_commit(&bar_full[b]);
                ++commits;
            }
            s_state[1] = commits;
            if (failed) {
                atomicExch(&g_tc_error, failed);
                s_state[0] = 1;
                if (failed == 1) mbar_wait(bar_load, load_parity);   // bounded: the loads still in flight
            }
        }
    } else if (warp <= EPI_WARPS) {
        const int quarter = warp & 3, slice = (warp - 1) >> 2, slices = EPI_WARPS / 4;
        const int chunks = g.N / 16;   // 16-column chunks; this warp's are [slice, slice + 1) x chunks / slices
        const int c0 = 16 * (slice * chunks / slices), c1 = 16 * ((slice + 1) * chunks / slices);
        for (int i = 0; i < my_tiles; ++i) {
            const int tile = blockIdx.x + i * gridDim.x, b = i & 1;
            if (!mbar_wait(&bar_full[b], (i >> 1) & 1)) {
                if (lane == 0) atomicExch(&g_tc_error, 4);
                break;
            }
            tc_fence_after();
            const int row = tile * TC_M + quarter * 32 + lane;
            const unsigned trow = tmem + (unsigned)b * g.tmem_cols + ((unsigned)(quarter * 32) << 16);
            const int nq = (c1 - c0) >> 4;   // at most 4: N <= 256 over 4 column slices
            for (int qb = 0; qb < nq; qb += 2) {   // two 16-column chunks in flight per wait
                unsigned r[2][16];
                __syncwarp();   // the TMEM loads are warp-collective
                tmem_ld16(trow + (unsigned)(c0 + 16 * qb), r[0]);
                if (qb + 1 < nq) tmem_ld16(trow + (unsigned)(c0 + 16 * qb + 16), r[1]);
                tmem_ld_wait<2>(r);
                if (row >= g.M) continue;
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    if (qb + q >= nq) break;
                    const int c = c0 + 16 * (qb + q);
                    const size_t o = (size_t)row * g.ldd + c;
                    float v[16];
#pragma unroll
                    for (int k = 0; k < 16; ++k) {
                        v[k] = __uint_as_float(r[q][k]) + s_bias[c + k];
                        if (g.act == ACT_GELU) {
                            if (g.pre) g.pre[o + k] = v[k];
                            v[k] = gelu_tc(v[k]);
                        }
                    }
                    if (g.D) {
                        float4* d4 = reinterpret_cast<float4*>(g.D + o);
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                            d4[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
                    }
                    if (g.Dh) {
                        __align__(16) __nv_bfloat16 h[16];
#pragma unroll
                        for (int k = 0; k < 16; ++k) h[k] = __float2bfloat16(v[k]);
                        uint4* d = reinterpret_cast<uint4*>(g.Dh + o);
                        d[0] = reinterpret_cast<const uint4*>(h)[0];
                        d[1] = reinterpret_cast<const uint4*>(h)[1];
                    }
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&bar_empty[b]);
        }
    }
    __syncthreads();
    if (s_state[0] && threadIdx.x == 0 && s_state[1] > 0) {   // bounded wait for the last commit before freeing TMEM
        const int last = s_state[1] - 1;
        mbar_wait(&bar_full[last & 1], (last >> 1) & 1);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * g.tmem_cols)
                     : "memory");
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

// [rows][K] BF16 row-major with leading dimension ld, boxes of 8 elements x box_rows
bool encode(CUtensorMap* map, const void* base, int K, int rows, int ld, int box_rows) {
    auto fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dim[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    cuuint64_t stride[1] = {(cuuint64_t)ld * 2};
    cuuint32_t box[2] = {8u, (cuuint32_t)box_rows};
    cuuint32_t estride[2] = {1u, 1u};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dim, stride, box, estride,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

std::atomic<int> g_enabled{-1};                // -1: from the environment on first use
std::atomic<unsigned long long> g_launches{0};

bool aligned16(const void* p) { return ((unsigned long long)p & 15u) == 0; }

}  // namespace

bool tcgen05_gemm_enabled() {
    int e = g_enabled.load();
    if (e < 0) {
        const char* v = std::getenv("GDTK_MLP_TCGEN05");
        e = (v && std::strcmp(v, "0") == 0) ? 0 : 1;
        g_enabled.store(e);
    }
    return e != 0;
}

int tcgen05_gemm_set(int enable) {
    const int prev = tcgen05_gemm_enabled() ? 1 : 0;
    if (enable >= 0) g_enabled.store(enable ? 1 : 0);
    return prev;
}

unsigned long long tcgen05_gemm_launches() { return g_launches.load(); }

cudaError_t tcgen05_gemm_error(int* error) {
    int zero = 0;
    cudaError_t e = cudaMemcpyFromSymbol(error, g_tc_error, sizeof(int));
    if (e != cudaSuccess) return e;
    return cudaMemcpyToSymbol(g_tc_error, &zero, sizeof(int));
}

bool tcgen05_gemm_eligible(const GemmArgs& g) {
    return !g.trans_a && g.trans_b && g.alpha == 1.f && g.beta == 0.f && g.splits == 1 &&
           (g.act == ACT_NONE || g.act == ACT_GELU) && g.K % 16 == 0 && g.K >= 16 && g.K <= 256 && g.N % 16 == 0 &&
           g.N >= 16 && g.N <= 256 && g.M >= 1 && g.lda % 8 == 0 && g.ldb % 8 == 0 && g.ldd % 8 == 0 &&
           aligned16(g.A) && aligned16(g.B) && (!g.D || aligned16(g.D)) && (!g.Dh || aligned16(g.Dh)) &&
           (!g.pre || aligned16(g.pre)) && (g.D || g.Dh || g.pre);
}

// The tcgen05 form of launch_gemm_bf16 for the shapes tcgen05_gemm_eligible accepts;
// cudaErrorNotSupported when it does not apply (the caller then uses the mma.sync kernel).
cudaError_t launch_gemm_bf16_tcgen05(const GemmArgs& g, cudaStream_t s) {
    if (!tcgen05_gemm_enabled() || !tcgen05_gemm_eligible(g)) return cudaErrorNotSupported;
    alignas(64) CUtensorMap ma, mw;
    if (!encode(&ma, g.A, g.K, g.M, g.lda, TC_M) || !encode(&mw, g.B, g.K, g.N, g.ldb, g.N))
        return cudaErrorNotSupported;
    TcArgs a{};
    a.M = g.M; a.N = g.N; a.K = g.K;
    a.a_bytes = TC_M * g.K * 2;
    a.w_bytes = g.N * g.K * 2;
    unsigned cols = 32;
    while (cols < (unsigned)g.N) cols <<= 1;
    a.tmem_cols = cols;
    a.bias = g.bias; a.act = g.act; a.pre = g.pre; a.D = g.D; a.Dh = g.Dh; a.ldd = g.ldd;
    // at least 64 KB: whatever the operand sizes, every core matrix an MMA of this kernel addresses lies
    // inside the allocation
    size_t smem = (size_t)a.a_bytes + a.w_bytes + 64 + (size_t)g.N * 4;   // operands, barriers and state, bias
    if (smem < 64 * 1024) smem = 64 * 1024;
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms < 1) sms = 1;
    }
    cudaError_t e = cudaFuncSetAttribute(gemm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int ntiles = (g.M + TC_M - 1) / TC_M;
    const int grid = ntiles < sms ? ntiles : sms;
    gemm_tc_kernel<<<grid, TC_THREADS, smem, s>>>(ma, mw, a);
    e = cudaGetLastError();
    if (e == cudaSuccess) g_launches.fetch_add(1);
    return e;
}

}  // namespace gdtk
