// surrogate.cpp -- the chemistry surrogate of include/gdtk_surrogate.h: network state, training
// step (forward, backward, AdamW on the kernels of mlp_kernels.cu), and the gated update with
// FP64 fallback (surrogate_kernels.cu + the plain update of chem_api.cpp).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/gdtk_chem.h"
#include "../../include/gdtk_surrogate.h"
#include "api_internal.h"
#include "mlp_launch.h"
#include "surrogate_launch.h"

namespace gdtk {
namespace {

// Weight of the relative temperature-increment error in the error network's target (a relative T error
// of 1e-3 counts as a mass-fraction error of 1e-4, the two accuracy bars of the surrogate).
constexpr float kErrorTWeight = 0.1f;

static_assert(GDTK_GATE_COUNT == GATE_COUNT, "gate codes");

void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename T>
struct Buf {
    T* p = nullptr;
    size_t n = 0;
    T* ensure(size_t want) {
        if (want > n) {
            if (p) cudaFree(p);
            p = nullptr;
            n = 0;
            ck(cudaMalloc(&p, std::max<size_t>(want, 1) * sizeof(T)), "cudaMalloc");
            n = want;
        }
        return p;
    }
    ~Buf() { if (p) cudaFree(p); }
};

// standard atomic weights (kg/mol) of the elements a prep-gas species record may name
double atomic_mass(const std::string& e) {
    static const std::map<std::string, double> W = {
        {"H", 1.00794e-3}, {"He", 4.002602e-3}, {"C", 12.0107e-3}, {"N", 14.0067e-3}, {"O", 15.9994e-3},
        {"F", 18.9984032e-3}, {"Ne", 20.1797e-3}, {"Na", 22.98976928e-3}, {"S", 32.065e-3}, {"Cl", 35.453e-3},
        {"Ar", 39.948e-3}, {"Kr", 83.798e-3}, {"Xe", 131.293e-3}, {"Si", 28.0855e-3}, {"B", 10.811e-3}};
    auto it = W.find(e);
    if (it == W.end()) throw std::runtime_error("surrogate: no atomic mass for element '" + e + "'");
    return it->second;
}

int pad8(int n) { return (n + 7) / 8 * 8; }

void gemm(int M, int N, int K, const __nv_bfloat16* A, int lda, int ta, const __nv_bfloat16* B, int ldb, int tb,
          const float* bias, int act, const float* pre_in, float* pre, float* D, __nv_bfloat16* Dh, int ldd,
          cudaStream_t s, int splits = 1, float* work = nullptr) {
    GemmArgs g;
    g.M = M; g.N = N; g.K = K;
    g.A = A; g.lda = lda; g.trans_a = ta;
    g.B = B; g.ldb = ldb; g.trans_b = tb;
    g.bias = bias; g.act = act; g.pre_in = pre_in; g.pre = pre;
    g.D = D; g.Dh = Dh; g.ldd = ldd;
    g.splits = splits; g.work = work;
    ck(launch_gemm_bf16(g, s), "surrogate GEMM");
}

// A multilayer perceptron: nin_pad -> depth x width (GELU) -> nout_pad, BF16 weights and
// activations, FP32 master parameters and AdamW moments.  Parameters are one flat array:
// W_0 .. W_depth (row-major [fan_out][fan_in]), then b_0 .. b_depth.
struct Mlp {
    int nin = 0, nout = 0, nin_pad = 0, nout_pad = 0, width = 0, depth = 0;
    std::vector<int> dims;   // d_0 = nin_pad, d_1..d_depth = width, d_{depth+1} = nout_pad
    std::vector<size_t> w_off, b_off;
    size_t n_params = 0, n_weights = 0;
    Buf<float> params, grad, adam_m, adam_v;
    Buf<__nv_bfloat16> params_h;
    int step = 0;
    int tb = 0;   // training buffers, for batches up to tb rows
    Buf<__nv_bfloat16> t_act, t_g16a, t_g16b, t_dout16;
    Buf<float> t_pre, t_out, t_dout, t_dpre, t_work, t_colpart;
    int ib = 0;   // inference buffers, for chunks up to ib rows
    Buf<__nv_bfloat16> i_a0, i_a1;

    // initial parameters: U(-1/sqrt(fan_in), 1/sqrt(fan_in)) over the real (unpadded) fan-in;
    // padded input columns and output rows start at zero
    void init(int nin_, int nout_, int width_, int depth_, unsigned long long seed) {
        nin = nin_; nout = nout_; nin_pad = pad8(nin_); nout_pad = pad8(nout_); width = width_; depth = depth_;
        dims.assign(1, nin_pad);
        for (int l = 0; l < depth; ++l) dims.push_back(width);
        dims.push_back(nout_pad);
        size_t off = 0;
        for (int l = 0; l <= depth; ++l) {
            w_off.push_back(off);
            off += (size_t)dims[l] * dims[l + 1];
        }
        n_weights = off;
        for (int l = 0; l <= depth; ++l) {
            b_off.push_back(off);
            off += dims[l + 1];
        }
        n_params = off;
        std::vector<float> h(n_params, 0.f);
        std::mt19937_64 rng(seed);
        for (int l = 0; l <= depth; ++l) {
            const int fin = l == 0 ? nin : dims[l];
            const int fout = l == depth ? nout : dims[l + 1];
            const float bound = 1.f / std::sqrt((float)fin);
            std::uniform_real_distribution<float> U(-bound, bound);
            for (int o = 0; o < fout; ++o)
                for (int k = 0; k < fin; ++k) h[w_off[l] + (size_t)o * dims[l] + k] = U(rng);
            for (int o = 0; o < fout; ++o) h[b_off[l] + o] = U(rng);
        }
        params.ensure(n_params);
        grad.ensure(n_params);
        adam_m.ensure(n_params);
        adam_v.ensure(n_params);
        params_h.ensure(n_params);
        ck(cudaMemcpy(params.p, h.data(), n_params * 4, cudaMemcpyHostToDevice), "H2D");
        reset_adam();
        refresh_bf16(nullptr);
    }

    __nv_bfloat16* W16(int l) { return params_h.p + w_off[l]; }
    float* bias(int l) { return params.p + b_off[l]; }

    void reset_adam() {
        ck(cudaMemset(adam_m.p, 0, n_params * 4), "cudaMemset");
        ck(cudaMemset(adam_v.p, 0, n_params * 4), "cudaMemset");
        step = 0;
    }

    void refresh_bf16(cudaStream_t s) { ck(launch_cast_bf16((int)n_params, params.p, params_h.p, s), "cast"); }

    void ensure_train(int B) {
        if (B <= tb) return;
        tb = B;
        const size_t W = width;
        t_act.ensure((size_t)depth * B * W);
        t_pre.ensure((size_t)depth * B * W);
        t_out.ensure((size_t)B * nout_pad);
        t_dout.ensure((size_t)B * nout_pad);
        t_dout16.ensure((size_t)B * nout_pad);
        t_dpre.ensure((size_t)B * W);
        t_g16a.ensure((size_t)B * W);
        t_g16b.ensure((size_t)B * W);
        t_work.ensure((size_t)32 * W * std::max<size_t>(W, nin_pad));
        t_colpart.ensure((size_t)column_sum_partials(B) * std::max<size_t>(W, nout_pad));
    }

    void ensure_infer(int chunk) {
        if (chunk <= ib) return;
        ib = chunk;
        i_a0.ensure((size_t)chunk * width);
        i_a1.ensure((size_t)chunk * width);
    }

    // forward over B rows of bf16 inputs xh; training (into t_out) keeps every layer's
    // pre-activation and activation.  The fp32 output goes to out.
    void forward(int B, const __nv_bfloat16* xh, bool train, float* out, cudaStream_t s) {
        if (train) ensure_train(B);
        else ensure_infer(B);
        const __nv_bfloat16* in = xh;
        for (int l = 0; l < depth; ++l) {
            __nv_bfloat16* act;
            float* pre = nullptr;
            if (train) {
                act = t_act.p + (size_t)l * B * width;
                pre = t_pre.p + (size_t)l * B * width;
            } else {
                act = (l & 1) ? i_a1.p : i_a0.p;
            }
            gemm(B, dims[l + 1], dims[l], in, dims[l], 0, W16(l), dims[l], 1, bias(l), ACT_GELU, nullptr, pre, nullptr,
                 act, dims[l + 1], s);
            in = act;
        }
        gemm(B, dims[depth + 1], dims[depth], in, dims[depth], 0, W16(depth), dims[depth], 1, bias(depth), ACT_NONE,
             nullptr, nullptr, out, nullptr, dims[depth + 1], s);
    }

    static int splits_for(int M, int N, int K, int sm) {
        const int tiles = ((M + 127) / 128) * ((N + 63) / 64);
        int sp = (2 * sm + tiles - 1) / tiles;
        sp = std::min(sp, std::max(1, K / 256));
        return std::max(1, std::min(sp, 32));
    }

    // gradient into `grad` from the output gradient in t_dout (fp32) / t_dout16 (bf16), after a
    // training forward over the same B rows of inputs xh
    void backward(int B, const __nv_bfloat16* xh, cudaStream_t s, int sm) {
        const float* g32 = t_dout.p;
        const __nv_bfloat16* g16 = t_dout16.p;
        __nv_bfloat16* nxt = t_g16a.p;
        for (int l = depth; l >= 0; --l) {
            const int din = dims[l], dout = dims[l + 1];
            const __nv_bfloat16* in16 = l == 0 ? xh : t_act.p + (size_t)(l - 1) * B * width;
            ck(launch_column_sum(B, dout, g32, t_colpart.p, grad.p + b_off[l], s), "bias gradient");
            const int sp = splits_for(dout, din, B, sm);
            gemm(dout, din, B, g16, dout, 1, in16, din, 0, nullptr, ACT_NONE, nullptr, nullptr, grad.p + w_off[l],
                 nullptr, din, s, sp, sp > 1 ? t_work.p : nullptr);
            if (l > 0) {
                gemm(B, din, dout, g16, dout, 0, W16(l), din, 0, nullptr, ACT_GELU_BWD,
                     t_pre.p + (size_t)(l - 1) * B * width, nullptr, t_dpre.p, nxt, din, s);
                g32 = t_dpre.p;
                g16 = nxt;
                nxt = (nxt == t_g16a.p) ? t_g16b.p : t_g16a.p;
            }
        }
    }

    // AdamW (beta 0.9, 0.999, eps 1e-8); weight decay on the weights, not the biases
    void adam(float lr, float wd, cudaStream_t s) {
        ++step;
        ck(launch_adamw((int)n_weights, params.p, grad.p, adam_m.p, adam_v.p, params_h.p, lr, 0.9f, 0.999f, 1e-8f, wd,
                        step, s),
           "adamw");
        const size_t nb = n_params - n_weights;
        ck(launch_adamw((int)nb, params.p + n_weights, grad.p + n_weights, adam_m.p + n_weights,
                        adam_v.p + n_weights, params_h.p + n_weights, lr, 0.9f, 0.999f, 1e-8f, 0.f, step, s),
           "adamw");
    }
};

struct Surrogate {
    int cr = -1;
    int nsp = 0, nin = 0, nin_pad = 0, nout = 0, nout_pad = 0, ne = 0;
    Mlp net;                    // state -> increment
    std::unique_ptr<Mlp> err;   // (standardised state, standardised increment) -> log10 of the increment's error
    double err_log10_tol = 0.0;
    bool err_gate = false;
    // standardisation and domain (host copies + device)
    std::vector<float> xs, xd, ys, yd, lw;
    std::vector<double> xmin, xmax;
    Buf<float> d_xs, d_xd, d_ys, d_yd, d_lw;
    Buf<double> d_xmin, d_xmax, d_elem, d_elemM;
    double elem_tol = 1e-4, neg_tol = 1e-5, T_tol = 1e-3, max_dY = 5e-4;
    // training inputs of the current batch (standardised)
    Buf<__nv_bfloat16> t_xh, e_xh;
    Buf<float> t_y, e_main, e_tgt;
    // inference buffers
    int ib = 0;
    Buf<__nv_bfloat16> i_xh, i_exh;
    Buf<float> i_out, i_err;
    Buf<int> gate, reject, counters, fails, mon_idx, cstatus, mstatus;
    Buf<unsigned long long> code_counts, mon_res;
    Buf<double> compact, mon_state, mon_compact, mon_sum;
    Buf<double> stats_partial, stats_out;

    void upload_norm() {
        ck(cudaMemcpy(d_xs.ensure(nin_pad), xs.data(), nin_pad * 4, cudaMemcpyHostToDevice), "H2D");
        ck(cudaMemcpy(d_xd.ensure(nin_pad), xd.data(), nin_pad * 4, cudaMemcpyHostToDevice), "H2D");
        ck(cudaMemcpy(d_ys.ensure(nout_pad), ys.data(), nout_pad * 4, cudaMemcpyHostToDevice), "H2D");
        ck(cudaMemcpy(d_yd.ensure(nout_pad), yd.data(), nout_pad * 4, cudaMemcpyHostToDevice), "H2D");
        ck(cudaMemcpy(d_lw.ensure(nout_pad), lw.data(), nout_pad * 4, cudaMemcpyHostToDevice), "H2D");
        ck(cudaMemcpy(d_xmin.ensure(nin_pad), xmin.data(), nin_pad * 8, cudaMemcpyHostToDevice), "H2D");
        ck(cudaMemcpy(d_xmax.ensure(nin_pad), xmax.data(), nin_pad * 8, cudaMemcpyHostToDevice), "H2D");
    }

    // rows of raw X, Y -> standardised t_xh (bf16) and t_y
    void gather(int B, const float* X, const float* Y, const int* rows, cudaStream_t s) {
        t_xh.ensure((size_t)B * nin_pad);
        t_y.ensure((size_t)B * nout_pad);
        ck(launch_gather_rows(B, rows, X, nin_pad, d_xs.p, d_xd.p, t_xh.p, Y, nout_pad, d_ys.p, d_yd.p, t_y.p, s),
           "gather rows");
    }

    // the increment network's weighted squared error and its gradient (net.grad)
    void loss_and_grad(int B, const float* X, const float* Y, const int* rows, float* loss_sum, cudaStream_t s,
                       int sm) {
        gather(B, X, Y, rows, s);
        net.ensure_train(B);   // before t_out is read as the output pointer
        net.forward(B, t_xh.p, true, net.t_out.p, s);
        ck(launch_mse_grad(B, nout_pad, net.t_out.p, t_y.p, d_lw.p, net.t_dout.p, net.t_dout16.p, loss_sum, s), "loss");
        net.backward(B, t_xh.p, s, sm);
    }

    // The error network's pinball loss at quantile tau and its gradient (err->grad): inputs are
    // the increment network's standardised input and output, the target is log10 of that output's
    // error on the sample: the larger of its largest |dY| error and 0.1 times its relative error in
    // the temperature increment (a relative T error of 1e-3 weighs as a mass-fraction error of 1e-4).
    void error_loss_and_grad(int B, const float* X, const float* Y, const int* rows, float tau, float* loss_sum,
                             cudaStream_t s, int sm) {
        gather(B, X, Y, rows, s);
        e_main.ensure((size_t)B * nout_pad);
        net.forward(B, t_xh.p, false, e_main.p, s);
        const int nin_e = err->nin_pad;
        e_xh.ensure((size_t)B * nin_e);
        e_tgt.ensure((size_t)B * err->nout_pad);
        ck(launch_error_features(B, t_xh.p, nin_pad, e_main.p, nout_pad, e_xh.p, s), "error features");
        ck(launch_error_targets(B, e_main.p, t_y.p, nout_pad, d_yd.p, nsp, X, rows, nin_pad, kErrorTWeight, e_tgt.p,
                                err->nout_pad, s), "error targets");
        err->ensure_train(B);
        err->forward(B, e_xh.p, true, err->t_out.p, s);
        ck(launch_pinball_grad(B, err->nout_pad, err->t_out.p, e_tgt.p, tau, err->t_dout.p, err->t_dout16.p, loss_sum,
                               s),
           "pinball loss");
        err->backward(B, e_xh.p, s, sm);
    }

    void ensure_infer(int chunk) {
        if (chunk <= ib) return;
        ib = chunk;
        i_xh.ensure((size_t)chunk * nin_pad);
        i_out.ensure((size_t)chunk * nout_pad);
    }

    void predict_raw(int n, const float* X, float* out, cudaStream_t s) {
        // out = standardised prediction * y_scale + y_shift, chunk by chunk
        const int chunk = std::min(n, 1 << 20);
        ensure_infer(chunk);
        for (int first = 0; first < n; first += chunk) {
            const int m = std::min(chunk, n - first);
            ck(launch_gather_rows(m, nullptr, X + (size_t)first * nin_pad, nin_pad, d_xs.p, d_xd.p, i_xh.p, nullptr,
                                  0, nullptr, nullptr, nullptr, s),
               "features");
            net.forward(m, i_xh.p, false, out + (size_t)first * nout_pad, s);
        }
        ck(launch_affine_columns(n, nout_pad, d_ys.p, d_yd.p, out, s), "destandardise");   // raw increments
    }

    // the error network's predicted log10 error of each chunk row (i_err, stride err->nout_pad)
    void predict_error_chunk(int m, cudaStream_t s) {
        i_exh.ensure((size_t)ib * err->nin_pad);
        i_err.ensure((size_t)ib * err->nout_pad);
        ck(launch_error_features(m, i_xh.p, nin_pad, i_out.p, nout_pad, i_exh.p, s), "error features");
        err->forward(m, i_exh.p, false, i_err.p, s);
    }
};

std::mutex g_smu;
std::vector<std::unique_ptr<Surrogate>> g_surr;

Surrogate& surr(int i) {
    std::lock_guard<std::mutex> lk(g_smu);
    if (i < 0 || i >= (int)g_surr.size() || !g_surr[i]) throw std::runtime_error("invalid surrogate handle");
    return *g_surr[i];
}

template <typename F>
int guard(F&& f) {
    try {
        return f();
    } catch (std::exception& e) {
        report_error(e.what());
        return -1;
    }
}

}  // namespace
}  // namespace gdtk

using namespace gdtk;

extern "C" {

int chem_surrogate_new(int cr_i, int width, int depth, unsigned long long seed) {
    return guard([&] {
        if (width < 8 || width % 8 || width > 4096) throw std::runtime_error("surrogate width must be a multiple of 8 in 8..4096");
        if (depth < 1 || depth > 16) throw std::runtime_error("surrogate depth must be in 1..16");
        ReactorInternals ri = reactor_internals(cr_i);
        if (ri.nsp > GDTK_MAX_SPECIES)
            throw std::runtime_error("the surrogate takes mechanisms of up to " + std::to_string(GDTK_MAX_SPECIES) +
                                     " species");
        auto S = std::make_unique<Surrogate>();
        S->cr = cr_i;
        S->nsp = ri.nsp;
        S->nin = ri.nsp + 3;
        S->nout = ri.nsp + 1;
        S->nin_pad = pad8(S->nin);
        S->nout_pad = pad8(S->nout);
        S->net.init(S->nin, S->nout, width, depth, seed);
        // identity standardisation, unbounded domain, unit loss weights until fitted
        S->xs.assign(S->nin_pad, 0.f);
        S->xd.assign(S->nin_pad, 1.f);
        S->ys.assign(S->nout_pad, 0.f);
        S->yd.assign(S->nout_pad, 1.f);
        S->xmin.assign(S->nin_pad, -1e300);
        S->xmax.assign(S->nin_pad, 1e300);
        S->lw.assign(S->nout_pad, 0.f);
        for (int k = 0; k < S->nout; ++k) S->lw[k] = 1.f;
        S->upload_norm();
        // element matrix of the gas model: atoms of e per kg of species s
        const GasModelHost& gm = *ri.gm;
        std::vector<std::string> els;
        for (auto& e : gm.elements)
            if (e != "e-" && e != "e") els.push_back(e);
        if ((int)els.size() > SURR_MAX_ELEMENTS) throw std::runtime_error("surrogate: too many elements");
        S->ne = (int)els.size();
        std::vector<double> E((size_t)S->ne * S->nsp, 0.0), EM(S->ne);
        for (int e = 0; e < S->ne; ++e) {
            EM[e] = atomic_mass(els[e]);
            for (int s = 0; s < S->nsp; ++s) {
                auto it = gm.composition.size() > (size_t)s ? gm.composition[s].find(els[e]) : gm.composition[0].end();
                if (gm.composition.size() > (size_t)s && it != gm.composition[s].end())
                    E[(size_t)e * S->nsp + s] = it->second / gm.M[s];
            }
        }
        S->d_elem.ensure(std::max<size_t>(E.size(), 1));
        S->d_elemM.ensure(std::max<size_t>(EM.size(), 1));
        if (!E.empty()) ck(cudaMemcpy(S->d_elem.p, E.data(), E.size() * 8, cudaMemcpyHostToDevice), "H2D");
        if (!EM.empty()) ck(cudaMemcpy(S->d_elemM.p, EM.data(), EM.size() * 8, cudaMemcpyHostToDevice), "H2D");
        ck(cudaDeviceSynchronize(), "surrogate init");
        std::lock_guard<std::mutex> lk(g_smu);
        g_surr.push_back(std::move(S));
        return (int)g_surr.size() - 1;
    });
}

int chem_surrogate_free(int sg) {
    return guard([&] {
        surr(sg);
        std::lock_guard<std::mutex> lk(g_smu);
        g_surr[sg].reset();
        return 0;
    });
}

int chem_surrogate_dims(int sg, int* dims) {
    return guard([&] {
        auto& S = surr(sg);
        int v[8] = {S.nin, S.nin_pad, S.nout, S.nout_pad, S.net.width, S.net.depth, (int)S.net.n_params, S.ne};
        std::memcpy(dims, v, sizeof v);
        return 0;
    });
}

int chem_surrogate_get_params(int sg, float* params) {
    return guard([&] {
        auto& S = surr(sg);
        ck(cudaMemcpy(params, S.net.params.p, S.net.n_params * 4, cudaMemcpyDeviceToHost), "D2H");
        return 0;
    });
}

int chem_surrogate_set_params(int sg, const float* params) {
    return guard([&] {
        auto& S = surr(sg);
        ck(cudaMemcpy(S.net.params.p, params, S.net.n_params * 4, cudaMemcpyHostToDevice), "H2D");
        S.net.reset_adam();
        S.net.refresh_bf16(nullptr);
        ck(cudaDeviceSynchronize(), "set params");
        return 0;
    });
}

int chem_surrogate_get_normalisation(int sg, float* x_shift, float* x_scale, float* y_shift, float* y_scale,
                                     double* x_min, double* x_max) {
    return guard([&] {
        auto& S = surr(sg);
        std::copy(S.xs.begin(), S.xs.end(), x_shift);
        std::copy(S.xd.begin(), S.xd.end(), x_scale);
        std::copy(S.ys.begin(), S.ys.end(), y_shift);
        std::copy(S.yd.begin(), S.yd.end(), y_scale);
        std::copy(S.xmin.begin(), S.xmin.end(), x_min);
        std::copy(S.xmax.begin(), S.xmax.end(), x_max);
        return 0;
    });
}

int chem_surrogate_set_normalisation(int sg, const float* x_shift, const float* x_scale, const float* y_shift,
                                     const float* y_scale, const double* x_min, const double* x_max) {
    return guard([&] {
        auto& S = surr(sg);
        for (int k = 0; k < S.nin_pad; ++k)
            if (!(x_scale[k] > 0.f)) throw std::runtime_error("x_scale must be > 0");
        for (int k = 0; k < S.nout_pad; ++k)
            if (!(y_scale[k] > 0.f)) throw std::runtime_error("y_scale must be > 0");
        S.xs.assign(x_shift, x_shift + S.nin_pad);
        S.xd.assign(x_scale, x_scale + S.nin_pad);
        S.ys.assign(y_shift, y_shift + S.nout_pad);
        S.yd.assign(y_scale, y_scale + S.nout_pad);
        S.xmin.assign(x_min, x_min + S.nin_pad);
        S.xmax.assign(x_max, x_max + S.nin_pad);
        S.upload_norm();
        return 0;
    });
}

int chem_surrogate_fit_normalisation(int sg, int nrows, const float* X, const float* Y, const int* rows,
                                     void* stream) {
    return guard([&] {
        auto& S = surr(sg);
        if (nrows <= 0) throw std::runtime_error("fit_normalisation needs rows");
        cudaStream_t s = (cudaStream_t)stream;
        const int np = 1024;
        const int wmax = std::max(S.nin_pad, S.nout_pad);
        S.stats_partial.ensure((size_t)np * 4 * wmax);
        S.stats_out.ensure((size_t)4 * wmax);
        std::vector<double> hx(4 * S.nin_pad), hy(4 * S.nout_pad);
        ck(launch_column_stats(nrows, S.nin_pad, X, rows, S.stats_partial.p, np, S.stats_out.p, s), "stats");
        ck(cudaMemcpyAsync(hx.data(), S.stats_out.p, hx.size() * 8, cudaMemcpyDeviceToHost, s), "D2H");
        ck(cudaStreamSynchronize(s), "sync");
        ck(launch_column_stats(nrows, S.nout_pad, Y, rows, S.stats_partial.p, np, S.stats_out.p, s), "stats");
        ck(cudaMemcpyAsync(hy.data(), S.stats_out.p, hy.size() * 8, cudaMemcpyDeviceToHost, s), "D2H");
        ck(cudaStreamSynchronize(s), "sync");
        const int nx = S.nin_pad, ny = S.nout_pad;
        for (int k = 0; k < nx; ++k) {
            const bool real = k < S.nin;
            const double sd = hx[nx + k];
            S.xs[k] = real ? (float)hx[k] : 0.f;
            S.xd[k] = (real && sd > 1e-12 * std::max(1.0, std::fabs(hx[k]))) ? (float)sd : 1.f;
            S.xmin[k] = real ? hx[2 * nx + k] : -1e300;
            S.xmax[k] = real ? hx[3 * nx + k] : 1e300;
        }
        for (int k = 0; k < ny; ++k) {
            const bool real = k < S.nout;
            const double sd = hy[ny + k];
            S.ys[k] = real ? (float)hy[k] : 0.f;
            S.yd[k] = (real && sd > 1e-30) ? (float)sd : 1.f;
        }
        S.upload_norm();
        return 0;
    });
}

int chem_surrogate_set_loss_weights(int sg, const float* w) {
    return guard([&] {
        auto& S = surr(sg);
        for (int k = 0; k < S.nout; ++k) S.lw[k] = w[k];
        S.upload_norm();
        return 0;
    });
}

int chem_surrogate_make_samples(int sg, int ncell, const double* T0, const double* p0, const double* massf0,
                                double dt, const double* T1, const double* massf1, const int* status, float* X,
                                float* Y, int* valid, void* stream) {
    return guard([&] {
        auto& S = surr(sg);
        if (ncell <= 0) return 0;
        if (!(dt > 0.0)) throw std::runtime_error("dt must be > 0");
        SampleArgs a{};
        a.ncell = ncell; a.nsp = S.nsp; a.nin_pad = S.nin_pad; a.nout_pad = S.nout_pad; a.dt = dt;
        a.T0 = T0; a.p0 = p0; a.massf0 = massf0; a.T1 = T1; a.massf1 = massf1; a.status = status;
        a.X = X; a.Y = Y; a.valid = valid;
        ck(launch_make_samples(a, (cudaStream_t)stream), "make samples");
        return 0;
    });
}

int chem_surrogate_train_step(int sg, int batch, const float* X, const float* Y, const int* rows, float lr,
                              float weight_decay, float* loss_sum, void* stream) {
    return guard([&] {
        auto& S = surr(sg);
        if (batch <= 0) throw std::runtime_error("batch must be > 0");
        cudaStream_t s = (cudaStream_t)stream;
        ReactorInternals ri = reactor_internals(S.cr);
        S.loss_and_grad(batch, X, Y, rows, loss_sum, s, ri.sm_count);
        S.net.adam(lr, weight_decay, s);
        return 0;
    });
}

int chem_surrogate_gradients(int sg, int batch, const float* X, const float* Y, const int* rows, float* grad,
                             float* loss_sum, void* stream) {
    return guard([&] {
        auto& S = surr(sg);
        if (batch <= 0) throw std::runtime_error("batch must be > 0");
        cudaStream_t s = (cudaStream_t)stream;
        ReactorInternals ri = reactor_internals(S.cr);
        S.loss_and_grad(batch, X, Y, rows, loss_sum, s, ri.sm_count);
        ck(cudaMemcpyAsync(grad, S.net.grad.p, S.net.n_params * 4, cudaMemcpyDeviceToDevice, s), "D2D");
        return 0;
    });
}

int chem_surrogate_predict(int sg, int n, const float* X, float* out, void* stream) {
    return guard([&] {
        auto& S = surr(sg);
        if (n <= 0) return 0;
        S.predict_raw(n, X, out, (cudaStream_t)stream);
        return 0;
    });
}

int chem_surrogate_set_gate(int sg, double elem_tol, double neg_tol, double T_tol, double max_dY) {
    return guard([&] {
        auto& S = surr(sg);
        if (!(elem_tol >= 0) || !(neg_tol >= 0) || !(T_tol >= 0)) throw std::runtime_error("gate tolerances must be >= 0");
        S.elem_tol = elem_tol;
        S.neg_tol = neg_tol;
        S.T_tol = T_tol;
        S.max_dY = max_dY;
        return 0;
    });
}

int chem_surrogate_update_cells(int sg, int ncell, const double* rho, const double* u, double* T, double* p,
                                double* massf, double* dt_chem, int* status, double t_interval, double T_frozen,
                                int flags, void* stream, int* gate, long long* counts, int monitor_stride,
                                double* monitor) {
    return guard([&] {
        auto& S = surr(sg);
        ReactorInternals ri = reactor_internals(S.cr);
        if (ncell < 0) throw std::runtime_error("ncell must be >= 0");
        if (counts) std::fill(counts, counts + GATE_COUNT + 2, 0LL);
        if (monitor) std::fill(monitor, monitor + 4, 0.0);
        if (ncell == 0) return 0;
        if (!rho || !u || !T || !p || !massf || !dt_chem) throw std::runtime_error("null cell array");
        if (!(t_interval > 0.0)) throw std::runtime_error("t_interval must be > 0");
        cudaStream_t s = (cudaStream_t)stream;
        const int nsp = S.nsp;
        const int chunk = std::min(ncell, 1 << 20);
        S.ensure_infer(chunk);
        int* gate_p = gate ? gate : S.gate.ensure(ncell);
        int* rej = S.reject.ensure(ncell);
        int* cnt = S.counters.ensure(2);
        unsigned long long* cc = S.code_counts.ensure(GATE_COUNT);
        const int cap = monitor_stride > 0 ? std::min(ncell / monitor_stride + 1, 1 << 18) : 0;
        if (cap) {
            S.mon_idx.ensure(cap);
            S.mon_state.ensure((size_t)(5 + nsp) * cap);
        }
        ck(cudaMemsetAsync(cnt, 0, 2 * sizeof(int), s), "memset");
        ck(cudaMemsetAsync(cc, 0, GATE_COUNT * sizeof(unsigned long long), s), "memset");
        for (int first = 0; first < ncell; first += chunk) {
            const int m = std::min(chunk, ncell - first);
            FeatureArgs fa{};
            fa.n = m; fa.first = first; fa.ncell = ncell; fa.nsp = nsp; fa.nin_pad = S.nin_pad;
            fa.dt = t_interval; fa.T_frozen = T_frozen;
            fa.rho = rho; fa.T = T; fa.p = p; fa.massf = massf;
            fa.x_shift = S.d_xs.p; fa.x_scale = S.d_xd.p; fa.x_min = S.d_xmin.p; fa.x_max = S.d_xmax.p;
            fa.Xh = S.i_xh.p; fa.gate = gate_p;
            ck(launch_features(fa, s), "surrogate features");
            S.net.forward(m, S.i_xh.p, false, S.i_out.p, s);
            const bool use_err = S.err && S.err_gate;
            if (use_err) S.predict_error_chunk(m, s);
            GateArgs ga{};
            ga.n = m; ga.first = first; ga.ncell = ncell; ga.nsp = nsp; ga.nout_pad = S.nout_pad; ga.ne = S.ne;
            ga.update_thermo = (flags & GDTK_CHEM_UPDATE_THERMO) ? 1 : 0;
            ga.mech_i = ri.mech_i; ga.mech_d = ri.mech_d;
            ga.elem = S.d_elem.p; ga.elem_M = S.d_elemM.p;
            ga.y_shift = S.d_ys.p; ga.y_scale = S.d_yd.p; ga.out = S.i_out.p;
            ga.elem_tol = S.elem_tol; ga.neg_tol = S.neg_tol; ga.T_tol = S.T_tol; ga.max_dY = S.max_dY;
            ga.rho = rho; ga.u = u; ga.T = T; ga.p = p; ga.massf = massf; ga.status = status; ga.gate = gate_p;
            ga.reject = rej; ga.counters = cnt; ga.code_counts = cc;
            ga.monitor_stride = cap ? monitor_stride : 0; ga.monitor_cap = cap;
            ga.mon_idx = S.mon_idx.p; ga.mon_state = S.mon_state.p; ga.dt_chem = dt_chem;
            ga.pred_err = use_err ? S.i_err.p : nullptr;
            ga.pred_err_ld = use_err ? S.err->nout_pad : 0;
            ga.err_log10_tol = S.err_log10_tol;
            ck(launch_gate(ga, s), "surrogate gate");
        }
        int hc[2] = {0, 0};
        unsigned long long hcc[GATE_COUNT];
        ck(cudaMemcpyAsync(hc, cnt, sizeof hc, cudaMemcpyDeviceToHost, s), "D2H");
        ck(cudaMemcpyAsync(hcc, cc, sizeof hcc, cudaMemcpyDeviceToHost, s), "D2H");
        ck(cudaStreamSynchronize(s), "surrogate gate");
        const int n_rej = hc[0];
        int n_fail = 0;
        if (n_rej > 0) {
            double* cb = S.compact.ensure((size_t)(5 + nsp) * n_rej);
            int* cst = S.cstatus.ensure(n_rej);
            int* fails = S.fails.ensure(1);
            ck(cudaMemsetAsync(fails, 0, sizeof(int), s), "memset");
            ck(launch_gather_cells(n_rej, rej, ncell, nsp, rho, u, T, p, dt_chem, massf, cb, s), "gather");
            const size_t n = n_rej;
            reactor_update(S.cr, n_rej, cb, cb + n, cb + 2 * n, cb + 3 * n, cb + 5 * n, cb + 4 * n, cst, t_interval,
                           T_frozen, flags, s);
            ck(launch_scatter_cells(n_rej, rej, ncell, nsp, cb, cst, T, p, dt_chem, massf, status, fails, s),
               "scatter");
            ck(cudaMemcpyAsync(&n_fail, fails, sizeof(int), cudaMemcpyDeviceToHost, s), "D2H");
        }
        const int n_mon = std::min(hc[1], cap);
        if (n_mon > 0) {
            double* mc = S.mon_compact.ensure((size_t)(5 + nsp) * n_mon);
            int* mst = S.mstatus.ensure(n_mon);
            unsigned long long* res = S.mon_res.ensure(3);
            double* msum = S.mon_sum.ensure(1);
            ck(launch_repack(n_mon, cap, 5 + nsp, S.mon_state.p, mc, s), "repack");
            const size_t n = n_mon;
            reactor_update(S.cr, n_mon, mc, mc + n, mc + 2 * n, mc + 3 * n, mc + 5 * n, mc + 4 * n, mst, t_interval,
                           T_frozen, flags, s);
            ck(cudaMemsetAsync(res, 0, 3 * sizeof(unsigned long long), s), "memset");
            ck(cudaMemsetAsync(msum, 0, sizeof(double), s), "memset");
            ck(launch_monitor_compare(n_mon, S.mon_idx.p, ncell, nsp, mc, mst, T, massf, res, msum, s), "monitor");
            unsigned long long hr[3];
            double hs = 0.0;
            ck(cudaMemcpyAsync(hr, res, sizeof hr, cudaMemcpyDeviceToHost, s), "D2H");
            ck(cudaMemcpyAsync(&hs, msum, sizeof hs, cudaMemcpyDeviceToHost, s), "D2H");
            ck(cudaStreamSynchronize(s), "monitor");
            if (monitor) {
                double ey, et;
                std::memcpy(&ey, &hr[1], 8);
                std::memcpy(&et, &hr[2], 8);
                monitor[0] = (double)hr[0];
                monitor[1] = ey;
                monitor[2] = et;
                monitor[3] = hr[0] ? hs / (double)hr[0] : 0.0;
            }
        }
        ck(cudaStreamSynchronize(s), "surrogate update");
        if (counts) {
            for (int k = 0; k < GATE_COUNT; ++k) counts[k] = (long long)hcc[k];
            counts[GATE_COUNT] = n_rej;
            counts[GATE_COUNT + 1] = n_fail;
        }
        return 0;
    });
}

int chem_surrogate_error_model_new(int sg, int width, int depth, unsigned long long seed) {
    return guard([&] {
        auto& S = surr(sg);
        if (width < 8 || width % 8 || width > 4096) throw std::runtime_error("width must be a multiple of 8 in 8..4096");
        if (depth < 1 || depth > 16) throw std::runtime_error("depth must be in 1..16");
        auto e = std::make_unique<Mlp>();
        e->init(S.nin_pad + S.nout_pad, 1, width, depth, seed);
        ck(cudaDeviceSynchronize(), "error model init");
        S.err = std::move(e);
        return 0;
    });
}

int chem_surrogate_error_dims(int sg, int* dims) {
    return guard([&] {
        auto& S = surr(sg);
        if (!S.err) throw std::runtime_error("the surrogate has no error model");
        int v[5] = {S.err->nin, S.err->nout_pad, S.err->width, S.err->depth, (int)S.err->n_params};
        std::memcpy(dims, v, sizeof v);
        return 0;
    });
}

int chem_surrogate_error_get_params(int sg, float* params) {
    return guard([&] {
        auto& S = surr(sg);
        if (!S.err) throw std::runtime_error("the surrogate has no error model");
        ck(cudaMemcpy(params, S.err->params.p, S.err->n_params * 4, cudaMemcpyDeviceToHost), "D2H");
        return 0;
    });
}

int chem_surrogate_error_set_params(int sg, const float* params) {
    return guard([&] {
        auto& S = surr(sg);
        if (!S.err) throw std::runtime_error("the surrogate has no error model");
        ck(cudaMemcpy(S.err->params.p, params, S.err->n_params * 4, cudaMemcpyHostToDevice), "H2D");
        S.err->reset_adam();
        S.err->refresh_bf16(nullptr);
        ck(cudaDeviceSynchronize(), "set params");
        return 0;
    });
}

int chem_surrogate_error_train_step(int sg, int batch, const float* X, const float* Y, const int* rows, float lr,
                                    float weight_decay, float quantile, float* loss_sum, void* stream) {
    return guard([&] {
        auto& S = surr(sg);
        if (!S.err) throw std::runtime_error("the surrogate has no error model");
        if (batch <= 0) throw std::runtime_error("batch must be > 0");
        if (!(quantile > 0.f && quantile < 1.f)) throw std::runtime_error("quantile must be in (0, 1)");
        cudaStream_t s = (cudaStream_t)stream;
        ReactorInternals ri = reactor_internals(S.cr);
        S.error_loss_and_grad(batch, X, Y, rows, quantile, loss_sum, s, ri.sm_count);
        S.err->adam(lr, weight_decay, s);
        return 0;
    });
}

int chem_surrogate_error_gradients(int sg, int batch, const float* X, const float* Y, const int* rows, float quantile,
                                   float* grad, float* loss_sum, void* stream) {
    return guard([&] {
        auto& S = surr(sg);
        if (!S.err) throw std::runtime_error("the surrogate has no error model");
        if (batch <= 0) throw std::runtime_error("batch must be > 0");
        cudaStream_t s = (cudaStream_t)stream;
        ReactorInternals ri = reactor_internals(S.cr);
        S.error_loss_and_grad(batch, X, Y, rows, quantile, loss_sum, s, ri.sm_count);
        ck(cudaMemcpyAsync(grad, S.err->grad.p, S.err->n_params * 4, cudaMemcpyDeviceToDevice, s), "D2D");
        return 0;
    });
}

int chem_surrogate_predict_error(int sg, int n, const float* X, float* out, void* stream) {
    return guard([&] {
        auto& S = surr(sg);
        if (!S.err) throw std::runtime_error("the surrogate has no error model");
        if (n <= 0) return 0;
        cudaStream_t s = (cudaStream_t)stream;
        const int chunk = std::min(n, 1 << 20);
        S.ensure_infer(chunk);
        for (int first = 0; first < n; first += chunk) {
            const int m = std::min(chunk, n - first);
            ck(launch_gather_rows(m, nullptr, X + (size_t)first * S.nin_pad, S.nin_pad, S.d_xs.p, S.d_xd.p, S.i_xh.p,
                                  nullptr, 0, nullptr, nullptr, nullptr, s),
               "features");
            S.net.forward(m, S.i_xh.p, false, S.i_out.p, s);
            S.predict_error_chunk(m, s);
            ck(launch_copy_column(m, S.i_err.p, S.err->nout_pad, 0, out + first, s), "copy");
        }
        return 0;
    });
}

int chem_surrogate_set_error_gate(int sg, double tol) {
    return guard([&] {
        auto& S = surr(sg);
        if (tol > 0.0 && !S.err) throw std::runtime_error("the surrogate has no error model");
        S.err_gate = tol > 0.0;
        S.err_log10_tol = tol > 0.0 ? std::log10(tol) : 0.0;
        return 0;
    });
}

int gdtk_mlp_tcgen05(int enable, unsigned long long* launches, int* error) {
    return guard([&] {
        const int prev = tcgen05_gemm_set(enable);
        if (launches) *launches = tcgen05_gemm_launches();
        if (error) ck(tcgen05_gemm_error(error), "gdtk_mlp_tcgen05");
        return prev;
    });
}

int gdtk_mlp_gemm(int M, int N, int K, const void* A, int lda, int trans_a, const void* B, int ldb, int trans_b,
                  const float* bias, int act, float* pre, float* D, void* Dh, int ldd, int splits, void* stream) {
    return guard([&] {
        if (act != ACT_NONE && act != ACT_GELU) throw std::runtime_error("act must be 0 or 1");
        GemmArgs g;
        g.M = M; g.N = N; g.K = K;
        g.A = (const __nv_bfloat16*)A; g.lda = lda; g.trans_a = trans_a;
        g.B = (const __nv_bfloat16*)B; g.ldb = ldb; g.trans_b = trans_b;
        g.bias = bias; g.act = act; g.pre = pre; g.D = D; g.Dh = (__nv_bfloat16*)Dh; g.ldd = ldd;
        g.splits = splits < 1 ? 1 : splits;
        Buf<float> work;
        if (g.splits > 1) g.work = work.ensure((size_t)g.splits * M * N);
        ck(launch_gemm_bf16(g, (cudaStream_t)stream), "gdtk_mlp_gemm");
        if (g.splits > 1) ck(cudaStreamSynchronize((cudaStream_t)stream), "gdtk_mlp_gemm");
        return 0;
    });
}

}  // extern "C"
