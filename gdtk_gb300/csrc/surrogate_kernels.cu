// surrogate_kernels.cu -- per-cell FP64 kernels around the chemistry surrogate network:
// training-sample assembly, feature standardisation with the training-domain test, the gate
// that checks every predicted increment (element conservation, non-negativity, energy
// consistency through the reference's T-from-(rho, u) Newton iteration), and the compaction
// of rejected cells for the plain FP64 update.  No counterpart in the reference.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "chem_types.h"
#include "mix_thermo.cuh"
#include "surrogate_launch.h"

namespace gdtk {
namespace {

__device__ __forceinline__ int warp_append(int* counter, bool want) {
    // one atomic per warp (all 32 lanes must call); returns this lane's slot (or -1)
    const unsigned FULL = 0xffffffffu;
    const unsigned m = __ballot_sync(FULL, want);
    if (!m) return -1;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(m));
    base = __shfl_sync(FULL, base, leader);
    return want ? base + __popc(m & ((1u << lane) - 1u)) : -1;
}

__global__ void make_samples_kernel(const SampleArgs a) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < a.ncell; c += gridDim.x * blockDim.x) {
        const double T0 = a.T0[c], p0 = a.p0[c];
        const bool ok = (!a.status || a.status[c] == CELL_OK) && T0 > 0.0 && p0 > 0.0;
        float* x = a.X + (size_t)c * a.nin_pad;
        float* y = a.Y + (size_t)c * a.nout_pad;
        for (int k = 0; k < a.nin_pad; ++k) x[k] = 0.f;
        for (int k = 0; k < a.nout_pad; ++k) y[k] = 0.f;
        if (ok) {
            x[0] = (float)log(T0);
            x[1] = (float)log(p0);
            for (int s = 0; s < a.nsp; ++s) {
                const double y0 = a.massf0[(size_t)s * a.ncell + c];
                x[2 + s] = (float)y0;
                y[s] = (float)(a.massf1[(size_t)s * a.ncell + c] - y0);
            }
            x[2 + a.nsp] = (float)log(a.dt);
            y[a.nsp] = (float)(a.T1[c] - T0);
        }
        if (a.valid) a.valid[c] = ok ? 1 : 0;
    }
}

// Block b reduces rows [b * chunk, (b + 1) * chunk) of the selected rows; thread t handles column
// t % ncol over the rows lane, lane + lanes, ... (lane = t / ncol); lanes are then combined in
// ascending order.  partial[b][4][ncol] = sum, sum of squares, min, max.
__global__ void column_stats_partial(int nrows, int ncol, const float* X, const int* rows, int chunk,
                                     double* partial) {
    extern __shared__ double sh[];
    const int lanes = blockDim.x / ncol;
    const int t = threadIdx.x, col = t % ncol, lane = t / ncol;
    const int r0 = blockIdx.x * chunk, r1 = min(nrows, r0 + chunk);
    double s = 0.0, q = 0.0, lo = 1e300, hi = -1e300;
    if (lane < lanes) {
        for (int r = r0 + lane; r < r1; r += lanes) {
            const size_t row = rows ? (size_t)rows[r] : (size_t)r;
            const double v = X[row * ncol + col];
            s += v;
            q += v * v;
            lo = fmin(lo, v);
            hi = fmax(hi, v);
        }
    }
    double* S = sh;
    double* Q = S + blockDim.x;
    double* L = Q + blockDim.x;
    double* H = L + blockDim.x;
    S[t] = s; Q[t] = q; L[t] = lo; H[t] = hi;
    __syncthreads();
    if (t < ncol) {
        for (int l = 1; l < lanes; ++l) {
            const int u = l * ncol + t;
            s += S[u]; q += Q[u]; lo = fmin(lo, L[u]); hi = fmax(hi, H[u]);
        }
        double* P = partial + (size_t)blockIdx.x * 4 * ncol;
        P[t] = s; P[ncol + t] = q; P[2 * ncol + t] = lo; P[3 * ncol + t] = hi;
    }
}

__global__ void column_stats_final(int nrows, int ncol, int nblocks, const double* partial, double* out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncol) return;
    double s = 0.0, q = 0.0, lo = 1e300, hi = -1e300;
    for (int b = 0; b < nblocks; ++b) {
        const double* P = partial + (size_t)b * 4 * ncol;
        s += P[c]; q += P[ncol + c]; lo = fmin(lo, P[2 * ncol + c]); hi = fmax(hi, P[3 * ncol + c]);
    }
    const double mean = s / nrows;
    const double var = fmax(q / nrows - mean * mean, 0.0);
    out[c] = mean;
    out[ncol + c] = sqrt(var);
    out[2 * ncol + c] = lo;
    out[3 * ncol + c] = hi;
}

__global__ void features_kernel(const FeatureArgs a) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
        const int c = a.first + i;
        const double T = a.T[c], rho = a.rho[c], p = a.p[c];
        __nv_bfloat16* x = a.Xh + (size_t)i * a.nin_pad;
        int code = GATE_ACCEPTED;
        if (T <= a.T_frozen) code = GATE_FROZEN;
        else if (isnan(rho) || rho <= 0.0 || !(T > 0.0) || !(p > 0.0)) code = GATE_BAD_INPUT;
        if (code != GATE_ACCEPTED) {
            for (int k = 0; k < a.nin_pad; ++k) x[k] = __float2bfloat16(0.f);
            a.gate[c] = code;
            continue;
        }
        bool inside = true;
        for (int k = 0; k < a.nin_pad; ++k) {
            double f = 0.0;
            if (k == 0) f = log(T);
            else if (k == 1) f = log(p);
            else if (k < 2 + a.nsp) f = a.massf[(size_t)(k - 2) * a.ncell + c];
            else if (k == 2 + a.nsp) f = log(a.dt);
            // the same rounding as the training features: raw value to float, standardised in float
            const float fr = (float)f;
            if (k < 3 + a.nsp && !((double)fr >= a.x_min[k] && (double)fr <= a.x_max[k])) inside = false;
            x[k] = __float2bfloat16((fr - a.x_shift[k]) / a.x_scale[k]);
        }
        a.gate[c] = inside ? GATE_ACCEPTED : GATE_DOMAIN;
    }
}

// Solves the ne x ne symmetric positive definite system G lam = r (Cholesky, in place).
// Returns false when G is not numerically positive definite.
__device__ bool spd_solve(double (*G)[SURR_MAX_ELEMENTS], double* r, int ne) {
    for (int j = 0; j < ne; ++j) {
        double d = G[j][j];
        for (int k = 0; k < j; ++k) d -= G[j][k] * G[j][k];
        if (!(d > 0.0)) return false;
        d = sqrt(d);
        G[j][j] = d;
        for (int i = j + 1; i < ne; ++i) {
            double v = G[i][j];
            for (int k = 0; k < j; ++k) v -= G[i][k] * G[j][k];
            G[i][j] = v / d;
        }
    }
    for (int i = 0; i < ne; ++i) {   // L z = r
        double v = r[i];
        for (int k = 0; k < i; ++k) v -= G[i][k] * r[k];
        r[i] = v / G[i][i];
    }
    for (int i = ne - 1; i >= 0; --i) {   // L^T lam = z
        double v = r[i];
        for (int k = i + 1; k < ne; ++k) v -= G[k][i] * r[k];
        r[i] = v / G[i][i];
    }
    return true;
}

__global__ void __launch_bounds__(128) gate_kernel(const GateArgs a) {
    __shared__ unsigned hist[GATE_COUNT];
    for (int k = threadIdx.x; k < GATE_COUNT; k += blockDim.x) hist[k] = 0;
    __syncthreads();
    MechView m;
    m.bind(a.mech_i, a.mech_d);
    const int nsp = a.nsp;
    // grid-stride loop with a uniform trip count per warp so that warp_append sees whole warps
    const int stride = gridDim.x * blockDim.x;
    const int iters = (a.n + stride - 1) / stride;
    for (int it = 0; it < iters; ++it) {
        const int i = it * stride + blockIdx.x * blockDim.x + threadIdx.x;
        const bool live = i < a.n;
        const int c = a.first + (live ? i : 0);
        int code = live ? a.gate[c] : GATE_ACCEPTED;
        bool reject = false, monitor = false;
        double Y0[GDTK_MAX_SPECIES], Y1[GDTK_MAX_SPECIES];
        double T0 = 0.0, p0 = 0.0, T1 = 0.0, p1 = 0.0;
        if (live && code == GATE_FROZEN) {
            if (a.status) a.status[c] = CELL_FROZEN;
        } else if (live && code == GATE_BAD_INPUT) {
            if (a.status) a.status[c] = CELL_BAD_INPUT;
        } else if (live && code == GATE_DOMAIN) {
            reject = true;
        } else if (live) {
            T0 = a.T[c];
            p0 = a.p[c];
            const float* o = a.out + (size_t)i * a.nout_pad;
            double dY[GDTK_MAX_SPECIES];
            double maxd = 0.0;
            for (int s = 0; s < nsp; ++s) {
                Y0[s] = a.massf[(size_t)s * a.ncell + c];
                dY[s] = (double)o[s] * (double)a.y_scale[s] + (double)a.y_shift[s];
                maxd = fmax(maxd, fabs(dY[s]));
            }
            const double dT = (double)o[nsp] * (double)a.y_scale[nsp] + (double)a.y_shift[nsp];
            if (a.max_dY > 0.0 && maxd > a.max_dY) code = GATE_MAGNITUDE;
            if (code == GATE_ACCEPTED && a.pred_err && !((double)a.pred_err[(size_t)i * a.pred_err_ld] <= a.err_log10_tol))
                code = GATE_PREDICTED_ERROR;
            // element balance of the predicted increment (mol of element per kg of mixture)
            double r[SURR_MAX_ELEMENTS];
            double worst = 0.0;
            for (int e = 0; e < a.ne; ++e) {
                double v = 0.0;
                for (int s = 0; s < nsp; ++s) v += a.elem[e * nsp + s] * dY[s];
                r[e] = v;
                worst = fmax(worst, fabs(v) * a.elem_M[e]);
            }
            if (code == GATE_ACCEPTED && worst > a.elem_tol) code = GATE_ELEMENTS;
            if (code == GATE_ACCEPTED && a.ne > 0) {
                // minimum-change projection onto exact element conservation, weighted by species
                // abundance: dY <- dY - W E^T (E W E^T)^-1 r, W = diag(max(Y0, Y0 + dY) + 1e-12)
                double w[GDTK_MAX_SPECIES];
                for (int s = 0; s < nsp; ++s) w[s] = fmax(Y0[s], Y0[s] + dY[s]) + 1e-12;
                double G[SURR_MAX_ELEMENTS][SURR_MAX_ELEMENTS];
                for (int e = 0; e < a.ne; ++e)
                    for (int f = 0; f <= e; ++f) {
                        double v = 0.0;
                        for (int s = 0; s < nsp; ++s) v += a.elem[e * nsp + s] * w[s] * a.elem[f * nsp + s];
                        G[e][f] = v;
                        G[f][e] = v;
                    }
                if (!spd_solve(G, r, a.ne)) {
                    code = GATE_ELEMENTS;
                } else {
                    for (int s = 0; s < nsp; ++s) {
                        double corr = 0.0;
                        for (int e = 0; e < a.ne; ++e) corr += a.elem[e * nsp + s] * r[e];
                        dY[s] -= w[s] * corr;
                    }
                }
            }
            if (code == GATE_ACCEPTED) {
                double most_neg = 0.0;
                bool clipped = false;
                for (int s = 0; s < nsp; ++s) {
                    double y = Y0[s] + dY[s];
                    most_neg = fmin(most_neg, y);
                    if (y < 0.0) { y = 0.0; clipped = true; }
                    Y1[s] = y;
                }
                if (most_neg < -a.neg_tol) code = GATE_NEGATIVE;
                if (code == GATE_ACCEPTED && clipped && a.ne > 0) {
                    // restore the element balance that clipping broke, moving only species present
                    // (weights Y1, so clipped species stay at zero)
                    double w[GDTK_MAX_SPECIES];
                    for (int s = 0; s < nsp; ++s) w[s] = Y1[s] + 1e-300;
                    for (int e = 0; e < a.ne; ++e) {
                        double v = 0.0;
                        for (int s = 0; s < nsp; ++s) v += a.elem[e * nsp + s] * (Y1[s] - Y0[s]);
                        r[e] = v;
                    }
                    double G[SURR_MAX_ELEMENTS][SURR_MAX_ELEMENTS];
                    for (int e = 0; e < a.ne; ++e)
                        for (int f = 0; f <= e; ++f) {
                            double v = 0.0;
                            for (int s = 0; s < nsp; ++s) v += a.elem[e * nsp + s] * w[s] * a.elem[f * nsp + s];
                            G[e][f] = v;
                            G[f][e] = v;
                        }
                    if (!spd_solve(G, r, a.ne)) {
                        code = GATE_ELEMENTS;
                    } else {
                        for (int s = 0; s < nsp; ++s) {
                            double corr = 0.0;
                            for (int e = 0; e < a.ne; ++e) corr += a.elem[e * nsp + s] * r[e];
                            Y1[s] = fmax(Y1[s] - w[s] * corr, 0.0);
                        }
                    }
                }
                if (code == GATE_ACCEPTED) {
                    double sum = 0.0;
                    for (int s = 0; s < nsp; ++s) sum += Y1[s];
                    if (!(sum > 0.0)) code = GATE_NEGATIVE;
                    else
                        for (int s = 0; s < nsp; ++s) Y1[s] /= sum;
                }
            }
            if (code == GATE_ACCEPTED) {
                int err = 0, its = 0;
                double guess = T0 + dT;
                if (!(guess > 0.0)) guess = T0;
                T1 = T_from_u(m, Vec{Y1, 1}, a.u[c], guess, err, its);
                if (err || !(T1 > 0.0)) code = GATE_NEWTON;
                else if (fabs(T1 - (T0 + dT)) > a.T_tol * T1) code = GATE_ENERGY;
                else p1 = a.rho[c] * gas_constant(m, Vec{Y1, 1}) * T1;
            }
            reject = code != GATE_ACCEPTED;
            monitor = !reject && a.monitor_stride > 0 && (c % a.monitor_stride) == 0;
        }
        if (live) {
            a.gate[c] = code;
            atomicAdd(&hist[code], 1u);
        }
        const int slot = warp_append(&a.counters[0], reject);
        if (slot >= 0) a.reject[slot] = c;
        const int mslot = warp_append(&a.counters[1], monitor);
        if (mslot >= 0 && mslot < a.monitor_cap) {   // the original state, before it is overwritten
            const int cap = a.monitor_cap;
            a.mon_idx[mslot] = c;
            a.mon_state[0 * cap + mslot] = a.rho[c];
            a.mon_state[1 * cap + mslot] = a.u[c];
            a.mon_state[2 * cap + mslot] = T0;
            a.mon_state[3 * cap + mslot] = p0;
            a.mon_state[4 * cap + mslot] = a.dt_chem[c];
            for (int s = 0; s < nsp; ++s) a.mon_state[(size_t)(5 + s) * cap + mslot] = Y0[s];
        }
        if (live && code == GATE_ACCEPTED) {
            for (int s = 0; s < nsp; ++s) a.massf[(size_t)s * a.ncell + c] = Y1[s];
            if (a.update_thermo) {
                a.T[c] = T1;
                a.p[c] = p1;
            }
            if (a.status) a.status[c] = CELL_OK;
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < GATE_COUNT; k += blockDim.x)
        if (hist[k]) atomicAdd(&a.code_counts[k], (unsigned long long)hist[k]);
}

__global__ void gather_cells_kernel(int n, const int* idx, int ncell, int nsp, const double* rho, const double* u,
                                    const double* T, const double* p, const double* dt_chem, const double* massf,
                                    double* cb) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int c = idx[i];
        cb[0 * (size_t)n + i] = rho[c];
        cb[1 * (size_t)n + i] = u[c];
        cb[2 * (size_t)n + i] = T[c];
        cb[3 * (size_t)n + i] = p[c];
        cb[4 * (size_t)n + i] = dt_chem[c];
        for (int s = 0; s < nsp; ++s) cb[(size_t)(5 + s) * n + i] = massf[(size_t)s * ncell + c];
    }
}

__global__ void scatter_cells_kernel(int n, const int* idx, int ncell, int nsp, const double* cb, const int* cst,
                                     double* T, double* p, double* dt_chem, double* massf, int* status,
                                     int* fail_count) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int c = idx[i];
        T[c] = cb[2 * (size_t)n + i];
        p[c] = cb[3 * (size_t)n + i];
        dt_chem[c] = cb[4 * (size_t)n + i];
        for (int s = 0; s < nsp; ++s) massf[(size_t)s * ncell + c] = cb[(size_t)(5 + s) * n + i];
        const int st = cst[i];
        if (status) status[c] = st;
        if (st != CELL_OK && st != CELL_FROZEN && fail_count) atomicAdd(fail_count, 1);
    }
}

__global__ void monitor_compare_kernel(int n, const int* idx, int ncell, int nsp, const double* cb, const int* cst,
                                       const double* T, const double* massf, unsigned long long* res, double* sum) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (cst[i] != CELL_OK) continue;
        const int c = idx[i];
        double ey = 0.0;
        for (int s = 0; s < nsp; ++s) ey = fmax(ey, fabs(cb[(size_t)(5 + s) * n + i] - massf[(size_t)s * ncell + c]));
        const double Tr = cb[2 * (size_t)n + i];
        const double et = fabs(Tr - T[c]) / Tr;
        atomicAdd(&res[0], 1ull);
        atomicMax(&res[1], (unsigned long long)__double_as_longlong(ey));   // non-negative: bit order = value order
        atomicMax(&res[2], (unsigned long long)__double_as_longlong(et));
        atomicAdd(sum, ey);
    }
}

// dst[k * n + i] = src[k * cap + i] for k < nk, i < n
__global__ void repack_kernel(int n, int cap, int nk, const double* src, double* dst) {
    const size_t total = (size_t)n * nk;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const size_t k = t / n, i = t % n;
        dst[k * n + i] = src[k * cap + i];
    }
}

int grid_for(long long n, int block) {
    long long g = (n + block - 1) / block;
    return (int)(g > 16384 ? 16384 : (g < 1 ? 1 : g));
}

}  // namespace

cudaError_t launch_make_samples(const SampleArgs& a, cudaStream_t s) {
    if (a.ncell <= 0) return cudaSuccess;
    make_samples_kernel<<<grid_for(a.ncell, 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_column_stats(int nrows, int ncol, const float* X, const int* rows, double* partial, int npartial,
                                double* out, cudaStream_t s) {
    if (nrows <= 0 || ncol <= 0 || ncol > 256) return cudaErrorInvalidValue;
    const int chunk = (nrows + npartial - 1) / npartial;
    const int nblocks = (nrows + chunk - 1) / chunk;
    const int block = 256;
    column_stats_partial<<<nblocks, block, 4 * block * sizeof(double), s>>>(nrows, ncol, X, rows, chunk, partial);
    column_stats_final<<<(ncol + 63) / 64, 64, 0, s>>>(nrows, ncol, nblocks, partial, out);
    return cudaGetLastError();
}

cudaError_t launch_features(const FeatureArgs& a, cudaStream_t s) {
    if (a.n <= 0) return cudaSuccess;
    features_kernel<<<grid_for(a.n, 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_gate(const GateArgs& a, cudaStream_t s) {
    if (a.n <= 0) return cudaSuccess;
    if (a.nsp > GDTK_MAX_SPECIES || a.ne > SURR_MAX_ELEMENTS) return cudaErrorInvalidValue;
    gate_kernel<<<grid_for(a.n, 128), 128, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_gather_cells(int n, const int* idx, int ncell, int nsp, const double* rho, const double* u,
                                const double* T, const double* p, const double* dt_chem, const double* massf,
                                double* compact, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    gather_cells_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, idx, ncell, nsp, rho, u, T, p, dt_chem, massf, compact);
    return cudaGetLastError();
}

cudaError_t launch_scatter_cells(int n, const int* idx, int ncell, int nsp, const double* compact,
                                 const int* cstatus, double* T, double* p, double* dt_chem, double* massf,
                                 int* status, int* fail_count, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    scatter_cells_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, idx, ncell, nsp, compact, cstatus, T, p, dt_chem, massf,
                                                          status, fail_count);
    return cudaGetLastError();
}

cudaError_t launch_monitor_compare(int n, const int* idx, int ncell, int nsp, const double* compact,
                                   const int* cstatus, const double* T, const double* massf,
                                   unsigned long long* res, double* sum, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    monitor_compare_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, idx, ncell, nsp, compact, cstatus, T, massf, res, sum);
    return cudaGetLastError();
}

cudaError_t launch_repack(int n, int cap, int nk, const double* src, double* dst, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    repack_kernel<<<grid_for((long long)n * nk, 256), 256, 0, s>>>(n, cap, nk, src, dst);
    return cudaGetLastError();
}

}  // namespace gdtk
