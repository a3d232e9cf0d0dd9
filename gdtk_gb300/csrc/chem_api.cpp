// chem_api.cpp -- the C ABI of include/gdtk_chem.h.
//
// Handle tables mirror the reference's global arrays in gas/gas_cwrap.d:35-38 (gas models,
// gas states, thermochemical reactors, reaction mechanisms).  Every physics evaluation is a
// kernel launch (chem_kernels.cu); a per-state call is a batch of one cell.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <array>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/gdtk_chem.h"
#include "api_internal.h"
#include "chem_launch.h"
#include "chem_types.h"
#include "codegen.h"
#include "fast_exp.h"
#include "mechanism.h"

namespace gdtk {
namespace {

thread_local std::string g_last_error;

void report(const std::string& msg) {
    g_last_error = msg;
    std::fprintf(stderr, "gdtk_chem: %s\n", msg.c_str());
}

struct Cuda {
    bool ok = false;
    int sm_count = 0;
    std::string why;
};

Cuda& cuda() {
    static Cuda c;
    static std::once_flag once;
    std::call_once(once, [] {
        int n = 0;
        cudaError_t e = cudaGetDeviceCount(&n);
        if (e != cudaSuccess || n == 0) {
            c.why = std::string("no CUDA device available: this library evaluates chemistry and thermo on the GPU only (") +
                    (e != cudaSuccess ? cudaGetErrorString(e) : "0 devices") + ")";
            return;
        }
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&c.sm_count, cudaDevAttrMultiProcessorCount, dev);
        c.ok = true;
    });
    return c;
}

void require_cuda() {
    if (!cuda().ok) throw std::runtime_error(cuda().why);
}

void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    void ensure(size_t want) {
        if (want <= n) return;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        check(cudaMalloc(&p, want * sizeof(T)), "cudaMalloc");
        n = want;
    }
    ~DevBuf() { if (p) cudaFree(p); }
};

struct DeviceMech {
    PackedMech host;
    int* I = nullptr;
    double* D = nullptr;
    void upload(const PackedMech& pm) {
        require_cuda();
        host = pm;
        check(cudaMalloc(&I, pm.I.size() * sizeof(int)), "cudaMalloc");
        check(cudaMalloc(&D, pm.D.size() * sizeof(double)), "cudaMalloc");
        check(cudaMemcpy(I, pm.I.data(), pm.I.size() * sizeof(int), cudaMemcpyHostToDevice), "cudaMemcpy");
        check(cudaMemcpy(D, pm.D.data(), pm.D.size() * sizeof(double), cudaMemcpyHostToDevice), "cudaMemcpy");
    }
    ~DeviceMech() {
        if (I) cudaFree(I);
        if (D) cudaFree(D);
    }
};

// Scratch for per-state (one-cell) calls and for the host-pointer batch form.
struct Staging {
    DevBuf<double> d;
    DevBuf<int> st;
    cudaStream_t stream = nullptr;
    cudaStream_t get_stream() {
        if (!stream) check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
        return stream;
    }
    ~Staging() { if (stream) cudaStreamDestroy(stream); }
};

struct GasModelObj {
    GasModelHost gm;
    std::unique_ptr<DeviceMech> dev;   // gas-only tables (no reactions), made on first GPU use
    Staging stage;
    DeviceMech& device() {
        if (!dev) {
            auto d = std::make_unique<DeviceMech>();
            d->upload(pack(gm, nullptr));
            dev = std::move(d);
        }
        return *dev;
    }
};

struct GasStateObj {
    int gm;
    double rho = 0, p = 0, T = 0, u = 0, a = 0, mu = 0, k = 0;
    std::vector<double> massf;
};

struct ReactorObj {
    int gm;
    MechanismHost mh;
    DeviceMech dev;
    int scratch = 0;
    unsigned* counter = nullptr;
    Staging stage;
    LaunchInfo last{};
    std::unique_ptr<FastKernel> fast;   // mechanism-specialised kernel, compiled on first use
    int req_block = 0, req_min_blocks = 0;   // launch shape chosen by chem_reactor_configure
    int refill_chunk = 0;                    // chem_reactor_set_refill_chunk
    unsigned long long* lane_stats = nullptr;   // when set, the fast kernel counts lane occupancy
    DevBuf<float> order_key;            // longest-first scheduling scratch
    DevBuf<int> order;
    DevBuf<int> order_hist;
    // one warp per cell: for mechanisms beyond the thread-per-cell kernels' limits, or on request
    bool large = false;                 // more than GDTK_MAX_SPECIES species or GDTK_MAX_REACTIONS reactions
    int warp_doubles = 0;
    DevBuf<int> wt_i;                   // warp-per-cell tables (WarpTables, chem_launch.h)
    DevBuf<double> wt_d;
    WarpTables wt{};
    ~ReactorObj() { if (counter) cudaFree(counter); }
};

struct MechObj {
    int gm;
    MechanismHost mh;
    DeviceMech dev;
    Staging stage;
};

std::mutex g_mu;
std::vector<std::unique_ptr<GasModelObj>> g_models;
std::vector<std::unique_ptr<GasStateObj>> g_states;
std::vector<std::unique_ptr<ReactorObj>> g_reactors;
std::vector<std::unique_ptr<MechObj>> g_mechs;

template <typename T>
T& lookup(std::vector<std::unique_ptr<T>>& v, int i, const char* what) {
    if (i < 0 || i >= (int)v.size() || !v[i]) throw std::runtime_error(std::string("invalid ") + what + " handle");
    return *v[i];
}

GasModelObj& model(int i) { return lookup(g_models, i, "gas model"); }
GasStateObj& state(int i) { return lookup(g_states, i, "gas state"); }
ReactorObj& reactor(int i) { return lookup(g_reactors, i, "thermochemical reactor"); }
MechObj& mechobj(int i) { return lookup(g_mechs, i, "reaction mechanism"); }

template <typename F>
int guarded(F&& f) {
    try {
        return f();
    } catch (std::exception& e) {
        report(e.what());
        return -1;
    }
}

// Runs one gas-service mode over `n` cells whose data sit in device buffers.
void run_service(const DeviceMech& dm, int mode, int clip, int n, double* rho, double* u, double* T, double* p,
                 const double* massf, double* out1, double* out2, int* status, cudaStream_t s) {
    GasServiceArgs a{};
    a.mech_i = dm.I;
    a.mech_d = dm.D;
    a.n_mech_i = (int)dm.host.I.size();
    a.n_mech_d = (int)dm.host.D.size();
    a.nsp_hint = dm.host.nsp;
    a.nr_hint = dm.host.nr;
    a.neff_hint = dm.host.neff;
    a.ncell = n;
    a.mode = mode;
    a.clip = clip;
    a.rho = rho; a.u = u; a.T = T; a.p = p; a.massf = massf; a.out1 = out1; a.out2 = out2; a.status = status;
    check(launch_gas_service(a, cuda().sm_count, s), "gas service launch");
}

// One-cell service on a gas state: uploads [rho, u, T, p, massf...], runs, downloads.
// Returns the cell status.  out1/out2 (host) receive nout1/nout2 values when given.
int state_service(const DeviceMech& dm, Staging& stg, int mode, int clip, GasStateObj& gs, double* out1, int nout1,
                  double* out2, int nout2) {
    require_cuda();
    const int nsp = (int)gs.massf.size();
    const size_t nd = 4 + nsp + nout1 + nout2;
    stg.d.ensure(nd);
    stg.st.ensure(1);
    cudaStream_t s = stg.get_stream();
    std::vector<double> h(nd, 0.0);
    h[0] = gs.rho; h[1] = gs.u; h[2] = gs.T; h[3] = gs.p;
    for (int i = 0; i < nsp; ++i) h[4 + i] = gs.massf[i];
    double* d = stg.d.p;
    check(cudaMemcpyAsync(d, h.data(), nd * sizeof(double), cudaMemcpyHostToDevice, s), "cudaMemcpyAsync");
    run_service(dm, mode, clip, 1, d + 0, d + 1, d + 2, d + 3, d + 4, d + 4 + nsp, d + 4 + nsp + nout1, stg.st.p, s);
    int st = 0;
    check(cudaMemcpyAsync(h.data(), d, nd * sizeof(double), cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
    check(cudaMemcpyAsync(&st, stg.st.p, sizeof(int), cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
    check(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    if (st == 0) {
        gs.rho = h[0]; gs.u = h[1]; gs.T = h[2]; gs.p = h[3];
        for (int k = 0; k < nout1; ++k) out1[k] = h[4 + nsp + k];
        for (int k = 0; k < nout2; ++k) out2[k] = h[4 + nsp + nout1 + k];
    }
    return st;
}

const char* status_text(int st) {
    switch (st) {
    case CELL_H_MIN: return "Hit the minimum allowable timestep in chemistry update.";
    case CELL_MAX_ATTEMPTS: return "Hit maximum number of step attempts within a subcycle for chemistry update.";
    case CELL_MAX_SUBCYCLES: return "Hit maximum number of subcycles while attempting chemistry update.";
    case CELL_NEWTON_FAIL: return "update_temperature_from_energy function failed to converge.";
    case CELL_BAD_INPUT: return "Invalid density.";
    case CELL_CEA_RANGE: return "Coefficients for CEA curve could not be determined.";
    default: return "chemistry update failed";
    }
}

// Fast-kernel launch of an assembled FastArgs, longest-first unless GDTK_CHEM_INDEX_ORDER.
void run_fast(ReactorObj& r, FastArgs& a, int flags, cudaStream_t s) {
    a.lane_stats = r.lane_stats;
    a.refill_chunk = r.refill_chunk;
    if (!(flags & GDTK_CHEM_INDEX_ORDER) && a.total > 1) {
        r.order_key.ensure((size_t)a.total);
        r.order.ensure((size_t)a.total);
        r.order_hist.ensure(ORDER_BUCKETS);
        check(launch_order(*r.fast, a, cuda().sm_count, r.order_key.p, r.order.p, r.order_hist.p, s),
              "ordering launch");
        a.order = r.order.p;
    }
    check(cudaMemsetAsync(r.counter, 0, sizeof(unsigned), s), "cudaMemsetAsync");
    check(launch_fast(*r.fast, a, cuda().sm_count, s, &r.last.grid, &r.last.block, &r.last.smem),
          "chemistry update launch");
    r.last.blocks_per_sm = r.fast->blocks_per_sm;
}

// Tables of the warp-per-cell kernel (layout in chem_launch.h) from the packed mechanism: reaction terms
// and third bodies, scaled tick-rate slots for coefficients above 1, the q / L gather tasks dealt whole to
// the 32 lanes longest first, and the efficiency lists transposed.
void prepare_warp_path(ReactorObj& r, const PackedMech& pm) {
    r.large = pm.nsp > GDTK_MAX_SPECIES || pm.nr > GDTK_MAX_REACTIONS;
    MechView m;
    m.bind(pm.I.data(), pm.D.data());
    const int nsp = pm.nsp, nr = pm.nr, neff = pm.neff;
    std::vector<int> tstart(nr + 1, 0), tmid(nr, 0), terms, rxeff(nr, -1), slot;
    auto term = [&](int isp, int coeff) {
        if (isp < 0 || isp >= nsp || coeff < 0 || coeff > 0xffffff) throw std::runtime_error("reaction term out of range");
        terms.push_back(isp | coeff << 8);
    };
    std::map<std::pair<int, int>, int> slot_of;   // (reaction, |nu|) -> slot
    struct Entry { int ir, nu; };
    std::vector<std::vector<Entry>> per(nsp);   // species -> (reaction, nu), ascending reaction
    for (int ir = 0; ir < nr; ++ir) {
        const int* x = m.rx(ir);
        for (int k = 0; k < x[RX_NREAC]; ++k) term(x[RX_REAC_IDX + k], x[RX_REAC_COEFF + k]);
        tmid[ir] = (int)terms.size();
        for (int k = 0; k < x[RX_NPROD]; ++k) term(x[RX_PROD_IDX + k], x[RX_PROD_COEFF + k]);
        tstart[ir + 1] = (int)terms.size();
        if (x[RX_COLLIDER]) rxeff[ir] = x[RX_EFFSET];
        for (int k = 0; k < x[RX_NPART]; ++k) {
            const int nu = x[RX_PART_NU + k];
            if (nu == 0) continue;
            const int a = nu < 0 ? -nu : nu;
            if (a > 255) throw std::runtime_error("stoichiometric coefficient out of range");
            if (a > 1 && !slot_of.count({ir, a})) {
                slot_of[{ir, a}] = (int)slot.size();
                slot.push_back(ir | a << 16);
            }
            per[x[RX_PART + k]].push_back({ir, nu});
        }
    }
    const int nslot = (int)slot.size();
    // element of w_f[nr], w_b[nr], |nu| w_f[nslot], |nu| w_b[nslot] that a (reaction, nu) term adds to q or L:
    // q gets nu w_f (nu > 0) or -nu w_b, L gets nu w_b (nu > 0) or -nu w_f (reaction_mechanism.d:82-96)
    auto index = [&](const Entry& e, bool to_L) {
        const int a = e.nu < 0 ? -e.nu : e.nu;
        const bool use_b = (e.nu > 0) == to_L;
        if (a == 1) return use_b ? nr + e.ir : e.ir;
        const int j = slot_of[{e.ir, a}];
        return 2 * nr + (use_b ? nslot : 0) + j;
    };
    if (2 * nr + 2 * nslot > 0x2000) throw std::runtime_error("too many tick-rate terms for the warp-per-cell gather");
    // tasks: the q and the L of each species, longest first onto the least-loaded lane (ties: lowest lane)
    std::vector<int> order(2 * nsp);
    for (int t = 0; t < 2 * nsp; ++t) order[t] = t;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return per[a >> 1].size() > per[b >> 1].size(); });
    std::vector<std::vector<int>> lane_tasks(32);
    std::vector<size_t> load(32, 0);
    for (int t : order) {
        if (per[t >> 1].empty()) continue;
        const int l = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        lane_tasks[l].push_back(t);
        load[l] += per[t >> 1].size();
    }
    std::vector<int> lane(33, 0), ent;
    for (int l = 0; l < 32; ++l) {
        for (int t : lane_tasks[l]) {
            const int isp = t >> 1;
            const bool to_L = t & 1;
            for (auto& e : per[isp]) ent.push_back(isp | index(e, to_L) << 8 | (to_L ? 1 : 0) << 21);
        }
        lane[l + 1] = (int)ent.size();
    }
    int maxlen = 0;
    for (int s = 0; s < neff; ++s) maxlen = std::max(maxlen, m.eff_i(s)[0]);
    std::vector<int> efflen(std::max(neff, 1), 0), effidx(std::max((size_t)maxlen * neff, (size_t)1), 0);
    std::vector<double> effval(std::max((size_t)maxlen * neff, (size_t)1), 0.0);
    for (int s = 0; s < neff; ++s) {
        const int* ei = m.eff_i(s);
        const double* ev = m.eff_d(s);
        efflen[s] = ei[0];
        for (int k = 0; k < ei[0]; ++k) {
            effidx[(size_t)k * neff + s] = ei[1 + k];
            effval[(size_t)k * neff + s] = ev[ei[1 + k]];
        }
    }
    std::vector<int> all;
    auto put = [&](const std::vector<int>& v) {
        const int off = (int)all.size();
        all.insert(all.end(), v.begin(), v.end());
        return off;
    };
    WarpTables& t = r.wt;
    t.nslot = nslot;
    t.off_tstart = put(tstart);
    t.off_tmid = put(tmid);
    t.off_terms = put(terms);
    t.off_rxeff = put(rxeff);
    t.off_slot = put(slot);
    t.off_lane = put(lane);
    t.off_ent = put(ent);
    t.n_smem_ints = (int)all.size();
    t.off_efflen = put(efflen);
    t.off_effidx = put(effidx);
    r.warp_doubles = chem_warp_doubles(nsp, nr, neff, pm.method, nslot);
    r.wt_i.ensure(all.size());
    r.wt_d.ensure(effval.size());
    check(cudaMemcpy(r.wt_i.p, all.data(), all.size() * sizeof(int), cudaMemcpyHostToDevice), "cudaMemcpy");
    check(cudaMemcpy(r.wt_d.p, effval.data(), effval.size() * sizeof(double), cudaMemcpyHostToDevice), "cudaMemcpy");
    t.gi = r.wt_i.p;
    t.eff_val = r.wt_d.p;
}

int launch_update(ReactorObj& r, int ncell, const double* rho, const double* u, double* T, double* p, double* massf,
                  double* dt_chem, int* status, double t_interval, double T_frozen, int flags, cudaStream_t s,
                  int* cell_counters, unsigned long long* totals) {
    require_cuda();
    if (ncell < 0) throw std::runtime_error("ncell must be >= 0");
    if (ncell == 0) return 0;
    if (!rho || !u || !T || !p || !massf || !dt_chem) throw std::runtime_error("null cell array");
    if (!(t_interval > 0.0)) throw std::runtime_error("t_interval must be > 0");
    if (!r.counter) check(cudaMalloc(&r.counter, sizeof(unsigned)), "cudaMalloc");
    check(cudaMemsetAsync(r.counter, 0, sizeof(unsigned), s), "cudaMemsetAsync");
    if ((flags & GDTK_CHEM_WARP_PER_CELL) || r.large) {
        if (!r.wt.gi) throw std::runtime_error("warp-per-cell tables were not uploaded");
        ChemUpdateArgs a{};
        a.mech_i = r.dev.I;
        a.mech_d = r.dev.D;
        a.n_mech_i = (int)r.dev.host.I.size();
        a.n_mech_d = (int)r.dev.host.D.size();
        a.ncell = ncell;
        a.rho = rho; a.u = u; a.T = T; a.p = p; a.massf = massf; a.dt_chem = dt_chem; a.status = status;
        a.t_interval = t_interval;
        a.T_frozen = T_frozen;
        a.flags = flags & (CHEM_FLAG_UPDATE_THERMO | CHEM_FLAG_RETRY);
        a.counter = r.counter;
        a.cell_counters = cell_counters;
        a.totals = totals;
        check(launch_chem_update_warp(a, r.mh.method, r.wt, r.warp_doubles, cuda().sm_count, s, &r.last),
              "warp-per-cell update launch");
        return 0;
    }
    if (flags & GDTK_CHEM_REFERENCE_ORDER) {
        ChemUpdateArgs a{};
        a.mech_i = r.dev.I;
        a.mech_d = r.dev.D;
        a.n_mech_i = (int)r.dev.host.I.size();
        a.n_mech_d = (int)r.dev.host.D.size();
        a.ncell = ncell;
        a.rho = rho; a.u = u; a.T = T; a.p = p; a.massf = massf; a.dt_chem = dt_chem; a.status = status;
        a.t_interval = t_interval;
        a.T_frozen = T_frozen;
        a.flags = flags & (CHEM_FLAG_UPDATE_THERMO | CHEM_FLAG_RETRY);
        a.counter = r.counter;
        a.cell_counters = cell_counters;
        a.totals = totals;
        check(launch_chem_update(a, r.mh.method, r.scratch, cuda().sm_count, s, &r.last), "chemistry update launch");
        return 0;
    }
    if (!r.fast) r.fast.reset(build_fast_kernel(model(r.gm).gm, r.mh, r.req_block, r.req_min_blocks));
    FastArgs a{};
    a.nblocks = 1;
    a.total = ncell;
    a.flags = flags & (CHEM_FLAG_UPDATE_THERMO | CHEM_FLAG_RETRY);
    a.T_frozen = T_frozen;
    a.counter = r.counter;
    a.cell_counters = cell_counters;
    a.totals = totals;
    CellBlock& b = a.blocks[0];
    b.ncell = ncell;
    b.first = 0;
    b.t_interval = t_interval;
    b.rho = rho; b.u = u; b.T = T; b.p = p; b.massf = massf; b.dt_chem = dt_chem; b.status = status;
    run_fast(r, a, flags, s);
    r.last.blocks_per_sm = r.fast->blocks_per_sm;
    return 0;
}

}  // namespace

void report_error(const std::string& msg) { report(msg); }

ReactorInternals reactor_internals(int cr_i) {
    auto& r = reactor(cr_i);
    require_cuda();
    ReactorInternals v;
    v.nsp = r.dev.host.nsp;
    v.mech_i = r.dev.I;
    v.mech_d = r.dev.D;
    v.gm = &model(r.gm).gm;
    v.sm_count = cuda().sm_count;
    return v;
}

void reactor_update(int cr_i, int ncell, const double* rho, const double* u, double* T, double* p, double* massf,
                    double* dt_chem, int* status, double t_interval, double T_frozen, int flags, cudaStream_t s) {
    launch_update(reactor(cr_i), ncell, rho, u, T, p, massf, dt_chem, status, t_interval, T_frozen, flags, s, nullptr,
                  nullptr);
}

// The fast-kernel update with caller-provided scratch (the allocation-free entry point of
// noalloc.cu).  Allocates nothing: the reactor's mechanism kernel must already be loaded (the
// first chem_reactor_update_cells call on the reactor compiles and loads it).  counter and
// hist are zeroed here on the stream; key and order are fully overwritten before use.
int update_cells_with_scratch(int cr_i, int ncell, const double* rho, const double* u, double* T, double* p,
                              double* massf, double* dt_chem, int* status, double t_interval, double T_frozen,
                              int flags, void* stream, unsigned* counter, float* key, int* order, int* hist) {
    return guarded([&] {
        auto& r = reactor(cr_i);
        if (!cuda().ok) throw std::runtime_error(cuda().why);
        if (!r.fast)
            throw std::runtime_error("chem_reactor_update_cells_noalloc: the reactor's mechanism kernel is not loaded "
                                     "yet; one chem_reactor_update_cells call on this reactor (which may allocate) "
                                     "loads it");
        if (flags & GDTK_CHEM_REFERENCE_ORDER)
            throw std::runtime_error("chem_reactor_update_cells_noalloc runs the mechanism-specialised kernel only");
        if (ncell < 0) throw std::runtime_error("ncell must be >= 0");
        if (ncell == 0) return 0;
        if (!rho || !u || !T || !p || !massf || !dt_chem) throw std::runtime_error("null cell array");
        if (!(t_interval > 0.0)) throw std::runtime_error("t_interval must be > 0");
        cudaStream_t s = (cudaStream_t)stream;
        FastArgs a{};
        a.nblocks = 1;
        a.total = ncell;
        a.flags = flags & (CHEM_FLAG_UPDATE_THERMO | CHEM_FLAG_RETRY);
        a.T_frozen = T_frozen;
        a.counter = counter;
        a.refill_chunk = r.refill_chunk;
        CellBlock& b = a.blocks[0];
        b.ncell = ncell;
        b.first = 0;
        b.t_interval = t_interval;
        b.rho = rho; b.u = u; b.T = T; b.p = p; b.massf = massf; b.dt_chem = dt_chem; b.status = status;
        if (!(flags & GDTK_CHEM_INDEX_ORDER) && ncell > 1) {
            check(launch_order(*r.fast, a, cuda().sm_count, key, order, hist, s), "ordering launch");
            a.order = order;
        }
        check(cudaMemsetAsync(counter, 0, sizeof(unsigned), s), "cudaMemsetAsync");
        int grid = 0, block = 0, smem = 0;
        check(launch_fast(*r.fast, a, cuda().sm_count, s, &grid, &block, &smem), "chemistry update launch");
        return 0;
    });
}

}  // namespace gdtk

using namespace gdtk;

extern "C" {

int cwrap_gas_init(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_reactors.clear();
    g_mechs.clear();
    g_states.clear();
    g_models.clear();
    return 0;
}

int gas_model_new(const char* file_name) {
    return guarded([&] {
        if (!file_name) throw std::runtime_error("null file name");
        auto m = std::make_unique<GasModelObj>();
        m->gm = load_gas_model(file_name);
        std::lock_guard<std::mutex> lk(g_mu);
        g_models.push_back(std::move(m));
        return (int)g_models.size() - 1;
    });
}

int gas_model_type_str(int gm_i, char* dest_str, int n) {
    return guarded([&] {
        const std::string& s = model(gm_i).gm.type_str;
        if (!dest_str || n <= 0) throw std::runtime_error("bad destination buffer");
        std::strncpy(dest_str, s.c_str(), (size_t)n);
        dest_str[n - 1] = '\0';
        return 0;
    });
}

int gas_model_n_species(int gm_i) { return guarded([&] { return model(gm_i).gm.n_species(); }); }

int gas_model_n_modes(int gm_i) { return guarded([&] { (void)model(gm_i); return 0; }); }

int gas_model_species_name(int gm_i, int isp, char* dest_name, int n) {
    return guarded([&] {
        auto& gm = model(gm_i).gm;
        if (isp < 0 || isp >= gm.n_species()) throw std::runtime_error("species index out of range");
        if (!dest_name || n <= 0) throw std::runtime_error("bad destination buffer");
        std::strncpy(dest_name, gm.names[isp].c_str(), (size_t)n);
        dest_name[n - 1] = '\0';
        return 0;
    });
}

int gas_model_mol_masses(int gm_i, double* mm) {
    return guarded([&] {
        auto& gm = model(gm_i).gm;
        for (int i = 0; i < gm.n_species(); ++i) mm[i] = gm.M[i];
        return 0;
    });
}

int gas_state_new(int gm_i) {
    return guarded([&] {
        auto& gm = model(gm_i).gm;
        auto s = std::make_unique<GasStateObj>();
        s->gm = gm_i;
        s->massf.assign(gm.n_species(), 0.0);
        if (gm.n_species() == 1) s->massf[0] = 1.0;
        std::lock_guard<std::mutex> lk(g_mu);
        g_states.push_back(std::move(s));
        return (int)g_states.size() - 1;
    });
}

int gas_state_set_scalar_field(int gs_i, const char* field_name, double value) {
    return guarded([&] {
        auto& s = state(gs_i);
        std::string f = field_name ? field_name : "";
        if (f == "rho") s.rho = value;
        else if (f == "p") s.p = value;
        else if (f == "T") s.T = value;
        else if (f == "u") s.u = value;
        else throw std::runtime_error("Cannot set field name: " + f);
        return 0;
    });
}

int gas_state_get_scalar_field(int gs_i, const char* field_name, double* value) {
    return guarded([&] {
        auto& s = state(gs_i);
        std::string f = field_name ? field_name : "";
        if (f == "rho") *value = s.rho;
        else if (f == "p") *value = s.p;
        else if (f == "T") *value = s.T;
        else if (f == "u") *value = s.u;
        else if (f == "a") *value = s.a;
        else if (f == "mu") *value = s.mu;
        else if (f == "k") *value = s.k;
        else throw std::runtime_error("Cannot get field name: " + f);
        return 0;
    });
}

int gas_state_get_thermo_scalars(int gs_i, double* values) {
    return guarded([&] {
        auto& s = state(gs_i);
        values[0] = s.rho; values[1] = s.p; values[2] = s.T; values[3] = s.u; values[4] = s.a;
        return 0;
    });
}

int gas_state_set_array_field(int gs_i, const char* field_name, double* values, int n) {
    return guarded([&] {
        auto& s = state(gs_i);
        std::string f = field_name ? field_name : "";
        if (f != "massf") throw std::runtime_error("Cannot set array field name: " + f);
        if (n != (int)s.massf.size()) throw std::runtime_error("massf length mismatch");
        for (int i = 0; i < n; ++i) s.massf[i] = values[i];
        return 0;
    });
}

int gas_state_get_array_field(int gs_i, const char* field_name, double* values, int n) {
    return guarded([&] {
        auto& s = state(gs_i);
        std::string f = field_name ? field_name : "";
        if (f != "massf") throw std::runtime_error("Cannot get array field name: " + f);
        if (n != (int)s.massf.size()) throw std::runtime_error("massf length mismatch");
        for (int i = 0; i < n; ++i) values[i] = s.massf[i];
        return 0;
    });
}

int gas_state_copy_values(int gs_to_i, int gs_from_i) {
    return guarded([&] {
        auto& to = state(gs_to_i);
        auto& from = state(gs_from_i);
        if (to.massf.size() != from.massf.size()) throw std::runtime_error("gas states of different models");
        int gm = to.gm;
        to = from;
        to.gm = gm;
        return 0;
    });
}

static int thermo_update(int gm_i, int gs_i, int mode) {
    return guarded([&] {
        auto& m = model(gm_i);
        auto& s = state(gs_i);
        if ((int)s.massf.size() != m.gm.n_species()) throw std::runtime_error("gas state does not belong to this model");
        int st = state_service(m.device(), m.stage, mode, 1, s, nullptr, 0, nullptr, 0);
        if (st) throw std::runtime_error(status_text(st));
        return 0;
    });
}

int gas_model_gas_state_update_thermo_from_pT(int gm_i, int gs_i) { return thermo_update(gm_i, gs_i, 0); }
int gas_model_gas_state_update_thermo_from_rhou(int gm_i, int gs_i) { return thermo_update(gm_i, gs_i, 1); }
int gas_model_gas_state_update_thermo_from_rhoT(int gm_i, int gs_i) { return thermo_update(gm_i, gs_i, 4); }

int gas_model_gas_state_update_thermo_from_rhop(int gm_i, int gs_i) {
    return guarded([&] {
        auto& s = state(gs_i);
        bool valid = std::isfinite(s.rho) && std::isfinite(s.p);   // gas_cwrap.d:544-566
        if (s.massf.size() > 1)
            for (double y : s.massf) valid = valid && std::isfinite(y);
        if (!valid) throw std::runtime_error("Gas state is not valid for rhop update.");
        return thermo_update(gm_i, gs_i, 7);
    });
}

}  // extern "C"

namespace {
// Mode-5 properties of a gas state at its (T, p, massf): Cv, Cp, R, u, h, s, a, dp/drho at constant T.
std::array<double, 8> state_properties(int gm_i, int gs_i) {
    auto& m = model(gm_i);
    auto& s = state(gs_i);
    if ((int)s.massf.size() != m.gm.n_species()) throw std::runtime_error("gas state does not belong to this model");
    GasStateObj tmp = s;
    std::array<double, 8> out{};
    int st = state_service(m.device(), m.stage, 5, 0, tmp, out.data(), 8, nullptr, 0);
    if (st) throw std::runtime_error(status_text(st));
    return out;
}

int state_property(int gm_i, int gs_i, int k, double* result) {
    return guarded([&] {
        if (!result) throw std::runtime_error("null result pointer");
        *result = state_properties(gm_i, gs_i)[k];
        return 0;
    });
}

// Mode-6 value `which` (0 h, 1 s, 2 g) of species isp.
int species_property(int gm_i, int gs_i, int isp, int which, double* result) {
    return guarded([&] {
        auto& m = model(gm_i);
        auto& s = state(gs_i);
        const int nsp = m.gm.n_species();
        if ((int)s.massf.size() != nsp) throw std::runtime_error("gas state does not belong to this model");
        if (isp < 0 || isp >= nsp) throw std::runtime_error("species index out of range");
        if (!result) throw std::runtime_error("null result pointer");
        GasStateObj tmp = s;
        std::vector<double> out(3 * (size_t)nsp);
        int st = state_service(m.device(), m.stage, 6, 0, tmp, out.data(), 3 * nsp, nullptr, 0);
        if (st) throw std::runtime_error(status_text(st));
        *result = out[(size_t)which * nsp + isp];
        return 0;
    });
}
}  // namespace

extern "C" {

int gas_model_gas_state_update_sound_speed(int gm_i, int gs_i) {
    return guarded([&] {
        auto& s = state(gs_i);
        bool valid = std::isfinite(s.rho) && std::isfinite(s.p) && std::isfinite(s.T);   // gas_cwrap.d:610-631
        if (s.massf.size() > 1)
            for (double y : s.massf) valid = valid && std::isfinite(y);
        if (!valid) throw std::runtime_error("Gas state is not valid for sound_speed update.");
        s.a = state_properties(gm_i, gs_i)[6];
        return 0;
    });
}

int gas_model_gas_state_Cv(int gm_i, int gs_i, double* result) { return state_property(gm_i, gs_i, 0, result); }
int gas_model_gas_state_Cp(int gm_i, int gs_i, double* result) { return state_property(gm_i, gs_i, 1, result); }
int gas_model_gas_state_dpdrho_const_T(int gm_i, int gs_i, double* result) {
    return state_property(gm_i, gs_i, 7, result);
}
int gas_model_gas_state_internal_energy(int gm_i, int gs_i, double* result) {
    return state_property(gm_i, gs_i, 3, result);
}
int gas_model_gas_state_enthalpy(int gm_i, int gs_i, double* result) { return state_property(gm_i, gs_i, 4, result); }
int gas_model_gas_state_entropy(int gm_i, int gs_i, double* result) { return state_property(gm_i, gs_i, 5, result); }

int gas_model_gas_state_gamma(int gm_i, int gs_i, double* result) {
    return guarded([&] {   // gas_model.d:205: Cp / Cv
        if (!result) throw std::runtime_error("null result pointer");
        auto v = state_properties(gm_i, gs_i);
        *result = v[1] / v[0];
        return 0;
    });
}

int gas_model_gas_state_enthalpy_isp(int gm_i, int gs_i, int isp, double* result) {
    return species_property(gm_i, gs_i, isp, 0, result);
}
int gas_model_gas_state_entropy_isp(int gm_i, int gs_i, int isp, double* result) {
    return species_property(gm_i, gs_i, isp, 1, result);
}
int gas_model_gas_state_gibbs_free_energy_isp(int gm_i, int gs_i, int isp, double* result) {
    return species_property(gm_i, gs_i, isp, 2, result);
}

int gas_model_gas_state_R(int gm_i, int gs_i, double* result) {
    return guarded([&] {
        auto& m = model(gm_i).gm;
        auto& s = state(gs_i);
        double r = 0.0;   // mass_average(Q, mR), gas_model.d:410-418
        for (int i = 0; i < m.n_species(); ++i) r += s.massf[i] * (8.31451 / m.M[i]);
        *result = r;
        return 0;
    });
}

int gas_model_gas_state_molecular_mass(int gm_i, int gs_i, double* result) {
    return guarded([&] {
        auto& m = model(gm_i).gm;
        auto& s = state(gs_i);
        double sum = 0.0;   // gas_model.d:454-462: 1 / sum(Y_i / M_i)
        for (int i = 0; i < m.n_species(); ++i) sum += s.massf[i] / m.M[i];
        *result = 1.0 / sum;
        return 0;
    });
}

int gas_model_massf2molef(int gm_i, double* massf, double* molef) {
    return guarded([&] {
        auto& m = model(gm_i).gm;
        double mix = 0.0;   // gas_model.d:454-472: M_mix = 1/sum(Y/M); X = Y M_mix / M
        for (int i = 0; i < m.n_species(); ++i) mix += massf[i] / m.M[i];
        mix = 1.0 / mix;
        for (int i = 0; i < m.n_species(); ++i) molef[i] = massf[i] * mix / m.M[i];
        return 0;
    });
}

int gas_model_molef2massf(int gm_i, double* molef, double* massf) {
    return guarded([&] {
        auto& m = model(gm_i).gm;
        double mix = 0.0;   // gas_model.d:474-482
        for (int i = 0; i < m.n_species(); ++i) mix += molef[i] * m.M[i];
        for (int i = 0; i < m.n_species(); ++i) massf[i] = molef[i] * m.M[i] / mix;
        return 0;
    });
}

int gas_model_gas_state_get_molef(int gm_i, int gs_i, double* molef) {
    return guarded([&] { return gas_model_massf2molef(gm_i, state(gs_i).massf.data(), molef); });
}

int gas_model_gas_state_get_conc(int gm_i, int gs_i, double* conc) {
    return guarded([&] {
        auto& m = model(gm_i).gm;
        auto& s = state(gs_i);
        if (std::isnan(s.rho) || s.rho <= 0.0) throw std::runtime_error("Invalid density.");
        for (int i = 0; i < m.n_species(); ++i) {   // gas_model.d:237-253
            double c = s.massf[i] * s.rho / m.M[i];
            conc[i] = c < 1.0e-30 ? 0.0 : c;
        }
        return 0;
    });
}

int thermochemical_reactor_new(int gm_i, const char* filename1, const char* filename2) {
    (void)filename2;   // a second file is used only by multi-temperature reactors
    return guarded([&] {
        auto& m = model(gm_i);
        if (!filename1) throw std::runtime_error("null file name");
        auto r = std::make_unique<ReactorObj>();
        r->gm = gm_i;
        r->mh = load_mechanism(filename1, m.gm, true);
        PackedMech pm = pack(m.gm, &r->mh);
        r->scratch = chem_scratch_doubles(pm.nsp, pm.nr, pm.neff, pm.method);
        r->dev.upload(pm);
        prepare_warp_path(*r, pm);
        std::lock_guard<std::mutex> lk(g_mu);
        g_reactors.push_back(std::move(r));
        return (int)g_reactors.size() - 1;
    });
}

int thermochemical_reactor_gas_state_update(int cr_i, int gs_i, double t_interval, double* dt_suggest) {
    return guarded([&] {
        auto& r = reactor(cr_i);
        auto& s = state(gs_i);
        const int nsp = (int)s.massf.size();
        if (nsp != r.dev.host.nsp) throw std::runtime_error("gas state does not match the reactor's gas model");
        require_cuda();
        const size_t nd = 5 + nsp;
        r.stage.d.ensure(nd);
        r.stage.st.ensure(1);
        cudaStream_t st = r.stage.get_stream();
        std::vector<double> h(nd);
        h[0] = s.rho; h[1] = s.u; h[2] = s.T; h[3] = s.p; h[4] = *dt_suggest;
        for (int i = 0; i < nsp; ++i) h[5 + i] = s.massf[i];
        double* d = r.stage.d.p;
        check(cudaMemcpyAsync(d, h.data(), nd * sizeof(double), cudaMemcpyHostToDevice, st), "cudaMemcpyAsync");
        // ThermochemicalReactor.opCall alone: no retry and no rhou update (gas_cwrap.d:906-921).
        launch_update(r, 1, d + 0, d + 1, d + 2, d + 3, d + 5, d + 4, r.stage.st.p, t_interval, -1.0e300,
                      GDTK_CHEM_REFERENCE_ORDER, st, nullptr, nullptr);
        int status = 0;
        check(cudaMemcpyAsync(h.data(), d, nd * sizeof(double), cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
        check(cudaMemcpyAsync(&status, r.stage.st.p, sizeof(int), cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
        check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
        if (status != CELL_OK) throw std::runtime_error(status_text(status));
        s.T = h[2]; s.p = h[3];
        *dt_suggest = h[4];
        for (int i = 0; i < nsp; ++i) s.massf[i] = h[5 + i];
        return 0;
    });
}

int thermochemical_reactor_eval_source_terms(int cr_i, int gm_i, int gs_i, int nsp, int nmodes, double* source) {
    return guarded([&] {
        auto& r = reactor(cr_i);
        (void)model(gm_i);
        auto& s = state(gs_i);
        if (nsp != r.dev.host.nsp || nmodes != 0) throw std::runtime_error("nsp/nmodes do not match the reactor");
        int st = state_service(r.dev, r.stage, 2, 1, s, source, nsp, nullptr, 0);
        if (st) throw std::runtime_error(status_text(st));
        return 0;
    });
}

int reaction_mechanism_new(int gm_i, const char* filename) {
    return guarded([&] {
        auto& m = model(gm_i);
        if (!filename) throw std::runtime_error("null file name");
        auto r = std::make_unique<MechObj>();
        r->gm = gm_i;
        r->mh = load_mechanism(filename, m.gm, false);
        r->mh.T_lower = 300.0;   // gas_cwrap.d:947: createReactionMechanism(..., 300.0, 30000.0)
        r->mh.T_upper = 30000.0;
        r->dev.upload(pack(m.gm, &r->mh));
        std::lock_guard<std::mutex> lk(g_mu);
        g_mechs.push_back(std::move(r));
        return (int)g_mechs.size() - 1;
    });
}

int reaction_mechanism_n_reactions(int rm_i) { return guarded([&] { return (int)mechobj(rm_i).mh.reactions.size(); }); }

int reaction_mechanism_tickrates(int rm_i, int gm_i, int gs_i, double* forwardrates, double* backwardrates) {
    return guarded([&] {
        auto& r = mechobj(rm_i);
        (void)model(gm_i);
        auto& s = state(gs_i);
        const int nr = (int)r.mh.reactions.size();
        int st = state_service(r.dev, r.stage, 3, 1, s, forwardrates, nr, backwardrates, nr);
        if (st) throw std::runtime_error(status_text(st));
        return 0;
    });
}

int chem_reactor_update_cells(int cr_i, int ncell, const double* rho, const double* u, double* T, double* p,
                              double* massf, double* dt_chem, int* status, double t_interval, double T_frozen,
                              int flags, void* stream) {
    return guarded([&] {
        return launch_update(reactor(cr_i), ncell, rho, u, T, p, massf, dt_chem, status, t_interval, T_frozen, flags,
                             (cudaStream_t)stream, nullptr, nullptr);
    });
}

int chem_reactor_update_cells_ex(int cr_i, int ncell, const double* rho, const double* u, double* T, double* p,
                                 double* massf, double* dt_chem, int* status, double t_interval, double T_frozen,
                                 int flags, void* stream, int* cell_counters, unsigned long long* totals) {
    return guarded([&] {
        return launch_update(reactor(cr_i), ncell, rho, u, T, p, massf, dt_chem, status, t_interval, T_frozen, flags,
                             (cudaStream_t)stream, cell_counters, totals);
    });
}

int chem_reactor_update_blocks(int cr_i, int nblock, const gdtk_cell_block* blocks, double T_frozen, int flags,
                               void* stream, int* cell_counters, unsigned long long* totals) {
    return guarded([&] {
        auto& r = reactor(cr_i);
        require_cuda();
        if (nblock < 0 || (nblock > 0 && !blocks)) throw std::runtime_error("bad block table");
        if (flags & GDTK_CHEM_REFERENCE_ORDER)
            throw std::runtime_error("the block API runs the fast or the warp-per-cell kernel, not the reference-order one");
        cudaStream_t s = (cudaStream_t)stream;
        if ((flags & GDTK_CHEM_WARP_PER_CELL) || r.large) {   // one warp per cell: one launch per block, in order
            if (cell_counters)
                throw std::runtime_error("per-cell counters of the block API need the thread-per-cell kernel");
            for (int k = 0; k < nblock; ++k) {
                const gdtk_cell_block& in = blocks[k];
                if (in.ncell < 0) throw std::runtime_error("negative block size");
                if (in.ncell == 0) continue;
                launch_update(r, in.ncell, in.rho, in.u, in.T, in.p, in.massf, in.dt_chem, in.status, in.t_interval,
                              T_frozen, flags | GDTK_CHEM_WARP_PER_CELL, s, nullptr, totals);
            }
            return 0;
        }
        if (!r.fast) r.fast.reset(build_fast_kernel(model(r.gm).gm, r.mh, r.req_block, r.req_min_blocks));
        if (!r.counter) check(cudaMalloc(&r.counter, sizeof(unsigned)), "cudaMalloc");
        long long done_cells = 0;
        for (int b0 = 0; b0 < nblock; b0 += FAST_MAX_BLOCKS) {   // one launch per 128 blocks
            FastArgs a{};
            a.flags = flags & (CHEM_FLAG_UPDATE_THERMO | CHEM_FLAG_RETRY);
            a.T_frozen = T_frozen;
            a.counter = r.counter;
            a.totals = totals;
            long long total = 0;
            for (int k = 0; k < FAST_MAX_BLOCKS && b0 + k < nblock; ++k) {
                const gdtk_cell_block& in = blocks[b0 + k];
                if (in.ncell < 0) throw std::runtime_error("negative block size");
                if (in.ncell > 0 && (!in.rho || !in.u || !in.T || !in.p || !in.massf || !in.dt_chem))
                    throw std::runtime_error("null cell array in a block");
                if (in.ncell > 0 && !(in.t_interval > 0.0)) throw std::runtime_error("t_interval must be > 0");
                CellBlock& b = a.blocks[a.nblocks++];
                b.ncell = in.ncell;
                b.first = (int)total;
                b.t_interval = in.t_interval;
                b.rho = in.rho; b.u = in.u; b.T = in.T; b.p = in.p; b.massf = in.massf; b.dt_chem = in.dt_chem;
                b.status = in.status;
                total += in.ncell;
            }
            if (total >= (1LL << 31)) throw std::runtime_error("too many cells in one launch");
            a.total = (int)total;
            a.cell_counters = cell_counters ? cell_counters + 0 : nullptr;
            if (cell_counters && done_cells) throw std::runtime_error("per-cell counters need <= 128 blocks");
            if (total == 0) continue;
            run_fast(r, a, flags, s);
            done_cells += total;
        }
        return 0;
    });
}

int chem_reactor_update_cells_host(int cr_i, int ncell, const double* rho, const double* u, double* T, double* p,
                                   double* massf, double* dt_chem, int* status, double t_interval, double T_frozen,
                                   int flags) {
    return guarded([&] {
        auto& r = reactor(cr_i);
        require_cuda();
        if (ncell <= 0) return 0;
        const int nsp = r.dev.host.nsp;
        const size_t n = (size_t)ncell;
        r.stage.d.ensure(n * (6 + nsp));
        r.stage.st.ensure(n);
        cudaStream_t s = r.stage.get_stream();
        double* d = r.stage.d.p;
        double *drho = d, *du = d + n, *dT = d + 2 * n, *dp = d + 3 * n, *ddt = d + 4 * n, *dmf = d + 5 * n;
        const size_t B = n * sizeof(double);
        check(cudaMemcpyAsync(drho, rho, B, cudaMemcpyHostToDevice, s), "H2D");
        check(cudaMemcpyAsync(du, u, B, cudaMemcpyHostToDevice, s), "H2D");
        check(cudaMemcpyAsync(dT, T, B, cudaMemcpyHostToDevice, s), "H2D");
        check(cudaMemcpyAsync(dp, p, B, cudaMemcpyHostToDevice, s), "H2D");
        check(cudaMemcpyAsync(ddt, dt_chem, B, cudaMemcpyHostToDevice, s), "H2D");
        check(cudaMemcpyAsync(dmf, massf, B * nsp, cudaMemcpyHostToDevice, s), "H2D");
        launch_update(r, ncell, drho, du, dT, dp, dmf, ddt, r.stage.st.p, t_interval, T_frozen, flags, s, nullptr,
                      nullptr);
        check(cudaMemcpyAsync(T, dT, B, cudaMemcpyDeviceToHost, s), "D2H");
        check(cudaMemcpyAsync(p, dp, B, cudaMemcpyDeviceToHost, s), "D2H");
        check(cudaMemcpyAsync(dt_chem, ddt, B, cudaMemcpyDeviceToHost, s), "D2H");
        check(cudaMemcpyAsync(massf, dmf, B * nsp, cudaMemcpyDeviceToHost, s), "D2H");
        std::vector<int> local;
        int* st_host = status;
        if (!st_host) { local.resize(n); st_host = local.data(); }
        check(cudaMemcpyAsync(st_host, r.stage.st.p, n * sizeof(int), cudaMemcpyDeviceToHost, s), "D2H");
        check(cudaStreamSynchronize(s), "cudaStreamSynchronize");
        int nfail = 0;
        for (size_t c = 0; c < n; ++c) nfail += (st_host[c] != CELL_OK && st_host[c] != CELL_FROZEN);
        return nfail;
    });
}

int chem_reactor_source_terms_cells(int cr_i, int ncell, const double* rho, const double* T, const double* massf,
                                    double* source, int* status, void* stream) {
    return guarded([&] {
        auto& r = reactor(cr_i);
        require_cuda();
        if (ncell <= 0) return 0;
        run_service(r.dev, 2, 1, ncell, const_cast<double*>(rho), nullptr, const_cast<double*>(T), nullptr, massf,
                    source, nullptr, status, (cudaStream_t)stream);
        return 0;
    });
}

int gas_model_update_thermo_from_pT_cells(int gm_i, int ncell, const double* p, const double* T, const double* massf,
                                          double* rho, double* u, int* status, void* stream) {
    return guarded([&] {
        auto& m = model(gm_i);
        require_cuda();
        if (ncell <= 0) return 0;
        run_service(m.device(), 0, 1, ncell, rho, u, const_cast<double*>(T), const_cast<double*>(p), massf, nullptr,
                    nullptr, status, (cudaStream_t)stream);
        return 0;
    });
}

int gas_model_update_thermo_from_rhou_cells(int gm_i, int ncell, const double* rho, const double* u,
                                            const double* massf, double* T, double* p, int* status, void* stream) {
    return guarded([&] {
        auto& m = model(gm_i);
        require_cuda();
        if (ncell <= 0) return 0;
        run_service(m.device(), 1, 1, ncell, const_cast<double*>(rho), const_cast<double*>(u), T, p, massf, nullptr,
                    nullptr, status, (cudaStream_t)stream);
        return 0;
    });
}

int chem_reactor_fast_source(int cr_i, char* dest, int n) {
    return guarded([&] {
        auto& r = reactor(cr_i);
        std::string src = r.fast ? r.fast->source : generate_fast_source(model(r.gm).gm, r.mh, 256, 1);
        if (dest && n > 0) {
            std::strncpy(dest, src.c_str(), (size_t)n);
            dest[n - 1] = '\0';
        }
        return (int)src.size() + 1;
    });
}

int chem_reactor_jit_log(int cr_i, char* dest, int n) {
    return guarded([&] {
        auto& r = reactor(cr_i);
        std::string log = r.fast ? r.fast->log : std::string();
        if (dest && n > 0) {
            std::strncpy(dest, log.c_str(), (size_t)n);
            dest[n - 1] = '\0';
        }
        return (int)log.size() + 1;
    });
}

int chem_reactor_flop_model(int cr_i, double* out) {
    return guarded([&] {
        auto& r = reactor(cr_i);
        flop_model(model(r.gm).gm, r.mh, out);
        return 0;
    });
}

int chem_reactor_configure(int cr_i, int block, int min_blocks) {
    return guarded([&] {
        auto& r = reactor(cr_i);
        require_cuda();
        std::unique_ptr<FastKernel> k(build_fast_kernel(model(r.gm).gm, r.mh, block, min_blocks));
        r.req_block = block;
        r.req_min_blocks = min_blocks;
        r.fast = std::move(k);
        return 0;
    });
}

int chem_reactor_set_refill_chunk(int cr_i, int cells) {
    return guarded([&] {
        if (!(cells == 0 || cells == 1 || (cells >= 32 && cells <= (1 << 20))))
            throw std::runtime_error("refill chunk must be 0, 1 or 32..1048576 cells");
        reactor(cr_i).refill_chunk = cells;
        return 0;
    });
}

int chem_reactor_set_lane_stats(int cr_i, unsigned long long* stats) {
    return guarded([&] {
        reactor(cr_i).lane_stats = stats;
        return 0;
    });
}

int chem_reactor_info(int cr_i, int* nsp, int* nr, int* method, int* tight) {
    return guarded([&] {
        auto& r = reactor(cr_i);
        if (nsp) *nsp = r.dev.host.nsp;
        if (nr) *nr = r.dev.host.nr;
        if (method) *method = r.mh.method;
        if (tight) *tight = r.mh.tight ? 1 : 0;
        return 0;
    });
}

int chem_reactor_last_launch(int cr_i, int* grid, int* block, int* smem_bytes, int* blocks_per_sm) {
    return guarded([&] {
        auto& r = reactor(cr_i);
        if (grid) *grid = r.last.grid;
        if (block) *block = r.last.block;
        if (smem_bytes) *smem_bytes = r.last.smem;
        if (blocks_per_sm) *blocks_per_sm = r.last.blocks_per_sm;
        return 0;
    });
}

const char* gdtk_last_error(void) { return g_last_error.c_str(); }

int gdtk_exp_host(int n, const double* x, double* y) {
    static const double tab[GDTK_EXP2_TABLE_SIZE] = GDTK_EXP2_TABLE_INIT;
    for (int i = 0; i < n; ++i) y[i] = gdtk_exp(x[i], tab);
    return 0;
}

int gdtk_compile_fast_source_check(const char* gas_file, const char* chem_file, int cc_major, int cc_minor,
                                   char* log, int n) {
    return guarded([&] {
        GasModelHost gm = load_gas_model(gas_file);
        MechanismHost mh = load_mechanism(chem_file, gm, true);
        std::string l = compile_fast_check(gm, mh, cc_major, cc_minor);
        if (log && n > 0) {
            std::strncpy(log, l.c_str(), (size_t)n);
            log[n - 1] = '\0';
        }
        return 0;
    });
}

int gdtk_generate_fast_source(const char* gas_file, const char* chem_file, char* dest, int n) {
    return guarded([&] {
        GasModelHost gm = load_gas_model(gas_file);
        MechanismHost mh = load_mechanism(chem_file, gm, true);
        std::string src = generate_fast_source(gm, mh, 256, 1);
        if (dest && n > 0) {
            std::strncpy(dest, src.c_str(), (size_t)n);
            dest[n - 1] = '\0';
        }
        return (int)src.size() + 1;
    });
}

}  // extern "C"
