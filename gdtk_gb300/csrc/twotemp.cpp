// twotemp.cpp -- the two-temperature thermochemical reactor's C ABI (include/gdtk_chem.h):
// the gas model, reaction and energy-exchange files of a two-temperature gas (as prep-gas,
// prep-chem and prep-kinetics write them), packed for the device, and the batch update of
// twotemp_kernels.cu over device-resident cells.
#include <cuda_runtime.h>

#include <cmath>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/gdtk_chem.h"
#include "api_internal.h"
#include "cea_thermo.h"
#include "lua_table.h"
#include "mechanism.h"
#include "twotemp.h"

namespace gdtk {
namespace {

constexpr double R_universal = 8.31451;   // gas/physical_constants.d:13
constexpr double Avogadro = 6.02214e23;   // gas/physical_constants.d:19
constexpr double T_REF = 298.15;          // two_temperature_gas.d:26

void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

int species_index(const GasModelHost& gm, const std::string& name) {
    for (int i = 0; i < gm.n_species(); ++i)
        if (gm.names[i] == name) return i;
    throw std::runtime_error("energy exchange names species '" + name + "', which the gas model does not have");
}

// One relaxation-time table (relaxation_time.d:578-600 createRelaxationTime) into e.
void relaxation_time(const LuaValue& t, Eem2T& e, const GasModelHost& gm, int p, int q) {
    const std::string model = t.get("model").string();
    if (model == "Millikan-White") {
        if (e.rt < 0) e.rt = RT_MILLIKAN_WHITE;
        e.a = t.get("a").number();
        e.b = t.get("b").number();
    } else if (model == "ParkHTC" || model == "ParkHTC2") {   // relaxation_time.d:81-175
        e.rt = model == "ParkHTC" ? RT_PARK_HTC : RT_PARK_HTC2;
        e.sigma = t.get("sigma").number();
        const double mq = gm.M[q] / Avogadro, mp = gm.M[p] / Avogadro;
        e.mu = mq * mp / (mq + mp);
        const LuaValue& sub = t.get("submodel");
        if (sub.get("model").string() != "Millikan-White")
            throw std::runtime_error("Park's high-temperature correction is supported over Millikan-White only");
        relaxation_time(sub, e, gm, p, q);
    } else {
        throw std::runtime_error("relaxation-time model '" + model + "' is not supported (Millikan-White, ParkHTC, "
                                 "ParkHTC2)");
    }
}

// energy_exchange_system.d:70-89 (TwoTemperatureEnergyExchange) reading the `mechanism` table.
std::vector<Eem2T> load_energy_exchange(const std::string& path, const GasModelHost& gm, int nr) {
    LuaValue f = read_lua_file(path);
    const LuaValue& mt = f.get("mechanism");
    std::vector<Eem2T> out;
    for (long k : mt.int_keys()) {
        const LuaValue& m = mt.at(k);
        Eem2T e{};
        e.rt = -1;
        const std::string rate = m.get("rate").string();
        if (m.has("mode_p") && m.get("mode_p").number() != 0)
            throw std::runtime_error("a two-temperature gas has one energy mode (mode_p = 0)");
        if (rate == "Landau-Teller") {   // energy_exchange_mechanism.d:56-101
            e.kind = EEM_LANDAU_TELLER;
            e.p = species_index(gm, m.get("p").string());
            e.q = species_index(gm, m.get("q").string());
            relaxation_time(m.get("relaxation_time"), e, gm, e.p, e.q);
        } else if (rate == "Marrone-Treanor") {   // energy_exchange_mechanism.d:195-253
            e.kind = EEM_MARRONE_TREANOR;
            e.p = species_index(gm, m.get("p").string());
            e.reaction = (int)m.get("reaction_index").number();
            if (e.reaction < 0 || e.reaction >= nr) throw std::runtime_error("reaction_index out of range");
            const LuaValue& cm = m.get("coupling_model");   // exchange_chemistry_coupling.d:71-227, 262-276
            const std::string model = cm.get("model").string();
            e.Thetav = cm.get("Thetav").number();
            if (model == "ImpartialDissociation") {
                e.coupling = CPL_IMPARTIAL;
                e.D = cm.get("D").number();
            } else if (model == "MarroneTreanorDissociation") {
                e.coupling = CPL_MARRONE_TREANOR;
                e.D = cm.get("D").number();
                e.U = cm.get("U").number();
            } else if (model == "ModifiedMarroneTreanorDissociation") {
                e.coupling = CPL_MODIFIED_MARRONE_TREANOR;
                e.D = cm.get("T_D").number();   // a temperature here
                e.aU = cm.get("aU").number();
                e.Ustar = cm.get("Ustar").number();
                e.nb = cm.has("non_boltzmann") ? cm.get("non_boltzmann").number() : 0.0;
            } else {
                throw std::runtime_error("chemistry-vibration coupling '" + model + "' is not supported "
                                         "(ImpartialDissociation, MarroneTreanorDissociation, "
                                         "ModifiedMarroneTreanorDissociation)");
            }
        } else {
            throw std::runtime_error("energy exchange rate '" + rate + "' is not supported (Landau-Teller, "
                                     "Marrone-Treanor)");
        }
        out.push_back(e);
    }
    if (out.size() > 64) throw std::runtime_error("too many energy-exchange mechanisms (max 64)");
    return out;
}

struct Reactor2TObj {
    GasModelHost gm;
    MechanismHost mh;
    int nsp = 0, nr = 0, neem = 0, electron = -1;
    int *d_i = nullptr;
    double* d_d = nullptr;
    int n_i = 0, n_d = 0;
    Species2T* d_sp = nullptr;
    Eem2T* d_eem = nullptr;
    unsigned* d_counter = nullptr;   // work counter of the update's persistent launch
    int sm_count = 0;
    ~Reactor2TObj() {
        if (d_counter) cudaFree(d_counter);
        if (d_i) cudaFree(d_i);
        if (d_d) cudaFree(d_d);
        if (d_sp) cudaFree(d_sp);
        if (d_eem) cudaFree(d_eem);
    }
};

std::mutex g_mu;
std::vector<std::unique_ptr<Reactor2TObj>> g_reactors;

Reactor2TObj& reactor2t(int h) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (h < 0 || h >= (int)g_reactors.size() || !g_reactors[h])
        throw std::runtime_error("invalid two-temperature reactor handle " + std::to_string(h));
    return *g_reactors[h];
}

template <typename F>
int guarded2t(F&& f) {
    try {
        return f();
    } catch (std::exception& e) {
        report_error(e.what());
        return -1;
    }
}

int device_sm_count() {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
        throw std::runtime_error(std::string("no CUDA device available: this library evaluates chemistry on the "
                                             "GPU only (") + (e != cudaSuccess ? cudaGetErrorString(e) : "0 devices") +
                                 ")");
    int dev = 0, sms = 0;
    ck(cudaGetDevice(&dev), "cudaGetDevice");
    ck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute");
    return sms;
}

}  // namespace
}  // namespace gdtk

using namespace gdtk;

extern "C" int chem_reactor2t_new(const char* gas_file, const char* chem_file, const char* eem_file) {
    return guarded2t([&] {
        auto r = std::make_unique<Reactor2TObj>();
        r->gm = load_gas_model(gas_file, true);
        if (!r->gm.two_temperature)
            throw std::runtime_error(std::string(gas_file) + " is not a two-temperature gas model");
        r->mh = load_mechanism(chem_file, r->gm, true);
        if (r->mh.method != METHOD_RKF)
            throw std::runtime_error("ERROR: the multi-temperature reactor takes the rkf odeStep only "
                                     "(multi_temperature_thermochemical_reactor.d:88-101)");
        for (auto& rx : r->mh.reactions)
            if (rx.frc.pressure_dependent() || rx.frc.model == RATE_ARRHENIUS2 || rx.brc.model == RATE_ARRHENIUS2)
                throw std::runtime_error("the two-temperature reactor takes Arrhenius, Park, Marrone-Treanor, "
                                         "modified Marrone-Treanor and K_c rate constants");
        r->nsp = r->gm.n_species();
        r->nr = (int)r->mh.reactions.size();
        if (r->nsp > GDTK_MAX_SPECIES || r->nr > GDTK_MAX_REACTIONS)
            throw std::runtime_error("the two-temperature reactor takes up to " + std::to_string(GDTK_MAX_SPECIES) +
                                     " species and " + std::to_string(GDTK_MAX_REACTIONS) + " reactions");
        std::vector<Eem2T> eem = load_energy_exchange(eem_file, r->gm, r->nr);
        r->neem = (int)eem.size();
        PackedMech pm = pack(r->gm, &r->mh);
        MechView v;
        v.bind(pm.I.data(), pm.D.data());
        std::vector<Species2T> sp(r->nsp);
        for (int i = 0; i < r->nsp; ++i) {   // two_temperature_gas.d:45-80
            const double R = R_universal / r->gm.M[i];
            const int k = r->gm.particle[i];
            if (k == PARTICLE_ELECTRON) r->electron = i;
            sp[i].cp_tr = k == PARTICLE_ATOM ? 2.5 * R : (k == PARTICLE_LINEAR ? 3.5 * R : (k == PARTICLE_NONLINEAR ? 4.0 * R : 0.0));
            int err = 0;
            sp[i].h_f = cea_h(v, i, T_REF, std::log(T_REF), err);
            if (err) throw std::runtime_error("CEA curve of " + r->gm.names[i] + " cannot be evaluated at 298.15 K");
        }
        r->sm_count = device_sm_count();
        r->n_i = (int)pm.I.size();
        r->n_d = (int)pm.D.size();
        ck(cudaMalloc(&r->d_i, pm.I.size() * sizeof(int)), "cudaMalloc");
        ck(cudaMalloc(&r->d_d, pm.D.size() * sizeof(double)), "cudaMalloc");
        ck(cudaMalloc(&r->d_sp, sp.size() * sizeof(Species2T)), "cudaMalloc");
        ck(cudaMalloc(&r->d_eem, std::max<size_t>(1, eem.size()) * sizeof(Eem2T)), "cudaMalloc");
        ck(cudaMalloc(&r->d_counter, sizeof(unsigned)), "cudaMalloc");
        ck(cudaMemcpy(r->d_i, pm.I.data(), pm.I.size() * sizeof(int), cudaMemcpyHostToDevice), "cudaMemcpy");
        ck(cudaMemcpy(r->d_d, pm.D.data(), pm.D.size() * sizeof(double), cudaMemcpyHostToDevice), "cudaMemcpy");
        ck(cudaMemcpy(r->d_sp, sp.data(), sp.size() * sizeof(Species2T), cudaMemcpyHostToDevice), "cudaMemcpy");
        if (!eem.empty())
            ck(cudaMemcpy(r->d_eem, eem.data(), eem.size() * sizeof(Eem2T), cudaMemcpyHostToDevice), "cudaMemcpy");
        std::lock_guard<std::mutex> lk(g_mu);
        g_reactors.push_back(std::move(r));
        return (int)g_reactors.size() - 1;
    });
}

extern "C" int chem_reactor2t_info(int h, int* nsp, int* nr, int* neem) {
    return guarded2t([&] {
        auto& r = reactor2t(h);
        if (nsp) *nsp = r.nsp;
        if (nr) *nr = r.nr;
        if (neem) *neem = r.neem;
        return 0;
    });
}

extern "C" int chem_reactor2t_thermo_from_pT_cells(int h, int ncell, const double* p, const double* T,
                                                   const double* T_ve, const double* massf, double* rho, double* u,
                                                   double* u_ve, void* stream) {
    return guarded2t([&] {
        auto& r = reactor2t(h);
        if (ncell < 0) throw std::runtime_error("negative cell count");
        Thermo2TArgs a{};
        a.mech_i = r.d_i; a.mech_d = r.d_d; a.n_mech_i = r.n_i; a.n_mech_d = r.n_d;
        a.species = r.d_sp; a.electron = r.electron; a.ncell = ncell;
        a.p = p; a.T = T; a.Tve = T_ve; a.massf = massf; a.rho = rho; a.u = u; a.u_ve = u_ve;
        ck(launch_two_temperature_thermo_pT(a, r.sm_count, (cudaStream_t)stream), "two-temperature thermo launch");
        return 0;
    });
}

extern "C" int chem_reactor2t_update_cells(int h, int ncell, const double* rho, double* T, double* T_ve, double* p,
                                           double* massf, double* u, double* u_ve, double* dt_chem, int* status,
                                           double t_interval, unsigned long long* steps, void* stream) {
    return guarded2t([&] {
        auto& r = reactor2t(h);
        if (ncell < 0) throw std::runtime_error("negative cell count");
        if (!(t_interval > 0.0)) throw std::runtime_error("t_interval must be positive");
        TwoTArgs a{};
        a.mech_i = r.d_i; a.mech_d = r.d_d; a.n_mech_i = r.n_i; a.n_mech_d = r.n_d;
        a.species = r.d_sp; a.eem = r.d_eem; a.neem = r.neem; a.electron = r.electron;
        a.tol = r.mh.errTol; a.max_subcycles = r.mh.maxSubcycles; a.max_attempts = r.mh.maxAttempts;
        a.ncell = ncell; a.rho = rho; a.T = T; a.Tve = T_ve; a.p = p; a.massf = massf; a.u = u; a.u_ve = u_ve;
        a.dt_chem = dt_chem; a.status = status; a.t_interval = t_interval; a.steps = steps;
        a.counter = r.d_counter;
        ck(launch_two_temperature_update(a, r.sm_count, (cudaStream_t)stream), "two-temperature update launch");
        return 0;
    });
}
