/* gdtk_chem.h -- C ABI of the GB300 chemistry-update engine (libgdtk_chem.so).
 *
 * Two groups of entry points:
 *
 * 1. The libgas-compatible subset.  Same names, signatures and 0 / -1 convention as the
 *    reference's C ABI in src/gas/gas_cwrap.d (gdtk), so that src/lib/gdtk/gas.py (CFFI) or the
 *    Ruby wrapper can bind this library in place of libgas.so for the chemistry path.  Objects
 *    are integer handles into library-owned tables; errors are a -1 return plus a message on
 *    stderr.  Every chemistry and thermo evaluation runs on the GPU; a call that needs one
 *    fails with -1 when no CUDA device is present.
 *
 * 2. Batch entry points over many cells (no counterpart in libgas; they replace the per-cell
 *    loop of lmr/simcore.d:322-340 -> fluidfvcell.d:883-997 and the legacy GPU path
 *    eilmer/cuda_gpu_chem.d:155-191).  Arrays are structure-of-arrays; mass fractions are
 *    species-major, massf[isp * ncell + cell].  The *_cells functions take DEVICE pointers and a
 *    cudaStream_t (as void*), enqueue work on that stream and return without synchronising;
 *    the *_cells_host functions take host pointers and return when the results are in them.
 */
#ifndef GDTK_CHEM_H
#define GDTK_CHEM_H

#ifdef __cplusplus
extern "C" {
#endif

/* Per-cell status codes written by the batch entry points. */
enum gdtk_cell_status {
    GDTK_CELL_OK = 0,
    GDTK_CELL_H_MIN = 1,          /* minimum step size hit (chemistry_update.d:233-238) */
    GDTK_CELL_MAX_ATTEMPTS = 2,   /* chemistry_update.d:241-247 */
    GDTK_CELL_MAX_SUBCYCLES = 3,  /* chemistry_update.d:281-289 */
    GDTK_CELL_NEWTON_FAIL = 4,    /* T from (rho, u) did not converge (therm_perf_gas_mix.d:458-466) */
    GDTK_CELL_BAD_INPUT = 5,      /* invalid density (gas_model.d:246-248) */
    GDTK_CELL_FROZEN = 6,         /* T <= T_frozen: left unchanged (fluidfvcell.d:887) */
    GDTK_CELL_CEA_RANGE = 7       /* no thermo-curve segment for T (cea_thermo_curves.d:178-181) */
};

/* Flags of chem_reactor_update_cells*. */
#define GDTK_CHEM_UPDATE_THERMO 1 /* follow the update with update_thermo_from_rhou (fluidfvcell.d:956) */
#define GDTK_CHEM_RETRY 2         /* retry a failed cell once with dt_chem = -1 (fluidfvcell.d:924-941) */
#define GDTK_CHEM_INDEX_ORDER 8   /* integrate cells in index order (default: a cheap pre-pass ranks
                                     cells by expected step count and the persistent kernel takes
                                     the most expensive first, which shortens the tail; results
                                     do not depend on the order) */
#define GDTK_CHEM_REFERENCE_ORDER 4 /* use the kernel that keeps the reference's operation order
                                       (default: the mechanism-specialised kernel, which rearranges
                                       the arithmetic to spend fewer FP64 operations) */
#define GDTK_CHEM_WARP_PER_CELL 16  /* use the warp-per-cell kernel: the reference's operation order
                                       with species and reactions spread over a warp's lanes.  It is
                                       taken without the flag for mechanisms of more than 32 species or
                                       128 reactions, which the thread-per-cell kernels do not take
                                       (the reader accepts up to 128 species and 1024 reactions) */

/* ---- 1. libgas-compatible subset (gas_cwrap.d) ---------------------------------------- */
int cwrap_gas_init(void);                                                   /* gas_cwrap.d:40-55 */
int gas_model_new(const char* file_name);                                   /* gas_cwrap.d:69-80 */
int gas_model_type_str(int gm_i, char* dest_str, int n);                    /* gas_cwrap.d:82-94 */
int gas_model_n_species(int gm_i);                                          /* gas_cwrap.d:96-105 */
int gas_model_n_modes(int gm_i);                                            /* gas_cwrap.d:107-116 */
int gas_model_species_name(int gm_i, int isp, char* dest_name, int n);      /* gas_cwrap.d:134-146 */
int gas_model_mol_masses(int gm_i, double* mm);                             /* gas_cwrap.d:148-160 */
int gas_state_new(int gm_i);                                                /* gas_cwrap.d:162-178 */
int gas_state_set_scalar_field(int gs_i, const char* field_name, double value);   /* gas_cwrap.d:180-210 */
int gas_state_get_scalar_field(int gs_i, const char* field_name, double* value);  /* gas_cwrap.d:212-252 */
int gas_state_get_thermo_scalars(int gs_i, double* values);                 /* gas_cwrap.d:254-268 */
int gas_state_set_array_field(int gs_i, const char* field_name, double* values, int n); /* gas_cwrap.d:270-294 */
int gas_state_get_array_field(int gs_i, const char* field_name, double* values, int n); /* gas_cwrap.d:296-323 */
int gas_state_copy_values(int gs_to_i, int gs_from_i);                      /* gas_cwrap.d:412-421 */
int gas_model_gas_state_update_thermo_from_pT(int gm_i, int gs_i);          /* gas_cwrap.d:469-492 */
int gas_model_gas_state_update_thermo_from_rhou(int gm_i, int gs_i);        /* gas_cwrap.d:494-517 */
int gas_model_gas_state_update_thermo_from_rhoT(int gm_i, int gs_i);        /* gas_cwrap.d:519-542 */
int gas_model_gas_state_update_thermo_from_rhop(int gm_i, int gs_i);        /* gas_cwrap.d:544-566 */
int gas_model_gas_state_update_sound_speed(int gm_i, int gs_i);             /* gas_cwrap.d:610-631 */
int gas_model_gas_state_Cv(int gm_i, int gs_i, double* result);             /* gas_cwrap.d:656-665 */
int gas_model_gas_state_Cp(int gm_i, int gs_i, double* result);             /* gas_cwrap.d:667-676 */
int gas_model_gas_state_dpdrho_const_T(int gm_i, int gs_i, double* result); /* gas_cwrap.d:678-687 */
int gas_model_gas_state_R(int gm_i, int gs_i, double* result);              /* gas_cwrap.d:689-698 */
int gas_model_gas_state_gamma(int gm_i, int gs_i, double* result);          /* gas_cwrap.d:700-709 */
int gas_model_gas_state_internal_energy(int gm_i, int gs_i, double* result);/* gas_cwrap.d:722-731 */
int gas_model_gas_state_enthalpy(int gm_i, int gs_i, double* result);       /* gas_cwrap.d:733-742 */
int gas_model_gas_state_entropy(int gm_i, int gs_i, double* result);        /* gas_cwrap.d:744-753 */
int gas_model_gas_state_enthalpy_isp(int gm_i, int gs_i, int isp, double* result);          /* :790-800 */
int gas_model_gas_state_entropy_isp(int gm_i, int gs_i, int isp, double* result);           /* :802-812 */
int gas_model_gas_state_gibbs_free_energy_isp(int gm_i, int gs_i, int isp, double* result); /* :814-824 */
int gas_model_gas_state_molecular_mass(int gm_i, int gs_i, double* result); /* gas_cwrap.d:755-764 */
int gas_model_massf2molef(int gm_i, double* massf, double* molef);          /* gas_cwrap.d:826-841 */
int gas_model_molef2massf(int gm_i, double* molef, double* massf);          /* gas_cwrap.d:843-858 */
int gas_model_gas_state_get_molef(int gm_i, int gs_i, double* molef);       /* gas_cwrap.d:860-873 */
int gas_model_gas_state_get_conc(int gm_i, int gs_i, double* conc);         /* gas_cwrap.d:875-888 */
int thermochemical_reactor_new(int gm_i, const char* filename1, const char* filename2); /* gas_cwrap.d:892-904 */
int thermochemical_reactor_gas_state_update(int cr_i, int gs_i, double t_interval,
                                            double* dt_suggest);            /* gas_cwrap.d:906-921 */
int thermochemical_reactor_eval_source_terms(int cr_i, int gm_i, int gs_i, int nsp, int nmodes,
                                             double* source);               /* gas_cwrap.d:923-941 */
int reaction_mechanism_new(int gm_i, const char* filename);                 /* gas_cwrap.d:944-955 */
int reaction_mechanism_n_reactions(int rm_i);                               /* gas_cwrap.d:957-966 */
int reaction_mechanism_tickrates(int rm_i, int gm_i, int gs_i, double* forwardrates,
                                 double* backwardrates);                    /* gas_cwrap.d:968-990 */

/* ---- 2. batch entry points ------------------------------------------------------------- */
/* One operator-split chemistry increment per cell: ChemistryUpdate.opCall
 * (chemistry_update.d:139-326) over t_interval with the cell's dt_chem as dtSuggest (in/out,
 * kinetics/thermochemical_reactor.d:44-50), inside the caller contract of
 * fluidfvcell.d:883-997 (T_frozen skip, optional retry, optional rhou update).
 * Inputs rho, u are read; T, p, massf, dt_chem are updated in place for cells whose status
 * is GDTK_CELL_OK; failed or frozen cells are left unchanged.  status may be NULL.
 * Device pointers, enqueued on `stream`.  Returns 0 or -1 (bad handle/argument, launch error).
 * One reactor handle serves one stream at a time (its work counter is shared). */
int chem_reactor_update_cells(int cr_i, int ncell, const double* rho, const double* u, double* T, double* p,
                              double* massf, double* dt_chem, int* status, double t_interval,
                              double T_frozen, int flags, void* stream);
/* As above, also recording per-cell work counters (cell_counters: int[6][ncell] = ODE step
 * attempts, RHS evaluations, rate-constant evaluations, Newton iterations, rejected attempts,
 * initial step-size estimates; may be NULL) and their sums (totals: unsigned long long[6],
 * accumulated; may be NULL). */
int chem_reactor_update_cells_ex(int cr_i, int ncell, const double* rho, const double* u, double* T, double* p,
                                 double* massf, double* dt_chem, int* status, double t_interval,
                                 double T_frozen, int flags, void* stream, int* cell_counters,
                                 unsigned long long* totals);
/* Cells of many independent blocks, each with its own interval (the multi-block batch of
 * lmr/simcore.d:322-340, where every block carries its own cell arrays).  The table is a host
 * array; the pointers in it are device pointers.  Blocks are integrated by one persistent
 * launch (per 128 blocks) whose work counter walks the cells of all blocks in table order, so
 * ordering the table by expected cost (most steps first) shortens the tail.  `first` is set
 * by the library.  The table is passed in the launch parameters: the call can be captured in a
 * CUDA graph and replayed.  cell_counters, when given, is int[6][total cells] in table order.
 * Mechanisms beyond 32 species / 128 reactions (or GDTK_CHEM_WARP_PER_CELL in flags) run one warp
 * per cell, one launch per block in table order (also capturable); cell_counters must then be NULL. */
typedef struct gdtk_cell_block {
    int ncell;
    int first;
    double t_interval;
    const double* rho;
    const double* u;
    double* T;
    double* p;
    double* massf;          /* [nsp][ncell] */
    double* dt_chem;
    int* status;            /* may be NULL */
} gdtk_cell_block;
int chem_reactor_update_blocks(int cr_i, int nblock, const gdtk_cell_block* blocks, double T_frozen, int flags,
                               void* stream, int* cell_counters, unsigned long long* totals);
/* Allocation-free form of chem_reactor_update_cells (no counterpart in the reference).  For
 * callers that cannot allocate device memory where they run the chemistry: inside CUDA graph
 * capture, under a fixed pre-reserved memory budget, or on a thread that must not take
 * cudaMalloc's device-wide synchronisation.  Same arguments and results; the per-call scratch
 * (work counter, ordering keys and visit order) comes from one static device array of about
 * 8 MiB that every GPU loading this library holds until exit, so ncell is limited to
 * 1,048,576 (larger batches are rejected with -1 and a message).  It calls no cudaMalloc or
 * cudaFree.  Its first call on a device looks up that array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.  The reactor's
 * mechanism kernel must already be loaded: one ordinary chem_reactor_update_cells call on the
 * reactor does it.  All calls share the array, so calls that overlap on the GPU (different
 * streams, or concurrent graphs) race on it; serialise them. */
int chem_reactor_update_cells_noalloc(int cr_i, int ncell, const double* rho, const double* u, double* T, double* p,
                                      double* massf, double* dt_chem, int* status, double t_interval,
                                      double T_frozen, int flags, void* stream);
/* Host-pointer form: copies in, updates, copies out, synchronises.  Page-locked host buffers
 * make the copies run at full link speed.  Returns the number of cells that failed (not
 * counting frozen ones), or -1 on error. */
int chem_reactor_update_cells_host(int cr_i, int ncell, const double* rho, const double* u, double* T, double* p,
                                   double* massf, double* dt_chem, int* status, double t_interval,
                                   double T_frozen, int flags);
/* Species source terms (kg/m^3/s) of ReactionMechanism.eval_source_terms
 * (reaction_mechanism.d:98-105): source[isp * ncell + cell].  Device pointers. */
int chem_reactor_source_terms_cells(int cr_i, int ncell, const double* rho, const double* T, const double* massf,
                                    double* source, int* status, void* stream);
/* ---- Two-temperature gas (gas/thermo/two_temperature_gas.d) and its multi-temperature thermochemical
 * reactor (kinetics/multi_temperature_thermochemical_reactor.d), the path thermochemical_reactor_new
 * (gas_cwrap.d:892-904, via init_thermochemical_reactor.d) takes for a gas with one energy mode.
 * gas_file: prep-gas output with physical_model 'two-temperature-gas'; chem_file: prep-chem output
 * (Arrhenius and Park rate constants, odeStep rkf); eem_file: prep-kinetics output (Landau-Teller
 * exchange with Millikan-White / ParkHTC / ParkHTC2 relaxation times, Marrone-Treanor coupling with
 * impartial dissociation).  Returns a handle or -1. */
int chem_reactor2t_new(const char* gas_file, const char* chem_file, const char* eem_file);
int chem_reactor2t_info(int h, int* nsp, int* nr, int* neem);
/* rho, u (translation-rotation) and u_ve (vibration-electronic) from p, T, T_ve and the mass fractions
 * (two_temperature_gas.d:84-92 updateFromPT).  Device pointers, massf[isp * ncell + cell]. */
int chem_reactor2t_thermo_from_pT_cells(int h, int ncell, const double* p, const double* T, const double* T_ve,
                                        const double* massf, double* rho, double* u, double* u_ve, void* stream);
/* One reactor update of every cell over t_interval (opCall, multi_temperature_thermochemical_reactor.d:
 * 137-294): in/out T, T_ve, p, massf, dt_chem (<= 0: estimate the first step); out u, u_ve (may be
 * NULL), status (may be NULL; the reference's failures as in chem_reactor_update_cells, a failed cell
 * keeping its input state); steps (may be NULL) += RKF step attempts.  Device pointers, stream-ordered. */
int chem_reactor2t_update_cells(int h, int ncell, const double* rho, double* T, double* T_ve, double* p,
                                double* massf, double* u, double* u_ve, double* dt_chem, int* status,
                                double t_interval, unsigned long long* steps, void* stream);
/* Gas-state thermo over many cells (therm_perf_gas_mix.d:57-73).  Device pointers. */
int gas_model_update_thermo_from_pT_cells(int gm_i, int ncell, const double* p, const double* T,
                                          const double* massf, double* rho, double* u, int* status, void* stream);
int gas_model_update_thermo_from_rhou_cells(int gm_i, int ncell, const double* rho, const double* u,
                                            const double* massf, double* T, double* p, int* status, void* stream);
/* Algorithmic FP64 operation counts of the reference algorithm for this mechanism, per unit of
 * work: out[0] per rate-constant evaluation (Gibbs energies, k_f, K_c, k_b), out[1] per RHS
 * evaluation (eval_split_rates, plus q - L for rkf), out[2] per ODE step attempt (stage
 * combinations or alpha-QSS predictor, error/convergence control, mass-fraction test),
 * out[3] per alpha-QSS corrector iteration beyond its RHS, out[4] per Newton iteration of
 * T from (rho, u).  add/sub/mul/div/sqrt count 1, exp and log 20, pow 40.  Multiplying by
 * the work counters of chem_reactor_update_cells_ex gives the FLOPs of a batch. */
int chem_reactor_flop_model(int cr_i, double* out);
/* The CUDA source generated for this reactor's mechanism-specialised kernel, and the NVRTC /
 * ptxas log of its compilation ("" before first use).  Both return the length + 1 and copy
 * at most n bytes (NUL-terminated) when dest is not NULL.  No counterpart in the reference. */
int chem_reactor_fast_source(int cr_i, char* dest, int n);
int chem_reactor_jit_log(int cr_i, char* dest, int n);
/* The same source for a gas-model file and a mechanism file, without a GPU (for inspection
 * and offline compilation checks). */
int gdtk_generate_fast_source(const char* gas_file, const char* chem_file, char* dest, int n);
/* The kernels' exponential (table-driven, Tang 1989), evaluated on the host for testing. */
int gdtk_exp_host(int n, const double* x, double* y);
/* Compiles that source with NVRTC for compute capability cc_major.cc_minor without a GPU and
 * copies the compiler log (register use) into log; 0 on success, -1 on a compile error. */
int gdtk_compile_fast_source_check(const char* gas_file, const char* chem_file, int cc_major, int cc_minor,
                                   char* log, int n);
/* Launch shape of the reactor's mechanism-specialised kernel: threads per block (a multiple of
 * 32) and resident blocks per SM it is compiled for (its register/shared-memory split).  0, 0
 * restores the default (largest block the shared-memory budget allows).  Compiles and loads the
 * variant now; later updates use it.  Used by the autotuner (gdtk_gb300/autotune.py). */
int chem_reactor_configure(int cr_i, int block, int min_blocks);
/* Work-queue refill of the mechanism-specialised kernel: with cells = 0 or 1 a warp takes, with one
 * atomic, exactly as many visit positions as it has lanes without a cell; with cells in 32..2^20 it
 * reserves that many consecutive positions per atomic and hands them out to its own lanes before
 * taking another chunk.  Only scheduling changes, never a cell's result.  Autotuner dimension. */
int chem_reactor_set_refill_chunk(int cr_i, int cells);
/* Diagnostics: when stats (device, unsigned long long[24]) is set, later fast-kernel launches
 * add, for each phase k (0 iteration, 1 rate constants, 2 right-hand side, 3 step control,
 * 4 Newton iteration, 5 cell completion, 6 refill, 7 the alpha-QSS update after a right-hand
 * side), the number of warp executions in stats[2k] and of active lanes in them in stats[2k+1].
 * A kernel generated with GDTK_PHASE_CLOCKS=1 in the environment also adds each warp's SM cycles
 * spent in phase k to stats[16 + k].  NULL turns it off.  No counterpart in the reference. */
int chem_reactor_set_lane_stats(int cr_i, unsigned long long* stats);
/* Reactor description: n species, n reactions, ODE method (0 rkf, 1 alpha-qss), tight coupling. */
int chem_reactor_info(int cr_i, int* nsp, int* nr, int* method, int* tight);
/* Launch shape of the last chem_reactor_update_cells* call on this reactor. */
int chem_reactor_last_launch(int cr_i, int* grid, int* block, int* smem_bytes, int* blocks_per_sm);
/* Text of the last error reported by this library on the calling thread ("" if none). */
const char* gdtk_last_error(void);
/* Measures this GPU's FP64 FMA throughput (TFLOP/s) with a register-resident DFMA loop. */
int gdtk_measure_fp64_peak(double* tflops);
/* The chemistry kernels' FP64 divisions and the IEEE division of the same device arrays a[n], b[n],
 * for testing: q_fast = gdtk_div (Newton-Raphson refinement of the hardware's approximate reciprocal
 * with a quotient correction), q_nr = gdtk_div_nr (without the correction); synchronises the device. */
int gdtk_div_device(int n, const double* a, const double* b, double* q_fast, double* q_nr, double* q_ieee);

#ifdef __cplusplus
}
#endif
#endif /* GDTK_CHEM_H */
