"""GB300-native engine for Eilmer's operator-split finite-rate chemistry update.

The compute path is libgdtk_chem.so (CUDA for sm_103a, built from csrc/ by buildlib.py); this
package only binds it.  `gas` mirrors the reference's Python wrapper gdtk.gas
(src/lib/gdtk/gas.py) over the libgas-compatible C ABI; `cells` drives the batch entry
points on device tensors.  There is no CPU implementation behind either: if the library
is missing, importing `lib()` raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgdtk_chem.so")
INCLUDE_H = os.path.join(os.path.dirname(HERE), "include", "gdtk_chem.h")

_lib = None

_d = ctypes.POINTER(ctypes.c_double)
_i = ctypes.POINTER(ctypes.c_int)
_c = ctypes.c_char_p
_v = ctypes.c_void_p
_ull = ctypes.POINTER(ctypes.c_ulonglong)

# name: (restype, argtypes) for every entry point of include/gdtk_chem.h and include/gdtk_surrogate.h
SIGNATURES = {
    "cwrap_gas_init": (ctypes.c_int, []),
    "gas_model_new": (ctypes.c_int, [_c]),
    "gas_model_type_str": (ctypes.c_int, [ctypes.c_int, _c, ctypes.c_int]),
    "gas_model_n_species": (ctypes.c_int, [ctypes.c_int]),
    "gas_model_n_modes": (ctypes.c_int, [ctypes.c_int]),
    "gas_model_species_name": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _c, ctypes.c_int]),
    "gas_model_mol_masses": (ctypes.c_int, [ctypes.c_int, _d]),
    "gas_state_new": (ctypes.c_int, [ctypes.c_int]),
    "gas_state_set_scalar_field": (ctypes.c_int, [ctypes.c_int, _c, ctypes.c_double]),
    "gas_state_get_scalar_field": (ctypes.c_int, [ctypes.c_int, _c, _d]),
    "gas_state_get_thermo_scalars": (ctypes.c_int, [ctypes.c_int, _d]),
    "gas_state_set_array_field": (ctypes.c_int, [ctypes.c_int, _c, _d, ctypes.c_int]),
    "gas_state_get_array_field": (ctypes.c_int, [ctypes.c_int, _c, _d, ctypes.c_int]),
    "gas_state_copy_values": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    "gas_model_gas_state_update_thermo_from_pT": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    "gas_model_gas_state_update_thermo_from_rhou": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    "gas_model_gas_state_update_thermo_from_rhoT": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    "gas_model_gas_state_update_thermo_from_rhop": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    "gas_model_gas_state_update_sound_speed": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    "gas_model_gas_state_Cv": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _d]),
    "gas_model_gas_state_Cp": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _d]),
    "gas_model_gas_state_dpdrho_const_T": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _d]),
    "gas_model_gas_state_R": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _d]),
    "gas_model_gas_state_gamma": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _d]),
    "gas_model_gas_state_internal_energy": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _d]),
    "gas_model_gas_state_enthalpy": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _d]),
    "gas_model_gas_state_entropy": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _d]),
    "gas_model_gas_state_enthalpy_isp": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _d]),
    "gas_model_gas_state_entropy_isp": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _d]),
    "gas_model_gas_state_gibbs_free_energy_isp": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _d]),
    "gas_model_gas_state_molecular_mass": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _d]),
    "gas_model_massf2molef": (ctypes.c_int, [ctypes.c_int, _d, _d]),
    "gas_model_molef2massf": (ctypes.c_int, [ctypes.c_int, _d, _d]),
    "gas_model_gas_state_get_molef": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _d]),
    "gas_model_gas_state_get_conc": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _d]),
    "thermochemical_reactor_new": (ctypes.c_int, [ctypes.c_int, _c, _c]),
    "thermochemical_reactor_gas_state_update": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_double, _d]),
    "thermochemical_reactor_eval_source_terms": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                                ctypes.c_int, ctypes.c_int, _d]),
    "reaction_mechanism_new": (ctypes.c_int, [ctypes.c_int, _c]),
    "reaction_mechanism_n_reactions": (ctypes.c_int, [ctypes.c_int]),
    "reaction_mechanism_tickrates": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _d, _d]),
    "chem_reactor_update_cells": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _v, _v, _v, _v, _v, _v, _v,
                                                 ctypes.c_double, ctypes.c_double, ctypes.c_int, _v]),
    "chem_reactor_update_cells_ex": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _v, _v, _v, _v, _v, _v, _v,
                                                    ctypes.c_double, ctypes.c_double, ctypes.c_int, _v, _v, _v]),
    "chem_reactor_update_cells_noalloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _v, _v, _v, _v, _v, _v, _v,
                                                         ctypes.c_double, ctypes.c_double, ctypes.c_int, _v]),
    "chem_reactor_update_blocks": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _v, ctypes.c_double, ctypes.c_int,
                                                  _v, _v, _v]),
    "chem_reactor_update_cells_host": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _v, _v, _v, _v, _v, _v, _v,
                                                      ctypes.c_double, ctypes.c_double, ctypes.c_int]),
    "chem_reactor_source_terms_cells": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _v, _v, _v, _v, _v, _v]),
    "gas_model_update_thermo_from_pT_cells": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _v, _v, _v, _v, _v,
                                                             _v, _v]),
    "gas_model_update_thermo_from_rhou_cells": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _v, _v, _v, _v, _v,
                                                               _v, _v]),
    "chem_reactor_flop_model": (ctypes.c_int, [ctypes.c_int, _d]),
    "chem_reactor_set_lane_stats": (ctypes.c_int, [ctypes.c_int, _v]),
    "chem_reactor_configure": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "chem_reactor_set_refill_chunk": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    "chem_reactor_info": (ctypes.c_int, [ctypes.c_int, _i, _i, _i, _i]),
    "chem_reactor2t_new": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p]),
    "chem_reactor2t_info": (ctypes.c_int, [ctypes.c_int, _i, _i, _i]),
    "chem_reactor2t_thermo_from_pT_cells": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _v, _v, _v, _v, _v, _v, _v,
                                                           _v]),
    "chem_reactor2t_update_cells": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _v, _v, _v, _v, _v, _v, _v, _v, _v,
                                                   ctypes.c_double, _v, _v]),
    "chem_reactor_last_launch": (ctypes.c_int, [ctypes.c_int, _i, _i, _i, _i]),
    "gdtk_last_error": (ctypes.c_char_p, []),
    "gdtk_generate_fast_source": (ctypes.c_int, [_c, _c, _c, ctypes.c_int]),
    "gdtk_exp_host": (ctypes.c_int, [ctypes.c_int, _d, _d]),
    "gdtk_compile_fast_source_check": (ctypes.c_int, [_c, _c, ctypes.c_int, ctypes.c_int, _c, ctypes.c_int]),
    "chem_reactor_fast_source": (ctypes.c_int, [ctypes.c_int, _c, ctypes.c_int]),
    "chem_reactor_jit_log": (ctypes.c_int, [ctypes.c_int, _c, ctypes.c_int]),
    "gdtk_measure_fp64_peak": (ctypes.c_int, [_d]),
    "gdtk_div_device": (ctypes.c_int, [ctypes.c_int] + [ctypes.c_void_p] * 5),
    # include/gdtk_surrogate.h
    "chem_surrogate_new": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong]),
    "chem_surrogate_free": (ctypes.c_int, [ctypes.c_int]),
    "chem_surrogate_dims": (ctypes.c_int, [ctypes.c_int, _i]),
    "chem_surrogate_get_params": (ctypes.c_int, [ctypes.c_int, _v]),
    "chem_surrogate_set_params": (ctypes.c_int, [ctypes.c_int, _v]),
    "chem_surrogate_get_normalisation": (ctypes.c_int, [ctypes.c_int, _v, _v, _v, _v, _v, _v]),
    "chem_surrogate_set_normalisation": (ctypes.c_int, [ctypes.c_int, _v, _v, _v, _v, _v, _v]),
    "chem_surrogate_fit_normalisation": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _v, _v, _v, _v]),
    "chem_surrogate_set_loss_weights": (ctypes.c_int, [ctypes.c_int, _v]),
    "chem_surrogate_make_samples": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _v, _v, _v, ctypes.c_double, _v, _v,
                                                   _v, _v, _v, _v, _v]),
    "chem_surrogate_train_step": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _v, _v, _v, ctypes.c_float,
                                                 ctypes.c_float, _v, _v]),
    "chem_surrogate_gradients": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _v, _v, _v, _v, _v, _v]),
    "chem_surrogate_predict": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _v, _v, _v]),
    "chem_surrogate_set_gate": (ctypes.c_int, [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                               ctypes.c_double]),
    "chem_surrogate_update_cells": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _v, _v, _v, _v, _v, _v, _v,
                                                   ctypes.c_double, ctypes.c_double, ctypes.c_int, _v, _v, _v,
                                                   ctypes.c_int, _v]),
    "chem_surrogate_error_model_new": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong]),
    "chem_surrogate_error_dims": (ctypes.c_int, [ctypes.c_int, _i]),
    "chem_surrogate_error_get_params": (ctypes.c_int, [ctypes.c_int, _v]),
    "chem_surrogate_error_set_params": (ctypes.c_int, [ctypes.c_int, _v]),
    "chem_surrogate_error_train_step": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _v, _v, _v, ctypes.c_float,
                                                       ctypes.c_float, ctypes.c_float, _v, _v]),
    "chem_surrogate_error_gradients": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _v, _v, _v, ctypes.c_float, _v, _v,
                                                      _v]),
    "chem_surrogate_predict_error": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _v, _v, _v]),
    "chem_surrogate_set_error_gate": (ctypes.c_int, [ctypes.c_int, ctypes.c_double]),
    "gdtk_mlp_gemm": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _v, ctypes.c_int, ctypes.c_int, _v,
                                     ctypes.c_int, ctypes.c_int, _v, ctypes.c_int, _v, _v, _v, ctypes.c_int,
                                     ctypes.c_int, _v]),
    "gdtk_mlp_tcgen05": (ctypes.c_int, [ctypes.c_int, _v, _v]),
}


def build():
    """Compiles the CUDA library for sm_103a (see buildlib.py)."""
    from . import buildlib
    return buildlib.build()


def lib():
    """The loaded libgdtk_chem.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libgdtk_chem.so is not built (run gdtk_gb300.build()); "
                               "this package has no CPU implementation")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def generate_fast_source(gas_file, chem_file):
    """CUDA source of the mechanism-specialised kernel (no GPU needed)."""
    L = lib()
    n = check(L.gdtk_generate_fast_source(gas_file.encode(), chem_file.encode(), None, 0), "generate source")
    buf = ctypes.create_string_buffer(n)
    check(L.gdtk_generate_fast_source(gas_file.encode(), chem_file.encode(), buf, n), "generate source")
    return buf.value.decode()


def compile_fast_source_check(gas_file, chem_file, cc=(10, 3)):
    """NVRTC-compiles the mechanism kernel for sm_<cc> (no GPU needed); returns the ptxas log."""
    buf = ctypes.create_string_buffer(1 << 16)
    check(lib().gdtk_compile_fast_source_check(gas_file.encode(), chem_file.encode(), cc[0], cc[1], buf, 1 << 16),
          "NVRTC compile")
    return buf.value.decode()


def last_error():
    return lib().gdtk_last_error().decode()


class ChemError(RuntimeError):
    pass


def check(rc, what):
    if rc < 0:
        raise ChemError("%s failed: %s" % (what, last_error()))
    return rc
