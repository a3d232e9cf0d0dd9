"""Python mirror of the reference's gdtk.gas wrapper (src/lib/gdtk/gas.py) for the chemistry path.

Same class names, attribute names and call semantics as the reference (GasModel,
GasState, PyGasState, ThermochemicalReactor, ReactionMechanism), bound by ctypes to the
libgas-compatible entry points of libgdtk_chem.so instead of CFFI to libgas.so.  Each
thermo or chemistry evaluation runs on the GPU.
"""
import ctypes

from . import lib, check

PC_P_atm = 101.325e3


def _dbuf(n, values=None):
    buf = (ctypes.c_double * max(n, 1))()
    if values is not None:
        for i, v in enumerate(values):
            buf[i] = v
    return buf


class GasModel:
    """gas.py:160-420 (GasModel)."""

    def __init__(self, file_name):
        self.file_name = file_name
        self.id = check(lib().gas_model_new(file_name.encode()), "gas_model_new")
        nsp = lib().gas_model_n_species(self.id)
        names = []
        buf = ctypes.create_string_buffer(64)
        for i in range(nsp):
            check(lib().gas_model_species_name(self.id, i, buf, 64), "gas_model_species_name")
            names.append(buf.value.decode())
        self.species_names = names

    def __str__(self):
        return 'GasModel(file="%s", id=%d, species=%s)' % (self.file_name, self.id, self.species_names)

    @property
    def type_str(self):
        buf = ctypes.create_string_buffer(64)
        check(lib().gas_model_type_str(self.id, buf, 64), "gas_model_type_str")
        return buf.value.decode()

    @property
    def n_species(self):
        return lib().gas_model_n_species(self.id)

    @property
    def n_modes(self):
        return lib().gas_model_n_modes(self.id)

    @property
    def mol_masses(self):
        mm = _dbuf(self.n_species)
        check(lib().gas_model_mol_masses(self.id, mm), "gas_model_mol_masses")
        return [mm[i] for i in range(self.n_species)]

    # gas.py:210-243: each thermo update is followed by the sound-speed update.
    def update_thermo_from_pT(self, gstate):
        check(lib().gas_model_gas_state_update_thermo_from_pT(self.id, gstate.id), "update_thermo_from_pT")
        self.update_sound_speed(gstate)

    def update_thermo_from_rhou(self, gstate):
        check(lib().gas_model_gas_state_update_thermo_from_rhou(self.id, gstate.id), "update_thermo_from_rhou")
        self.update_sound_speed(gstate)

    def update_thermo_from_rhoT(self, gstate):
        check(lib().gas_model_gas_state_update_thermo_from_rhoT(self.id, gstate.id), "update_thermo_from_rhoT")
        self.update_sound_speed(gstate)

    def update_thermo_from_rhop(self, gstate):
        check(lib().gas_model_gas_state_update_thermo_from_rhop(self.id, gstate.id), "update_thermo_from_rhop")
        self.update_sound_speed(gstate)

    def update_sound_speed(self, gstate):
        check(lib().gas_model_gas_state_update_sound_speed(self.id, gstate.id), "update_sound_speed")

    def _value(self, fn, gstate, *args):
        v = ctypes.c_double()
        check(getattr(lib(), fn)(self.id, gstate.id, *args, ctypes.byref(v)), fn)
        return v.value

    # gas.py:249-306
    def Cv(self, gstate):
        return self._value("gas_model_gas_state_Cv", gstate)

    def Cp(self, gstate):
        return self._value("gas_model_gas_state_Cp", gstate)

    def dpdrho_const_T(self, gstate):
        return self._value("gas_model_gas_state_dpdrho_const_T", gstate)

    def gamma(self, gstate):
        return self._value("gas_model_gas_state_gamma", gstate)

    def internal_energy(self, gstate):
        return self._value("gas_model_gas_state_internal_energy", gstate)

    def enthalpy(self, gstate):
        return self._value("gas_model_gas_state_enthalpy", gstate)

    def entropy(self, gstate):
        return self._value("gas_model_gas_state_entropy", gstate)

    def enthalpy_isp(self, gstate, isp):
        return self._value("gas_model_gas_state_enthalpy_isp", gstate, int(isp))

    def entropy_isp(self, gstate, isp):
        return self._value("gas_model_gas_state_entropy_isp", gstate, int(isp))

    def gibbs_free_energy_isp(self, gstate, isp):
        return self._value("gas_model_gas_state_gibbs_free_energy_isp", gstate, int(isp))

    def R(self, gstate):
        v = ctypes.c_double()
        check(lib().gas_model_gas_state_R(self.id, gstate.id, ctypes.byref(v)), "R")
        return v.value

    def molecular_mass(self, gstate):
        v = ctypes.c_double()
        check(lib().gas_model_gas_state_molecular_mass(self.id, gstate.id, ctypes.byref(v)), "molecular_mass")
        return v.value

    def massf2molef(self, massf_given):
        nsp = self.n_species
        if isinstance(massf_given, dict):
            massf = [massf_given.get(name, 0.0) for name in self.species_names]
        else:
            massf = list(massf_given)
        mf, mo = _dbuf(nsp, massf), _dbuf(nsp)
        check(lib().gas_model_massf2molef(self.id, mf, mo), "massf2molef")
        return [mo[i] for i in range(nsp)]

    def molef2massf(self, molef_given):
        nsp = self.n_species
        if isinstance(molef_given, dict):
            molef = [molef_given.get(name, 0.0) for name in self.species_names]
        else:
            molef = list(molef_given)
        mo, mf = _dbuf(nsp, molef), _dbuf(nsp)
        check(lib().gas_model_molef2massf(self.id, mo, mf), "molef2massf")
        return [mf[i] for i in range(nsp)]


class GasState:
    """gas.py:349-720 (GasState): data held in the library."""

    def __init__(self, gmodel):
        self.gmodel = gmodel
        self.id = check(lib().gas_state_new(gmodel.id), "gas_state_new")
        self._v = ctypes.c_double()

    def _get(self, name):
        check(lib().gas_state_get_scalar_field(self.id, name.encode(), ctypes.byref(self._v)), "get " + name)
        return self._v.value

    def _set(self, name, value):
        check(lib().gas_state_set_scalar_field(self.id, name.encode(), float(value)), "set " + name)

    rho = property(lambda s: s._get("rho"), lambda s, v: s._set("rho", v))
    p = property(lambda s: s._get("p"), lambda s, v: s._set("p", v))
    T = property(lambda s: s._get("T"), lambda s, v: s._set("T", v))
    u = property(lambda s: s._get("u"), lambda s, v: s._set("u", v))
    a = property(lambda s: s._get("a"))
    Cv = property(lambda s: s.gmodel.Cv(s))
    Cp = property(lambda s: s.gmodel.Cp(s))
    gamma = property(lambda s: s.gmodel.gamma(s))
    R = property(lambda s: s.gmodel.R(s))
    internal_energy = property(lambda s: s.gmodel.internal_energy(s))
    enthalpy = property(lambda s: s.gmodel.enthalpy(s))
    entropy = property(lambda s: s.gmodel.entropy(s))

    @property
    def massf(self):
        n = self.gmodel.n_species
        buf = _dbuf(n)
        check(lib().gas_state_get_array_field(self.id, b"massf", buf, n), "get massf")
        return [buf[i] for i in range(n)]

    @massf.setter
    def massf(self, mf_given):
        n = self.gmodel.n_species
        if isinstance(mf_given, dict):
            mf = [mf_given.get(name, 0.0) for name in self.gmodel.species_names]
        else:
            mf = list(mf_given)
        if abs(sum(mf) - 1.0) > 1.0e-6:
            raise Exception("mass fractions do not sum to 1.")
        check(lib().gas_state_set_array_field(self.id, b"massf", _dbuf(n, mf), n), "set massf")

    @property
    def molef(self):
        n = self.gmodel.n_species
        buf = _dbuf(n)
        check(lib().gas_model_gas_state_get_molef(self.gmodel.id, self.id, buf), "get molef")
        return [buf[i] for i in range(n)]

    @molef.setter
    def molef(self, molef_given):
        self.massf = self.gmodel.molef2massf(molef_given)

    @property
    def conc(self):
        n = self.gmodel.n_species
        buf = _dbuf(n)
        check(lib().gas_model_gas_state_get_conc(self.gmodel.id, self.id, buf), "get conc")
        return [buf[i] for i in range(n)]

    def copy_values(self, other):
        check(lib().gas_state_copy_values(self.id, other.id), "copy_values")

    def update_thermo_from_pT(self):
        self.gmodel.update_thermo_from_pT(self)

    def update_thermo_from_rhou(self):
        self.gmodel.update_thermo_from_rhou(self)

    def update_thermo_from_rhoT(self):
        self.gmodel.update_thermo_from_rhoT(self)

    def update_thermo_from_rhop(self):
        self.gmodel.update_thermo_from_rhop(self)

    def update_sound_speed(self):
        self.gmodel.update_sound_speed(self)


class PyGasState:
    """gas.py:730-1000 (PyGasState): Python-side attributes over a library GasState."""

    def __init__(self, gmodel):
        self.gmodel = gmodel
        self.dgs = GasState(gmodel)
        self.rho = 0.0
        self.p = 0.0
        self.T = 0.0
        self.u = 0.0
        self.a = 0.0
        self.n_species = gmodel.n_species
        self.massf = [0.0] * self.n_species if self.n_species > 1 else [1.0]

    @property
    def id(self):
        return self.dgs.id

    @property
    def massf(self):
        return self._massf

    @massf.setter
    def massf(self, mf_given):
        if isinstance(mf_given, dict):
            self._massf = [mf_given.get(name, 0.0) for name in self.gmodel.species_names]
        else:
            self._massf = list(mf_given)

    @property
    def molef(self):
        return self.gmodel.massf2molef(self._massf)

    @molef.setter
    def molef(self, molef_given):
        self._massf = self.gmodel.molef2massf(molef_given)

    @property
    def conc(self):
        M = self.gmodel.mol_masses
        return [mf * self.rho / m for mf, m in zip(self._massf, M)]

    def copy_mass_fractions_into_dgs(self):
        if abs(sum(self._massf) - 1.0) > 1.0e-6:
            raise Exception("mass fractions do not sum to 1.")
        n = self.n_species
        check(lib().gas_state_set_array_field(self.id, b"massf", _dbuf(n, self._massf), n), "set massf")

    def update_python_data(self):
        vals = _dbuf(5)
        check(lib().gas_state_get_thermo_scalars(self.id, vals), "get thermo scalars")
        self.rho, self.p, self.T, self.u, self.a = vals[0], vals[1], vals[2], vals[3], vals[4]
        self._massf = self.dgs.massf

    def update_thermo_from_pT(self):
        self.dgs.p = self.p
        self.dgs.T = self.T
        if self.n_species > 1:
            self.copy_mass_fractions_into_dgs()
        self.gmodel.update_thermo_from_pT(self.dgs)
        self.update_python_data()

    def update_thermo_from_rhou(self):
        self.dgs.rho = self.rho
        self.dgs.u = self.u
        self.dgs.T = self.T
        if self.n_species > 1:
            self.copy_mass_fractions_into_dgs()
        self.gmodel.update_thermo_from_rhou(self.dgs)
        self.update_python_data()

    def update_thermo_from_rhoT(self):
        self.dgs.rho = self.rho
        self.dgs.T = self.T
        if self.n_species > 1:
            self.copy_mass_fractions_into_dgs()
        self.gmodel.update_thermo_from_rhoT(self.dgs)
        self.update_python_data()

    def update_thermo_from_rhop(self):
        self.dgs.rho = self.rho
        self.dgs.p = self.p
        if self.n_species > 1:
            self.copy_mass_fractions_into_dgs()
        self.gmodel.update_thermo_from_rhop(self.dgs)
        self.update_python_data()


class ThermochemicalReactor:
    """gas.py:1109-1146 (ThermochemicalReactor)."""

    def __init__(self, gmodel, filename1, filename2=""):
        self.filename1 = filename1
        self.filename2 = filename2
        self.gmodel = gmodel
        self.id = check(lib().thermochemical_reactor_new(gmodel.id, filename1.encode(), filename2.encode()),
                        "thermochemical_reactor_new")
        self.dt_suggestp = ctypes.c_double()

    def __str__(self):
        return 'ThermochemicalReactor(id=%d, gmodel.id=%d, file1="%s", file2="%s")' % \
            (self.id, self.gmodel.id, self.filename1, self.filename2)

    def update_state(self, gstate, t_interval, dt_suggest=-1.0):
        if isinstance(gstate, PyGasState):
            gstate.dgs.rho, gstate.dgs.u, gstate.dgs.T, gstate.dgs.p = gstate.rho, gstate.u, gstate.T, gstate.p
            gstate.copy_mass_fractions_into_dgs()
        self.dt_suggestp.value = dt_suggest
        flag = lib().thermochemical_reactor_gas_state_update(self.id, gstate.id, t_interval,
                                                             ctypes.byref(self.dt_suggestp))
        if flag < 0:
            raise Exception("could not update state.")
        if isinstance(gstate, PyGasState):
            gstate.update_python_data()
        return self.dt_suggestp.value

    def source_terms(self, gstate):
        nsp = self.gmodel.n_species
        nmodes = self.gmodel.n_modes
        if isinstance(gstate, PyGasState):
            gstate.dgs.rho, gstate.dgs.u, gstate.dgs.T, gstate.dgs.p = gstate.rho, gstate.u, gstate.T, gstate.p
            gstate.copy_mass_fractions_into_dgs()
        source = _dbuf(nsp + nmodes)
        flag = lib().thermochemical_reactor_eval_source_terms(self.id, self.gmodel.id, gstate.id, nsp, nmodes, source)
        if flag < 0:
            raise Exception("Could not compute source terms.")
        return [source[i] for i in range(nsp + nmodes)]


class ReactionMechanism:
    """gas.py:1150-1190 (ReactionMechanism)."""

    def __init__(self, gmodel, filename):
        self.gmodel = gmodel
        self.filename = filename
        self.id = check(lib().reaction_mechanism_new(gmodel.id, filename.encode()), "reaction_mechanism_new")

    @property
    def n_reactions(self):
        return lib().reaction_mechanism_n_reactions(self.id)

    def _tick(self, gstate):
        if isinstance(gstate, PyGasState):
            gstate.dgs.rho, gstate.dgs.u, gstate.dgs.T, gstate.dgs.p = gstate.rho, gstate.u, gstate.T, gstate.p
            gstate.copy_mass_fractions_into_dgs()
        n = self.n_reactions
        fwd, bwd = _dbuf(n), _dbuf(n)
        flag = lib().reaction_mechanism_tickrates(self.id, self.gmodel.id, gstate.id, fwd, bwd)
        if flag < 0:
            raise Exception("Could not compute reaction tickrates.")
        return [fwd[i] for i in range(n)], [bwd[i] for i in range(n)]

    def reaction_tickrates(self, gstate):
        f, b = self._tick(gstate)
        return [x - y for x, y in zip(f, b)]

    def forward_tickrates(self, gstate):
        return self._tick(gstate)[0]

    def backward_tickrates(self, gstate):
        return self._tick(gstate)[1]
