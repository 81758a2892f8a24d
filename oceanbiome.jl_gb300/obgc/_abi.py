"""ctypes mirror of include/obgc.h and the loader of libobgc.so.

The structs below are field-for-field copies of the C declarations; tests check their sizes and
offsets against the compiled library (obgc_struct_layout).  Loading fails loudly when the shared
library has not been built: there is no CPU fallback for any entry point.
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libobgc.so")

# ----------------------------------------------------------------------------- enums
OBGC_OK = 0
ERR_NOT_CONVERGED, ERR_NAN = 3, 4
STATUS_NAMES = {
    0: "OBGC_OK", 1: "OBGC_ERR_INVALID_ARGUMENT", 2: "OBGC_ERR_CUDA", 3: "OBGC_ERR_NOT_CONVERGED",
    4: "OBGC_ERR_NAN", 5: "OBGC_ERR_UNSUPPORTED", 6: "OBGC_ERR_OUT_OF_MEMORY",
    7: "OBGC_ERR_NO_DEVICE", 8: "OBGC_ERR_BUSY", 9: "OBGC_ERR_TIMEOUT",
}
F32, F64 = 0, 1
PREC_F32, PREC_F64, PREC_MIXED = 0, 1, 2
NEGATIVES_NONE, NEGATIVES_SCALE, NEGATIVES_ZERO = 0, 1, 2

TRACER_NAMES = ["NO₃", "NH₄", "Fe", "N", "P", "Z", "T", "sPOM", "bPOM", "DOM", "sPON", "bPON",
                "DON", "sPOC", "bPOC", "DOC", "D", "DIC", "Alk", "O₂", "S"]
ASCII_NAMES = ["NO3", "NH4", "Fe", "N", "P", "Z", "T", "sPOM", "bPOM", "DOM", "sPON", "bPON",
               "DON", "sPOC", "bPOC", "DOC", "D", "DIC", "Alk", "O2", "S"]
NUM_NAMED = len(TRACER_NAMES)
MAX_PASSIVE = 8
MAX_GAS_CONDITIONS = 4
EXPLICIT, VERTICALLY_IMPLICIT = 0, 1
MAX_FORCINGS = 4


def PASSIVE(p):
    """Tracer code of passive tracer p (OBGC_PASSIVE)."""
    return NUM_NAMED + p
NAME_INDEX = {n: i for i, n in enumerate(TRACER_NAMES)}
NAME_INDEX.update({n: i for i, n in enumerate(ASCII_NAMES)})
for _i, _n in enumerate(ASCII_NAMES):
    globals()["OBGC_" + _n.upper()] = _i

NUT_NITRATE_AMMONIA, NUT_NITRATE_AMMONIA_IRON, NUT_NUTRIENT = 0, 1, 2
DET_TWO_PARTICLE, DET_VARIABLE_REDFIELD, DET_SINGLE, DET_NONE = 0, 1, 2, 3
LIGHT_MONDO, LIGHT_ANALYTICAL = 0, 1
LINEAR, QUADRATIC = 0, 1
PRESET_LOBSTER, PRESET_NPZD = 0, 1
SURFACE_DEFAULT, SURFACE_CONSTANT, SURFACE_FIELD = 0, 1, 2
PERIODIC, BOUNDED, FLAT = 0, 1, 2
ADVECTION_NONE, ADVECTION_WENO5 = 0, 1
FLAG_NAN, FLAG_NOT_CONVERGED, FLAG_TIMEOUT = 1, 2, 4     # enum obgc_step_flags
OUT_FCO2, OUT_PCO2, OUT_PH_FREE, OUT_PH_TOTAL, OUT_PH_SWS, OUT_H, OUT_CARBONATE, OUT_OMEGA = range(8)
DENSITY_EOS80, DENSITY_CONSTANT, DENSITY_TEOS10_POLYNOMIAL = 0, 1, 2


# ----------------------------------------------------------------------------- structs
_NPD_INT_FIELDS = ["nutrients", "detritus", "carbonate_system", "oxygen", "light_limitation",
                   "has_temperature_coefficient", "phytoplankton_mortality_formulation",
                   "grazing_concentration_formulation", "open_bottom", "reserved0"]
_NPD_DBL_FIELDS = [
    "nitrification_rate",
    "nitrate_half_saturation", "ammonia_half_saturation", "iron_half_saturation",
    "nitrate_ammonia_inhibition", "light_half_saturation", "phytoplankton_maximum_growth_rate",
    "iron_ratio", "phytoplankton_exudation_fraction", "ammonia_fraction_of_exudate",
    "temperature_coefficient", "phytoplankton_mortality_rate", "zooplankton_mortality_rate",
    "zooplankton_excretion_rate", "phytoplankton_solid_waste_fraction",
    "excretion_inorganic_fraction", "preference_for_phytoplankton", "maximum_grazing_rate",
    "grazing_half_saturation", "zooplankton_assimilation_fraction",
    "zooplankton_calcite_dissolution", "redfield_ratio", "carbon_calcite_ratio",
    "zooplankton_gut_calcite_dissolution", "phytoplankton_chlorophyll_ratio",
    "phytoplankton_sinking_speed", "zooplankton_sinking_speed",
    "remineralisation_inorganic_fraction", "small_remineralisation_rate",
    "large_remineralisation_rate", "dissolved_remineralisation_rate",
    "small_solid_waste_fraction", "detritus_redfield_ratio", "small_particle_sinking_speed",
    "large_particle_sinking_speed",
    "detritus_remineralisation_rate", "small_particle_fraction", "detritus_sinking_speed",
    "respiration_oxygen_nitrogen_ratio", "nitrification_oxygen_nitrogen_ratio",
]


class NPDParams(C.Structure):
    _fields_ = [(n, C.c_int32) for n in _NPD_INT_FIELDS] + [(n, C.c_double) for n in _NPD_DBL_FIELDS]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}

    def copy(self):
        out = NPDParams()
        C.pointer(out)[0] = self
        return out


class TwoBandParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "water_red_attenuation", "water_blue_attenuation", "chlorophyll_red_attenuation",
        "chlorophyll_blue_attenuation", "chlorophyll_red_exponent", "chlorophyll_blue_exponent",
        "pigment_ratio", "phytoplankton_chlorophyll_ratio")]


class Surface(C.Structure):
    _fields_ = [("kind", C.c_int32), ("reserved0", C.c_int32), ("value", C.c_double),
                ("field", C.c_void_p)]


class Grid(C.Structure):
    _fields_ = [("Nx", C.c_int32), ("Ny", C.c_int32), ("Nz", C.c_int32),
                ("topology_x", C.c_int32), ("topology_y", C.c_int32), ("reserved0", C.c_int32),
                ("Lx", C.c_double), ("Ly", C.c_double), ("Lz", C.c_double),
                ("stride_j", C.c_int64), ("stride_k", C.c_int64)]


class CarbonOptions(C.Structure):
    _fields_ = [("output", C.c_int32), ("density", C.c_int32), ("has_pressure", C.c_int32),
                ("ph_given", C.c_int32), ("max_iters", C.c_int32), ("warm_start", C.c_int32),
                ("density_value", C.c_double), ("initial_pH_guess", C.c_double),
                ("atol", C.c_double), ("damping", C.c_double), ("armijo_constant", C.c_double),
                ("min_damping", C.c_double), ("calcium_ion_per_salinity", C.c_double),
                ("saturation_mineral", C.c_int32), ("reserved0", C.c_int32)]


GAS_CO2, GAS_O2 = 0, 1


class GasExchange(C.Structure):
    _fields_ = [("gas", C.c_int32), ("reserved0", C.c_int32), ("k660", C.c_double * 4), ("schmidt", C.c_double * 5),
                ("wind_speed", C.c_double), ("wind_field", C.c_void_p), ("air_concentration", C.c_double),
                ("air_field", C.c_void_p), ("o2_solubility", C.c_double * 6), ("carbon", CarbonOptions)]


class MultiGParams(C.Structure):
    """obgc_multig_params (SimpleMultiGSediment, nitrogen-only form)."""
    _fields_ = [("fast_decay_rate", C.c_double), ("slow_decay_rate", C.c_double), ("fast_redfield", C.c_double),
                ("slow_redfield", C.c_double), ("fast_fraction", C.c_double), ("slow_fraction", C.c_double),
                ("refactory_fraction", C.c_double), ("sedimentation_rate", C.c_double),
                ("anoxia_half_saturation", C.c_double), ("sinking_redfield", C.c_double),
                ("nitrate_oxidation", C.c_double * 6), ("denitrification", C.c_double * 6), ("anoxic", C.c_double * 6)]


class ModelDesc(C.Structure):
    _fields_ = [("npd", NPDParams), ("light", TwoBandParams), ("surface", Surface),
                ("grid", Grid), ("precision", C.c_int32), ("advection", C.c_int32),
                ("n_passive", C.c_int32), ("carry_T", C.c_int32), ("carry_S", C.c_int32),
                ("negatives", C.c_int32), ("zero_exclude", C.c_uint32), ("reserved1", C.c_int32),
                ("invalid_fill_value", C.c_double), ("passive_tendency_of", C.c_int8 * MAX_PASSIVE)]


class Fields(C.Structure):
    _fields_ = [("tracers", C.c_void_p * NUM_NAMED), ("passive", C.c_void_p * MAX_PASSIVE),
                ("u", C.c_void_p), ("v", C.c_void_p), ("w", C.c_void_p), ("PAR", C.c_void_p),
                ("G", C.c_void_p * NUM_NAMED)]


def _fields(spec):
    """[(name, ctype)] from 'int32 a, b; double c, d[5]; ...' in declaration order."""
    out = []
    for decl in spec.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        kind, names = decl.split(None, 1)
        ct = {"int32": C.c_int32, "double": C.c_double}[kind]
        for n in names.split(","):
            n = n.strip()
            if "[" in n:
                base, cnt = n[:-1].split("[")
                out.append((base, ct * int(cnt)))
            else:
                out.append((n, ct))
    return out


class PiscesPhyto(C.Structure):
    _fields_ = _fields("""
        int32 growth_kind, silicate_limited;
        double exudated_fraction, blue_light_absorption, green_light_absorption, red_light_absorption;
        double mortality_half_saturation, linear_mortality_rate, base_quadratic_mortality, maximum_quadratic_mortality;
        double minimum_chlorophyll_ratio, maximum_chlorophyll_ratio, maximum_iron_ratio;
        double silicate_half_saturation, enhanced_silicate_half_saturation, optimal_silicate_ratio;
        double half_saturation_for_iron_uptake, threshold_for_size_dependency, size_ratio;
        double base_growth_rate, temperature_sensitivity, dark_tolerance, initial_slope_of_PI_curve,
               low_light_adaptation, basal_respiration_rate, reference_growth_rate;
        double minimum_ammonium_half_saturation, minimum_nitrate_half_saturation,
               minimum_phosphate_half_saturation, optimal_iron_quota, minimum_silicate_half_saturation,
               silicate_half_saturation_parameter""")


class PiscesZoo(C.Structure):
    _fields_ = _fields("""
        double temperature_sensitivity, maximum_grazing_rate;
        double preference_P, preference_D, preference_POC, preference_Z;
        double food_threshold_concentration, specific_food_threshold_concentration, grazing_half_saturation;
        double maximum_flux_feeding_rate, iron_ratio, minimum_growth_efficiency, non_assimilated_fraction;
        double mortality_half_saturation, quadratic_mortality, linear_mortality;
        double dissolved_excretion_fraction, undissolved_calcite_fraction""")


class PiscesParams(C.Structure):
    _fields_ = ([("nano", PiscesPhyto), ("diatoms", PiscesPhyto), ("base_rain_ratio", C.c_double),
                 ("micro", PiscesZoo), ("meso", PiscesZoo)] + _fields("""
        double micro_bacteria, meso_bacteria, maximum_bacteria, bacteria_depth_exponent;
        double doc_half_saturation_bacteria, nitrate_half_saturation_bacteria, ammonia_half_saturation_bacteria,
               phosphate_half_saturation_bacteria, iron_half_saturation_bacteria;
        double doc_remineralisation_rate, doc_bacteria_depth_exponent, doc_reference_bacteria,
               doc_temperature_sensitivity, doc_aggregation[5];
        double pom_temperature_sensitivity, pom_base_breakdown_rate, pom_aggregation[4];
        double minimum_iron_scavenging_rate, load_specific_iron_scavenging_rate, bacterial_iron_uptake_efficiency;
        double small_fraction_bacterial_iron, large_fraction_bacterial_iron, base_liable_silicate_fraction;
        double fast_dissolution_rate_of_silicate, slow_dissolution_rate_of_silicate;
        double base_calcite_dissolution_rate, calcite_dissolution_exponent;
        double maximum_iron_ratio_in_bacteria, iron_half_saturation_for_bacteria, maximum_bacterial_growth_rate;
        double maximum_nitrification_rate, maximum_fixation_rate, iron_half_saturation_for_fixation,
               phosphate_half_saturation_for_fixation, light_saturation_for_fixation;
        double excess_scavenging_enhancement, maximum_ligand_concentration, dissolved_ligand_ratio;
        double ratio_for_respiration, ratio_for_nitrification;
        double first_anoxia_threshold, second_anoxia_threshold, nitrogen_redfield_ratio, phosphate_redfield_ratio;
        double mixed_layer_shear, background_shear, latitude, day_length_coefficient;
        double poc_sinking_speed, goc_minimum_speed, goc_maximum_speed, goc_maximum_depth;
        double silicate_climatology;
        int32 open_bottom, reserved0"""))


class PiscesField(C.Structure):
    _fields_ = [("kind", C.c_int32), ("reserved0", C.c_int32), ("value", C.c_double), ("data", C.c_void_p)]


PF_CONSTANT, PF_XY, PF_XYZ, PF_ZFACE, PF_AUTO, PF_ZPROFILE = 0, 1, 2, 3, 4, 5


class PiscesModelDesc(C.Structure):
    _fields_ = [("pisces", PiscesParams), ("grid", Grid), ("precision", C.c_int32), ("advection", C.c_int32),
                ("nbands", C.c_int32), ("negatives", C.c_int32), ("kw", C.c_double * 4), ("e", C.c_double * 4),
                ("chi", C.c_double * 4), ("division", C.c_double * 4), ("surface", Surface),
                ("mixed_layer_depth", C.c_double), ("mean_kappa", C.c_double), ("invalid_fill_value", C.c_double),
                ("carbon", CarbonOptions)]

PISCES_TRACERS = ["P", "PChl", "PFe", "D", "DChl", "DFe", "DSi", "Z", "M", "DOC", "POC", "GOC", "SFe", "BFe", "PSi",
                  "CaCO₃", "NO₃", "NH₄", "PO₄", "Fe", "Si", "DIC", "Alk", "O₂", "T", "S"]
PISCES_ASCII = ["P", "PChl", "PFe", "D", "DChl", "DFe", "DSi", "Z", "M", "DOC", "POC", "GOC", "SFe", "BFe", "PSi",
                "CaCO3", "NO3", "NH4", "PO4", "Fe", "Si", "DIC", "Alk", "O2", "T", "S"]
PISCES_INDEX = {n: i for i, n in enumerate(PISCES_TRACERS)}
PISCES_INDEX.update({n: i for i, n in enumerate(PISCES_ASCII)})
PISCES_NUM_BGC = 24
PISCES_AUX = ["zmxl", "zeu", "Si_clim", "Omega", "kappa", "mixed_layer_PAR", "wPOC", "wGOC", "PAR", "PAR1", "PAR2",
              "PAR3"]


class ColumnSpec(C.Structure):
    _fields_ = [("Nz", C.c_int32), ("nsteps", C.c_int32), ("dz", C.c_double), ("dt", C.c_double),
                ("surface_PAR", C.c_double), ("mu0", C.c_double), ("pulse_step", C.c_int32),
                ("pulse_k", C.c_int32), ("pulse_amount", C.c_double), ("temperature", C.c_double),
                ("salinity", C.c_double)]


class ColumnsDesc(C.Structure):
    _fields_ = [("npd", NPDParams), ("light", TwoBandParams), ("precision", C.c_int32),
                ("pack_cells", C.c_int32), ("threads", C.c_int32), ("max_columns", C.c_int32),
                ("arena_cells", C.c_int64), ("negatives", C.c_int32), ("zero_exclude", C.c_uint32),
                ("invalid_fill_value", C.c_double), ("gas_exchange", C.c_int32), ("reserved1", C.c_int32),
                ("gas", GasExchange)]


BOX_MAX_DRIVERS = 4


class BoxDrivers(C.Structure):
    _fields_ = [("PAR", C.c_void_p), ("par_constant", C.c_double), ("n_prescribed", C.c_int32),
                ("n_forced", C.c_int32), ("prescribed_names", C.c_int32 * BOX_MAX_DRIVERS),
                ("forced_names", C.c_int32 * BOX_MAX_DRIVERS), ("prescribed", C.c_void_p * BOX_MAX_DRIVERS),
                ("forcing", C.c_void_p * BOX_MAX_DRIVERS)]


class ServiceDesc(C.Structure):
    _fields_ = [("columns", ColumnsDesc), ("chunk_steps", C.c_int32), ("max_queue", C.c_int32)]


class ServiceStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("admitted", C.c_int64), ("completed", C.c_int64),
                ("launches", C.c_int64), ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("mean_ms", C.c_double),
                ("max_ms", C.c_double), ("span_s", C.c_double)]


def default_twoband():
    """TwoBandPhotosyntheticallyActiveRadiation defaults (src/Light/2band.jl:106-117)."""
    return TwoBandParams(0.225, 0.0232, 0.037, 0.074, 0.629, 0.674, 0.7, 1.31)


# ----------------------------------------------------------------------------- loader
_lib = None


class ObgcError(RuntimeError):
    def __init__(self, status, where):
        msg = ""
        if _lib is not None:
            raw = _lib.obgc_last_error_message()
            msg = raw.decode() if raw else ""
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)} {msg}")
        self.status = status


def check(status, where):
    if status != OBGC_OK:
        raise ObgcError(status, where)
    return status


def _sig(lib, name, res, *args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = list(args)


def load():
    """Load libobgc.so (built by __graft_entry__.build()).  Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libobgc.so is not built ({LIB_PATH}); run __graft_entry__.build()")
    lib = C.CDLL(LIB_PATH)
    P, I32, I64, D, VP = C.POINTER, C.c_int32, C.c_int64, C.c_double, C.c_void_p
    _sig(lib, "obgc_abi_version", C.c_int)
    _sig(lib, "obgc_last_error_message", C.c_char_p)
    _sig(lib, "obgc_kernel_launch_count", I64)
    _sig(lib, "obgc_gas_exchange_defaults", C.c_int, I32, P(GasExchange))
    _sig(lib, "obgc_gas_exchange_flux", C.c_int, P(GasExchange), P(Grid), I32, VP, VP, VP, VP, VP, VP, VP)
    _sig(lib, "obgc_gas_exchange_point", C.c_int, P(GasExchange), D, D, D, D, D, D, D, P(D))
    _sig(lib, "obgc_set_gas_exchange", C.c_int, VP, I32, P(GasExchange))
    _sig(lib, "obgc_set_gas_exchange_on", C.c_int, VP, I32, P(GasExchange), I32, I32)
    _sig(lib, "obgc_set_forcing", C.c_int, VP, I32, VP, D, D)
    _sig(lib, "obgc_set_vertical_time_discretization", C.c_int, VP, I32)
    _sig(lib, "obgc_set_diffusivity", C.c_int, VP, D, D, P(D))
    _sig(lib, "obgc_set_sediment", C.c_int, VP, I32, P(I32), I32, D, D, D)
    _sig(lib, "obgc_sediment_storage", C.c_int, VP, P(D), P(D))
    _sig(lib, "obgc_fp64_fma_peak", C.c_int, P(D), VP)
    _sig(lib, "obgc_struct_layout", C.c_int, I32, P(I64), I32)
    _sig(lib, "obgc_npd_preset", C.c_int, I32, P(NPDParams))
    _sig(lib, "obgc_npd_required_tracers", C.c_int, P(NPDParams), P(I32), I32)
    _sig(lib, "obgc_npd_drift_velocity", C.c_int, P(NPDParams), I32, I32, P(D))
    _sig(lib, "obgc_npd_eval_point", C.c_int, P(NPDParams), I32, D, D, D, D, P(D), D, P(D))
    _sig(lib, "obgc_npd_tendencies", C.c_int, P(NPDParams), P(Grid), I32, P(VP), VP, P(VP), D, VP)
    _sig(lib, "obgc_twoband_par", C.c_int, P(TwoBandParams), P(Surface), P(Grid), I32, VP, VP, D, VP)
    _sig(lib, "obgc_multiband_par", C.c_int, I32, P(D), P(D), P(D), P(D), P(Surface), P(Grid), I32,
         VP, P(VP), VP, D, VP)
    _sig(lib, "obgc_multiband_coefficients", C.c_int, I32, P(D), I32, P(D), P(D), P(D), P(D),
         P(D), P(D), P(D))
    _sig(lib, "obgc_euphotic_depth", C.c_int, P(Surface), P(Grid), I32, VP, VP, D, D, VP)
    _sig(lib, "obgc_carbon_default_options", C.c_int, P(CarbonOptions))
    _sig(lib, "obgc_carbon_chemistry", C.c_int, P(CarbonOptions), I64, I32, VP, VP, VP, VP, VP, VP,
         VP, VP, VP, VP, VP, VP)
    _sig(lib, "obgc_carbon_chemistry_point", C.c_int, P(CarbonOptions), D, D, D, D, D, D, D, D, P(D))
    _sig(lib, "obgc_create", C.c_int, P(ModelDesc), P(VP))
    _sig(lib, "obgc_destroy", C.c_int, VP)
    _sig(lib, "obgc_bind_fields", C.c_int, VP, P(Fields))
    _sig(lib, "obgc_update_state", C.c_int, VP, D, VP)
    _sig(lib, "obgc_compute_tendencies", C.c_int, VP, D, VP)
    _sig(lib, "obgc_step", C.c_int, VP, D, D, I32, VP)
    _sig(lib, "obgc_step_graph", C.c_int, VP, D, D, I32, VP)
    _sig(lib, "obgc_last_step_timing", C.c_int, VP, P(D), P(D), P(I64))
    _sig(lib, "obgc_step_status", C.c_int, VP, P(I32))
    _sig(lib, "obgc_set_status_check", C.c_int, VP, I32)
    _sig(lib, "obgc_substep", C.c_int, VP, D, D, I32, P(VP), P(VP), VP)
    _sig(lib, "obgc_multig_default_params", C.c_int, P(MultiGParams))
    _sig(lib, "obgc_set_multig_sediment", C.c_int, VP, P(MultiGParams), I32, P(I32))
    _sig(lib, "obgc_multig_sediment_state", C.c_int, VP, P(D), P(D))
    _sig(lib, "obgc_set_staging", C.c_int, VP, I32)
    _sig(lib, "obgc_get_staging", C.c_int, VP, P(I32), P(I32))
    _sig(lib, "obgc_halo_pack", C.c_int, P(Grid), I32, I32, P(VP), I32, VP, VP, VP)
    _sig(lib, "obgc_halo_unpack", C.c_int, P(Grid), I32, I32, P(VP), I32, VP, VP, VP)
    _sig(lib, "obgc_tracer_budget", C.c_int, VP, I32, P(D), VP)
    _sig(lib, "obgc_tracer_budget_static", C.c_int, P(Grid), I32, I32, P(VP), P(D), P(D), VP)
    _sig(lib, "obgc_set_profiling", C.c_int, VP, I32)
    _sig(lib, "obgc_set_tiling", C.c_int, VP, I32)
    _sig(lib, "obgc_autotune_step", C.c_int, VP, D, D, I32, P(I32), P(I32), P(D), VP)
    _sig(lib, "obgc_box_run", C.c_int, P(NPDParams), VP, I64, VP, VP, D, D, D, I32, I32, VP, I32, VP)
    _sig(lib, "obgc_box_run_drivers", C.c_int, P(NPDParams), VP, I64, VP, P(BoxDrivers), D, D, I32, I32, VP, I32, VP)
    _sig(lib, "obgc_npd_conserved_tracers", C.c_int, P(NPDParams), I32, P(I32), P(D), I32)
    _sig(lib, "obgc_scale_negatives", C.c_int, P(Grid), I32, I32, P(VP), P(D), D, VP)
    _sig(lib, "obgc_zero_negatives", C.c_int, P(Grid), I32, I32, P(VP), VP)
    _sig(lib, "obgc_columns_create", C.c_int, P(ColumnsDesc), P(VP))
    _sig(lib, "obgc_columns_destroy", C.c_int, VP)
    _sig(lib, "obgc_columns_tracers", C.c_int, VP, P(I32), I32)
    _sig(lib, "obgc_columns_add", C.c_int, VP, P(ColumnSpec), P(D), P(D), P(I64))
    _sig(lib, "obgc_columns_advance", C.c_int, VP, I32, VP)
    _sig(lib, "obgc_columns_run", C.c_int, VP, I32, I32, I32, VP)
    _sig(lib, "obgc_columns_remaining", C.c_int, VP, I64, P(I32))
    _sig(lib, "obgc_columns_read", C.c_int, VP, I64, P(D))
    _sig(lib, "obgc_columns_remove", C.c_int, VP, I64)
    _sig(lib, "obgc_columns_autotune", C.c_int, VP, I32, P(I32), P(I32), VP)
    _sig(lib, "obgc_pisces_default_params", C.c_int, P(PiscesParams))
    _sig(lib, "obgc_pisces_eval_point", C.c_int, P(PiscesParams), P(D), P(D), D, D, P(D))
    _sig(lib, "obgc_pisces_tendencies", C.c_int, P(PiscesParams), P(Grid), I32, P(VP), P(PiscesField), P(VP), D, VP)
    _sig(lib, "obgc_mixed_layer_mean", C.c_int, P(Grid), I32, VP, P(PiscesField), VP, VP)
    _sig(lib, "obgc_pisces_calcite_saturation", C.c_int, P(CarbonOptions), P(Grid), I32, VP, VP, VP, VP, VP, VP, VP)
    _sig(lib, "obgc_pisces_model_create", C.c_int, P(PiscesModelDesc), P(VP))
    _sig(lib, "obgc_pisces_model_destroy", C.c_int, VP)
    _sig(lib, "obgc_pisces_model_bind", C.c_int, VP, P(VP), VP, VP)
    _sig(lib, "obgc_pisces_model_update_state", C.c_int, VP, D, VP)
    _sig(lib, "obgc_pisces_model_step", C.c_int, VP, D, D, I32, VP)
    _sig(lib, "obgc_pisces_model_substep", C.c_int, VP, D, D, I32, P(VP), P(VP), I32, VP)
    _sig(lib, "obgc_pisces_model_field", C.c_int, VP, I32, P(VP))
    _sig(lib, "obgc_pisces_model_read_field", C.c_int, VP, I32, P(D))
    _sig(lib, "obgc_pisces_model_set_profiling", C.c_int, VP, I32)
    _sig(lib, "obgc_pisces_model_last_timing", C.c_int, VP, P(D), P(I32))
    _sig(lib, "obgc_service_create", C.c_int, P(ServiceDesc), P(VP))
    _sig(lib, "obgc_service_destroy", C.c_int, VP)
    _sig(lib, "obgc_service_submit", C.c_int, VP, P(ColumnSpec), P(D), P(D), P(I64))
    _sig(lib, "obgc_service_wait", C.c_int, VP, I64, D, P(D), P(D))
    _sig(lib, "obgc_service_drain", C.c_int, VP, D)
    _sig(lib, "obgc_service_get_stats", C.c_int, VP, P(ServiceStats))
    _sig(lib, "obgc_service_reset_stats", C.c_int, VP)
    _sig(lib, "obgc_service_engine", C.c_int, VP, P(VP))
    _lib = lib
    return lib


# Every symbol include/obgc.h declares (checked by the CPU test suite).
EXPORTED = [
    "obgc_abi_version", "obgc_last_error_message", "obgc_kernel_launch_count", "obgc_fp64_fma_peak",
    "obgc_gas_exchange_defaults", "obgc_gas_exchange_flux", "obgc_gas_exchange_point", "obgc_set_gas_exchange",
    "obgc_set_gas_exchange_on", "obgc_set_forcing", "obgc_set_vertical_time_discretization",
    "obgc_set_diffusivity", "obgc_set_sediment", "obgc_sediment_storage",
    "obgc_npd_preset", "obgc_npd_required_tracers", "obgc_npd_drift_velocity",
    "obgc_npd_eval_point", "obgc_npd_tendencies", "obgc_twoband_par", "obgc_multiband_par",
    "obgc_multiband_coefficients", "obgc_euphotic_depth", "obgc_carbon_default_options",
    "obgc_carbon_chemistry", "obgc_carbon_chemistry_point", "obgc_create", "obgc_destroy",
    "obgc_bind_fields", "obgc_update_state", "obgc_compute_tendencies", "obgc_step",
    "obgc_step_graph", "obgc_step_status", "obgc_set_status_check", "obgc_substep", "obgc_halo_pack", "obgc_halo_unpack",
    "obgc_multig_default_params", "obgc_set_multig_sediment", "obgc_multig_sediment_state",
    "obgc_set_staging", "obgc_get_staging", "obgc_last_step_timing", "obgc_tracer_budget", "obgc_box_run", "obgc_box_run_drivers",
    "obgc_set_profiling", "obgc_set_tiling", "obgc_autotune_step", "obgc_struct_layout", "obgc_tracer_budget_static",
    "obgc_columns_create", "obgc_columns_destroy", "obgc_columns_tracers", "obgc_columns_add",
    "obgc_columns_advance", "obgc_columns_run", "obgc_columns_remaining", "obgc_columns_read", "obgc_columns_remove",
    "obgc_columns_autotune", "obgc_npd_conserved_tracers", "obgc_scale_negatives", "obgc_zero_negatives",
    "obgc_service_create", "obgc_service_destroy", "obgc_service_submit", "obgc_service_wait", "obgc_service_drain",
    "obgc_service_get_stats", "obgc_service_reset_stats", "obgc_service_engine",
    "obgc_pisces_default_params", "obgc_pisces_eval_point", "obgc_pisces_tendencies", "obgc_mixed_layer_mean",
    "obgc_pisces_calcite_saturation", "obgc_pisces_model_create", "obgc_pisces_model_destroy", "obgc_pisces_model_bind",
    "obgc_pisces_model_update_state", "obgc_pisces_model_step", "obgc_pisces_model_substep", "obgc_pisces_model_field",
    "obgc_pisces_model_read_field", "obgc_pisces_model_set_profiling", "obgc_pisces_model_last_timing",
]
