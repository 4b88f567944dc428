"""ctypes mirrors of the structs in include/mbsolve_gb300.h.

Pure data definitions: importing this module loads no native library.
"""
import ctypes as C

MBG_OK = 0
MBG_ERR_INVALID_ARGUMENT = 1
MBG_ERR_CUDA = 2
MBG_ERR_RUNTIME = 3

MBG_SOURCE_HARD, MBG_SOURCE_SOFT = 0, 1
MBG_SHAPE_TABLE, MBG_SHAPE_SECH, MBG_SHAPE_GAUSSIAN = 0, 1, 2
(MBG_RECORD_ELECTRIC, MBG_RECORD_POLAR_DT, MBG_RECORD_MAGNETIC,
 MBG_RECORD_DENSITY, MBG_RECORD_INVERSION) = range(5)
MBG_RELAX_NONE, MBG_RELAX_LINDBLAD = 0, 1
MBG_FIELD_IC_CONST, MBG_FIELD_IC_VALUES = 0, 1
MBG_BC_PMC, MBG_BC_MIRROR = 0, 1

PD = C.POINTER(C.c_double)


class mbg_qm(C.Structure):
    _fields_ = [
        ("num_levels", C.c_uint32),
        ("carrier_density", C.c_double),
        ("h_diag", PD),
        ("h_off", PD),
        ("mu_diag", PD),
        ("mu_off", PD),
        ("relax_kind", C.c_int32),
        ("scattering", PD),
        ("dephasing", PD),
    ]


class mbg_material(C.Structure):
    _fields_ = [
        ("rel_permittivity", C.c_double),
        ("rel_permeability", C.c_double),
        ("overlap_factor", C.c_double),
        ("losses", C.c_double),
        ("qm", C.POINTER(mbg_qm)),
    ]


class mbg_region(C.Structure):
    _fields_ = [
        ("material", C.c_uint32),
        ("x_start", C.c_double),
        ("x_end", C.c_double),
    ]


class mbg_device(C.Structure):
    _fields_ = [
        ("num_materials", C.c_uint32),
        ("materials", C.POINTER(mbg_material)),
        ("num_regions", C.c_uint32),
        ("regions", C.POINTER(mbg_region)),
        ("bc_kind", C.c_int32),
        ("refl_left", C.c_double),
        ("refl_right", C.c_double),
    ]


class mbg_source(C.Structure):
    _fields_ = [
        ("type", C.c_int32),
        ("shape", C.c_int32),
        ("position", C.c_double),
        ("ampl", C.c_double),
        ("freq", C.c_double),
        ("phase", C.c_double),
        ("beta_or_tau", C.c_double),
        ("phase_sin", C.c_double),
        ("table", PD),
        ("table_len", C.c_uint32),
    ]


class mbg_record(C.Structure):
    _fields_ = [
        ("type", C.c_int32),
        ("row", C.c_uint32),
        ("col", C.c_uint32),
        ("interval", C.c_double),
        ("position", C.c_double),
        ("is_complex", C.c_int32),
        ("coherence", C.c_int32),
    ]


class mbg_scenario(C.Structure):
    _fields_ = [
        ("num_gridpoints", C.c_uint32),
        ("endtime", C.c_double),
        ("num_timesteps", C.c_uint32),
        ("rho_diag", PD),
        ("rho_off", PD),
        ("rho_levels", C.c_uint32),
        ("rho_num_off", C.c_uint32),
        ("e_init_kind", C.c_int32),
        ("e_init_value", C.c_double),
        ("e_init_values", PD),
        ("h_init_kind", C.c_int32),
        ("h_init_value", C.c_double),
        ("h_init_values", PD),
        ("num_sources", C.c_uint32),
        ("sources", C.POINTER(mbg_source)),
        ("num_records", C.c_uint32),
        ("records", C.POINTER(mbg_record)),
    ]


class mbg_grid(C.Structure):
    _fields_ = [
        ("num_gridpoints", C.c_uint32),
        ("num_timesteps", C.c_uint32),
        ("gridpoint_size", C.c_double),
        ("timestep_size", C.c_double),
        ("endtime", C.c_double),
    ]


class mbg_tuning(C.Structure):
    _fields_ = [
        ("cells_per_thread", C.c_uint32),
        ("threads", C.c_uint32),
        ("depth", C.c_uint32),
        ("launches_per_graph", C.c_uint32),
        ("staging", C.c_uint32),
        ("persistent", C.c_uint32),
    ]


def dbuf(values):
    """A ctypes double array holding `values` (kept alive by the caller)."""
    vals = list(values)
    arr = (C.c_double * max(1, len(vals)))(*vals)
    return arr


class PodBundle:
    """Owns every ctypes buffer a device/scenario description points into."""

    def __init__(self):
        self.keep = []
        self.device = None
        self.scenario = None

    def hold(self, obj):
        self.keep.append(obj)
        return obj


# ---- include/mbsolve_fno.h
MBG_F32, MBG_BF16 = 0, 1
MBG_GEMM_STORE, MBG_GEMM_ACCUM, MBG_GEMM_ATOMIC = 0, 1, 2
MBG_ACT_NONE, MBG_ACT_GELU, MBG_ACT_GELU_BWD = 0, 1, 2


class mbg_gemm_segment(C.Structure):
    _fields_ = [
        ("a", C.c_void_p),
        ("b", C.c_void_p),
        ("a_sm", C.c_int64), ("a_sk", C.c_int64), ("a_sz", C.c_int64),
        ("b_sn", C.c_int64), ("b_sk", C.c_int64), ("b_sz", C.c_int64),
        ("k", C.c_int32),
        ("a_type", C.c_int32),
        ("b_type", C.c_int32),
        ("negate", C.c_int32),
    ]


class mbg_gemm_desc(C.Structure):
    _fields_ = [
        ("m", C.c_int32), ("n", C.c_int32), ("batch", C.c_int32),
        ("nseg", C.c_int32),
        ("seg", mbg_gemm_segment * 3),
        ("c", C.c_void_p),
        ("c_sm", C.c_int64), ("c_sn", C.c_int64), ("c_sz", C.c_int64),
        ("c_type", C.c_int32),
        ("mode", C.c_int32),
        ("act", C.c_int32),
        ("split_k", C.c_int32),
        ("alpha", C.c_float),
        ("bias", C.c_void_p),
        ("pre", C.c_void_p),
        ("gate", C.c_void_p),
        ("c2", C.c_void_p),
        ("c2_sm", C.c_int64), ("c2_sn", C.c_int64), ("c2_sz", C.c_int64),
        ("rowdot", C.c_void_p), ("rowdot_bias", C.c_void_p),
    ]


MBG_LAYER_LIFT, MBG_LAYER_MID, MBG_LAYER_LAST = 0, 1, 2


class mbg_fno_layer_desc(C.Structure):
    _fields_ = [
        ("mode", C.c_int32), ("act", C.c_int32),
        ("batch", C.c_int32), ("S", C.c_int32), ("W", C.c_int32),
        ("Mo", C.c_int32), ("Fi", C.c_int32), ("Hq", C.c_int32),
        ("X", C.c_void_p), ("P", C.c_void_p),
        ("v", C.c_void_p), ("Y", C.c_void_p), ("G", C.c_void_p),
        ("Wl", C.c_void_p), ("bias", C.c_void_p),
        ("v_out", C.c_void_p), ("F", C.c_void_p), ("vhT", C.c_void_p),
        ("Q1", C.c_void_p), ("bq1", C.c_void_p), ("q2", C.c_void_p),
        ("bq2", C.c_void_p), ("y", C.c_void_p),
    ]
