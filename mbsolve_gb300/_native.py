"""ctypes binding of libmbsolve_gb300.so (include/mbsolve_gb300.h).

The library is built in-tree by mbsolve_gb300/build.py. There is no CPU
fallback: if it is missing, load() raises.
"""
import ctypes as C
import os

from . import capi_types as T

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmbsolve_gb300.so")

_lib = None


class MbgError(RuntimeError):
    """An error reported by the engine (the C++ layer throws
    std::invalid_argument / std::runtime_error for these)."""

    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            "mbsolve_gb300: CUDA engine %s is not built; run "
            "`python -c 'import __graft_entry__ as g; g.build()'`" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    P = C.POINTER
    L.mbg_version.restype = C.c_char_p
    L.mbg_last_error.restype = C.c_char_p
    L.mbg_solver_names.restype = C.c_size_t
    L.mbg_solver_names.argtypes = [C.c_char_p, C.c_size_t]
    L.mbg_scenario_grid.argtypes = [P(T.mbg_device), P(T.mbg_scenario),
                                    P(T.mbg_grid)]
    L.mbg_solver_create.argtypes = [C.c_char_p, P(T.mbg_device),
                                    P(T.mbg_scenario), P(T.mbg_tuning),
                                    P(C.c_void_p)]
    L.mbg_solver_grid.argtypes = [C.c_void_p, P(T.mbg_grid)]
    L.mbg_solver_run.argtypes = [C.c_void_p]
    L.mbg_solver_num_results.argtypes = [C.c_void_p, P(C.c_uint32)]
    L.mbg_solver_result_shape.argtypes = [C.c_void_p, C.c_uint32,
                                          P(C.c_uint32), P(C.c_uint32),
                                          P(C.c_int32)]
    L.mbg_solver_copy_result.argtypes = [C.c_void_p, C.c_uint32, T.PD, T.PD]
    L.mbg_solver_destroy.argtypes = [C.c_void_p]
    L.mbg_ensemble_create.argtypes = [C.c_char_p, C.c_uint32,
                                      P(P(T.mbg_device)),
                                      P(P(T.mbg_scenario)),
                                      P(T.mbg_tuning), P(C.c_void_p)]
    L.mbg_ensemble_advance.argtypes = [C.c_void_p, C.c_uint32]
    L.mbg_ensemble_run.argtypes = [C.c_void_p]
    L.mbg_ensemble_progress.argtypes = [C.c_void_p, P(C.c_uint64),
                                        P(C.c_uint64)]
    L.mbg_ensemble_grid.argtypes = [C.c_void_p, C.c_uint32, P(T.mbg_grid)]
    L.mbg_ensemble_result_shape.argtypes = [C.c_void_p, C.c_uint32,
                                            C.c_uint32, P(C.c_uint32),
                                            P(C.c_uint32), P(C.c_int32)]
    L.mbg_ensemble_copy_result.argtypes = [C.c_void_p, C.c_uint32,
                                           C.c_uint32, T.PD, T.PD]
    L.mbg_ensemble_copy_probe_rows.argtypes = [C.c_void_p, C.c_uint32,
                                               C.c_uint64, C.c_uint64, T.PD]
    L.mbg_ensemble_info.argtypes = [C.c_void_p, P(C.c_uint64),
                                    P(C.c_uint32), P(T.mbg_tuning)]
    L.mbg_ensemble_set_timing.argtypes = [C.c_void_p, C.c_int]
    L.mbg_ensemble_kernel_time.argtypes = [C.c_void_p, P(C.c_uint64),
                                           P(C.c_double), C.c_int]
    L.mbg_ensemble_status.argtypes = [C.c_void_p, P(C.c_uint32)]
    L.mbg_ensemble_launches.argtypes = [C.c_void_p, P(C.c_uint64)]
    L.mbg_ensemble_stream_time.argtypes = [C.c_void_p, C.c_int,
                                           P(C.c_double)]
    L.mbg_ensemble_destroy.argtypes = [C.c_void_p]
    L.mbg_material_constants.argtypes = [C.c_char_p, P(T.mbg_material),
                                         C.c_double, C.c_int, T.PD,
                                         C.c_size_t, P(C.c_size_t)]
    L.mbg_material_constants_noalloc.argtypes = [
        C.c_char_p, P(T.mbg_material), C.c_double, C.c_void_p, C.c_size_t,
        P(C.c_size_t), C.c_void_p]
    L.mbg_material_layout.restype = C.c_size_t
    L.mbg_material_layout.argtypes = [C.c_char_p, C.c_uint32, C.c_char_p,
                                      C.c_size_t]
    L.mbg_ensemble_state_size.argtypes = [C.c_void_p, P(C.c_uint64)]
    L.mbg_ensemble_save_state.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64]
    L.mbg_ensemble_load_state.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64]
    # include/mbsolve_fno.h
    vp, i32, i64, f32, f64 = C.c_void_p, C.c_int32, C.c_int64, C.c_float, C.c_double
    L.mbg_fno_gemm.argtypes = [P(T.mbg_gemm_desc), vp]
    L.mbg_fno_spectral_layer.argtypes = [P(T.mbg_fno_layer_desc), vp]
    L.mbg_fno_mode_blocks.argtypes = [vp, vp, i32, i32, vp, vp]
    L.mbg_fno_cast_bf16.argtypes = [vp, vp, i64, vp]
    L.mbg_fno_image_bf16.argtypes = [vp, i32, i32, i32, i64, i64, i32, i32,
                                     vp, vp]
    L.mbg_fno_colsum.argtypes = [vp, i64, i32, i64, vp, vp]
    L.mbg_fno_mse.argtypes = [vp, vp, i64, vp, vp, vp]
    L.mbg_fno_adam.argtypes = [vp, vp, vp, vp, i64, f32, f32, f32, f32, f32,
                               i32, vp]
    L.mbg_fno_envelope.argtypes = [vp, i32, i32, i64, f64, f64, f64, i32,
                                   f64, f64, vp, vp]
    L.mbg_fno_status.argtypes = [P(C.c_uint32)]
    _lib = L
    return L


def check(rc):
    if rc != T.MBG_OK:
        raise MbgError(rc, load().mbg_last_error().decode())


def solver_names():
    L = load()
    n = L.mbg_solver_names(None, 0)
    buf = C.create_string_buffer(n)
    L.mbg_solver_names(buf, n)
    return buf.value.decode().split("\n")


def material_layout(algo, num_levels):
    L = load()
    n = L.mbg_material_layout(algo.encode(), num_levels, None, 0)
    buf = C.create_string_buffer(n)
    L.mbg_material_layout(algo.encode(), num_levels, buf, n)
    out = {}
    for line in buf.value.decode().split("\n"):
        k, v = line.split("=")
        out[k] = int(v)
    return out
