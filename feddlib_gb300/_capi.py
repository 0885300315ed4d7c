"""ctypes binding of the C ABI declared in include/feddgpu.h.

Loads the in-tree libfeddgpu.so.  There is no fallback: if the library is
missing, loading fails with an error that says how to build it.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfeddgpu.so")

OK, ERR_ARG, ERR_CUDA, ERR_MESH, ERR_NONFINITE, ERR_TIMEOUT, ERR_NOMEM, ERR_STATE, ERR_UNSUPPORTED, ERR_CAPACITY = range(10)
LAPLACE, LINEAR_ELASTICITY, NONLINEAR_ELASTICITY, NAVIER_STOKES, ANISO_FIBER, NONLINEAR_ELASTICITY2 = 1, 2, 3, 4, 5, 6
JACOBIAN, RESIDUAL = 1, 2


MESH_DEVICE = 1  # fedd_mesh.flags: coords / elements are device pointers


class Mesh(C.Structure):
    _fields_ = [("num_nodes", C.c_int64), ("num_elements", C.c_int64), ("fe_order", C.c_int32),
                ("flags", C.c_uint32), ("coords", C.c_void_p), ("elements", C.c_void_p),
                ("num_nodes_p", C.c_int64), ("elements_p", C.c_void_p)]


class Params(C.Structure):
    _fields_ = [("problem", C.c_int32), ("linearization", C.c_int32), ("quad_points", C.c_int32),
                ("surrogate", C.c_int32), ("viscosity", C.c_double), ("density", C.c_double),
                ("E", C.c_double), ("poisson_ratio", C.c_double), ("k1", C.c_double), ("k2", C.c_double),
                ("fiber_angle_deg", C.c_double), ("source", C.c_double)]


class MLPDesc(C.Structure):
    _fields_ = [("hidden", C.c_int32), ("in_clamp", C.c_int32), ("W1", C.c_void_p), ("b1", C.c_void_p),
                ("W2", C.c_void_p), ("b2", C.c_void_p), ("w3", C.c_void_p), ("b3", C.c_float),
                ("out_scale", C.c_float), ("in_shift", C.c_float * 4), ("in_scale", C.c_float * 4),
                ("inv_lo", C.c_float * 4), ("inv_hi", C.c_float * 4)]


class FeddError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{status_string(code)} ({code}): {msg}")
        self.code = code


_lib = None

_vp, _i32, _i64, _u32, _u64, _d, _f, _sz = (C.c_void_p, C.c_int32, C.c_int64, C.c_uint32, C.c_uint64,
                                            C.c_double, C.c_float, C.c_size_t)
SIGNATURES = {
    "fedd_abi_version": (C.c_int, []),
    "fedd_status_string": (C.c_char_p, [C.c_int]),
    "fedd_create": (C.c_int, [_vp, _vp, C.c_int, _vp]),
    "fedd_destroy": (C.c_int, [_vp]),
    "fedd_last_error": (C.c_int, [_vp, C.c_char_p, _sz]),
    "fedd_block_info": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp]),
    "fedd_get_pattern": (C.c_int, [_vp, C.c_int, _vp, _vp]),
    "fedd_device_pattern": (C.c_int, [_vp, C.c_int, _vp, _vp]),
    "fedd_residual_sizes": (C.c_int, [_vp, _vp, _vp]),
    "fedd_assemble": (C.c_int, [_vp, C.c_uint, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fedd_assemble_device": (C.c_int, [_vp, C.c_uint, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fedd_check": (C.c_int, [_vp, _vp]),
    "fedd_element_matrices": (C.c_int, [_vp, _vp, _vp, _i64, _i64, _vp, _vp]),
    "fedd_set_viscosity_law": (C.c_int, [_vp, C.c_int32, _vp, C.c_double]),
    "fedd_set_outflow_faces": (C.c_int, [_vp, _vp, C.c_int64]),
    "fedd_set_coeff": (C.c_int, [_vp, _vp]),
    "fedd_set_element_moduli": (C.c_int, [_vp, _vp]),
    "fedd_rhs_points": (C.c_int, [_vp, _vp, _vp]),
    "fedd_assemble_rhs": (C.c_int, [_vp, _vp, C.c_int32, _vp]),
    "fedd_dirichlet_set": (C.c_int, [_vp, _vp, _vp]),
    "fedd_dirichlet_system": (C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "fedd_dirichlet_rhs": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fedd_element_matrices_noalloc": (C.c_int, [_vp, _vp, _vp, _i64, _i64, _vp, _vp, _vp]),
    "fedd_element_geometry": (C.c_int, [_vp, _i64, _i64, _vp, _vp]),
    "fedd_launch_count": (C.c_int, [_vp, _vp]),
    "fedd_set_profiling": (C.c_int, [_vp, C.c_int]),
    "fedd_stage_times": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp]),
    "fedd_stage_name": (C.c_char_p, [_vp, C.c_int]),
    "fedd_set_surrogate": (C.c_int, [_vp, _vp]),
    "fedd_surrogate_fallbacks": (C.c_int, [_vp, _vp, _vp]),
    "fedd_law_eval": (C.c_int, [_vp, _i64, _vp, _vp, _vp, _vp]),
    "fedd_qp_invariants": (C.c_int, [_vp, _vp, _vp]),
    "fedd_trainer_create": (C.c_int, [_i32, _i64, _vp, _vp, _vp, C.c_int, _vp]),
    "fedd_trainer_set_params": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _f]),
    "fedd_trainer_get_params": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fedd_trainer_run": (C.c_int, [_vp, _i32, _i64, _f, _f, _f, _u64, _vp]),
    "fedd_trainer_grad": (C.c_int, [_vp, _f, _f, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fedd_trainer_destroy": (C.c_int, [_vp]),
    "fedd_mesh_sizes": (C.c_int, [_i32, _i32, _vp, _vp]),
    "fedd_mesh_structured": (C.c_int, [_i32, _i32, _u64, _d, _vp, _vp]),
    "fedd_field_fourier": (C.c_int, [_u64, _i32, _i32, _i64, _vp, _d, _vp]),
    "fedd_field_uniform": (C.c_int, [_u64, _i64, _d, _d, _vp]),
    "fedd_mesh_structured_device": (C.c_int, [_i32, _i32, _u64, _d, _vp, _vp, _vp]),
    "fedd_p2_of_p1": (C.c_int, [_i64, _i64, _vp, _vp, _u32, C.c_int, _vp, _vp]),
    "fedd_p2_copy": (C.c_int, [_vp, _vp, _vp, _u32]),
    "fedd_p2_destroy": (C.c_int, [_vp]),
    "fedd_medit_sizes": (C.c_int, [C.c_char_p, _vp, _vp, _vp]),
    "fedd_medit_read": (C.c_int, [C.c_char_p, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fedd_medit_write": (C.c_int, [C.c_char_p, _i64, _vp, _vp, _i64, _vp, _vp, _i64, _vp, _vp]),
}


def lib():
    """The loaded engine library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError(f"{LIB_PATH} is missing: build it with `python -m feddlib_gb300.build`")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def status_string(code):
    try:
        return lib().fedd_status_string(code).decode()
    except OSError:
        return "status"


def check(code, handle=None):
    """Raises FeddError for a failing status; without a handle the message is
    the calling thread's last failing handle-less call (mesh front end)."""
    if code != OK:
        buf = C.create_string_buffer(512)
        lib().fedd_last_error(handle if handle else None, buf, 512)
        raise FeddError(code, buf.value.decode(errors="replace"))
