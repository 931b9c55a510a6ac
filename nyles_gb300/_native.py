"""ctypes binding of libnyles_gb300.so (declared in include/nyles_gb300.h).

The library is built in-tree by ``python -m nyles_gb300.build`` (or
``__graft_entry__.build()``). There is no fallback: every compute call of this
package goes through the CUDA library, and importing the binding without it raises.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libnyles_gb300.so")

NYLES_OK = 0
NYLES_BAD_ARG = 1
NYLES_CUDA_ERROR = 2
NYLES_NOT_CONVERGED = 3
NYLES_BLOWUP = 4
NYLES_TIMEOUT = 5
NYLES_UNSUPPORTED = 6

MODEL = {"LES": 0, "Euler3d": 1, "linear": 2, "advection": 3}
SCHEME = {"EF": 0, "LFAM3": 1, "RK3_SSP": 2}
PRECISION = {"fp64": 0, "mixed": 1}
MG_TOPOLOGY = {"closed": 1, "perio_x": 2, "perio_y": 3, "perio_xy": 5, "perio_xyz": 6}

# NYLES_F_* field ids (state table-of-contents order)
FIELD_IDS = {"b": 0, "p": 1, "ke": 2, "div": 3, "u_i": 4, "u_j": 5, "u_k": 6,
             "U_i": 7, "U_j": 8, "U_k": 9, "vor_i": 10, "vor_j": 11, "vor_k": 12, "work": 13}
NF_BASE = 14
MAX_TRACERS = 8


class NylesError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("libnyles_gb300 error %d: %s" % (code, msg))
        self.code = code


class NotConverged(NylesError):
    pass


class BlowUp(NylesError):
    pass


class NylesDesc(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("nh", ctypes.c_int),
                ("periodic_x", ctypes.c_int), ("periodic_y", ctypes.c_int), ("periodic_z", ctypes.c_int),
                ("n_tracers", ctypes.c_int), ("model", ctypes.c_int), ("add_viscosity", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
                ("idx2", ctypes.c_double), ("idy2", ctypes.c_double), ("idz2", ctypes.c_double),
                ("dx2", ctypes.c_double), ("fparam", ctypes.c_double), ("viscosity", ctypes.c_double),
                ("tracer_diffusivity", ctypes.c_double * (MAX_TRACERS + 1)), ("tracer_diffusion", ctypes.c_int),
                ("tracer_order", ctypes.c_int), ("vf_order", ctypes.c_int)]


class NylesMgStats(ctypes.Structure):
    _fields_ = [("nite", ctypes.c_int), ("res", ctypes.c_double), ("solves", ctypes.c_longlong),
                ("vcycles", ctypes.c_longlong), ("not_converged", ctypes.c_int), ("nonfinite", ctypes.c_int)]


BATCH_RUNS = 32   # NYLES_BATCH_RUNS


class NylesBatchTable(ctypes.Structure):
    _fields_ = [("delta", ctypes.c_longlong * BATCH_RUNS), ("active", ctypes.c_int * BATCH_RUNS),
                ("live", ctypes.c_int * BATCH_RUNS), ("loop_iterations", ctypes.c_longlong)]


# user forcing callback: fn(user, reg, t, stream)
FORCING_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_void_p)

# exported symbol -> (restype, argtypes); the complete list of include/nyles_gb300.h
_P, _I, _D, _VP = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_void_p
_PP = ctypes.POINTER(ctypes.c_void_p)
SIGNATURES = {
    "nyles_last_error": (ctypes.c_char_p, []),
    "nyles_version": (_I, []),
    "nyles_flux1d_f64": (_I, [_P, _P, _P, _I, _I, _P]),
    "nyles_flux1d_f32": (_I, [_P, _P, _P, _I, _I, _P]),
    "nyles_vortex_force_f64": (_I, [ctypes.POINTER(NylesDesc), _PP, _PP, _P]),
    "nyles_vortex_force_f32": (_I, [ctypes.POINTER(NylesDesc), _PP, _PP, _P]),
    "nyles_rhs_f64": (_I, [ctypes.POINTER(NylesDesc), _PP, _PP, _I, _P]),
    "nyles_rhs_f32": (_I, [ctypes.POINTER(NylesDesc), _PP, _PP, _I, _P]),
    "nyles_fill_f64": (_I, [ctypes.POINTER(NylesDesc), _P, _P]),
    "nyles_fill_f32": (_I, [ctypes.POINTER(NylesDesc), _P, _P]),
    "nyles_mg_create": (_I, [_I, _I, _I, _I, _I, _PP]),
    "nyles_mg_destroy": (_I, [_P]),
    "nyles_mg_workspace_bytes": (_I, [_P, ctypes.POINTER(ctypes.c_size_t)]),
    "nyles_mg_bind": (_I, [_P, _P]),
    "nyles_mg_nlevels": (_I, [_P, ctypes.POINTER(ctypes.c_int)]),
    "nyles_mg_level_shape": (_I, [_P, _I, ctypes.POINTER(ctypes.c_int)]),
    "nyles_mg_level_ptr": (_I, [_P, _I, _I, _PP]),
    "nyles_mg_set_params": (_I, [_P, _D, _I, _D]),
    "nyles_mg_set_krylov": (_I, [_P, _I]),
    "nyles_mg_solve": (_I, [_P, ctypes.POINTER(NylesMgStats), _P]),
    "nyles_model_create": (_I, [ctypes.POINTER(NylesDesc), _I, _I, _PP]),
    "nyles_model_destroy": (_I, [_P]),
    "nyles_model_workspace_bytes": (_I, [_P, ctypes.POINTER(ctypes.c_size_t)]),
    "nyles_model_bind": (_I, [_P, _PP, _PP, _P]),
    "nyles_model_set_mg_params": (_I, [_P, _D, _I, _D]),
    "nyles_model_set_mg_krylov": (_I, [_P, _I]),
    "nyles_model_set_mg_warm_start": (_I, [_P, _I]),
    "nyles_model_forward": (_I, [_P, _D, _D, _P]),
    "nyles_model_diagnose": (_I, [_P, _P]),
    "nyles_model_rhs": (_I, [_P, _I, _D, _I, _P]),
    "nyles_model_project": (_I, [_P, _P]),
    "nyles_model_set_forcing": (_I, [_P, _P, _P]),
    "nyles_model_max_U2": (_I, [_P, ctypes.POINTER(ctypes.c_double), _P]),
    "nyles_model_vfwork": (_I, [_P, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_double), _P]),
    "nyles_model_mg_stats": (_I, [_P, ctypes.POINTER(NylesMgStats)]),
    "nyles_model_reset_scheme": (_I, [_P]),
    "nyles_model_get_first_step": (_I, [_P, ctypes.POINTER(ctypes.c_int)]),
    "nyles_model_set_first_step": (_I, [_P, ctypes.c_int]),
    "nyles_model_capture": (_I, [_P, _D, _I]),
    "nyles_model_graph_launch": (_I, [_P, _P]),
    "nyles_model_graph_release": (_I, [_P]),
    "nyles_model_profile": (_I, [_P, _I]),
    "nyles_model_profile_read": (_I, [_P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong), _I]),
    "nyles_model_batch_capture": (_I, [_P, _D, _I, _I, _P, _PP]),
    "nyles_batch_launch": (_I, [_P, _P]),
    "nyles_batch_note_iterations": (_I, [_P, ctypes.c_longlong]),
    "nyles_batch_destroy": (_I, [_P]),
    "nyles_model_device_stats": (_I, [_P, ctypes.POINTER(NylesMgStats), _P]),
    "nyles_launch_count": (ctypes.c_longlong, []),
    "nyles_max_U2_static_f64": (_I, [_P, _P, _P, ctypes.c_longlong, _P, _P]),
}

NPHASE = 12
PHASES = ["rhs", "update", "fill", "div", "mg_solve", "correct", "diag", "cfl", "mg_smooth", "mg_restrict",
          "mg_prolong", "mg_norm"]

_lib = None


def lib():
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                "libnyles_gb300.so is missing (%s). Build it with `python -m nyles_gb300.build`; "
                "this package has no CPU fallback." % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc):
    if rc == NYLES_OK:
        return
    msg = lib().nyles_last_error().decode(errors="replace")
    if rc == NYLES_NOT_CONVERGED:
        raise NotConverged(rc, msg)
    if rc == NYLES_BLOWUP:
        raise BlowUp(rc, msg)
    raise NylesError(rc, msg)


def ptr_array(ptrs):
    arr = (ctypes.c_void_p * len(ptrs))()
    for i, p in enumerate(ptrs):
        arr[i] = p
    return arr


def stream_ptr(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)
