"""ctypes binding of include/opflow_gpu.h (libopflow_gpu.so).

This is the only place the Python side touches the library.  Loading fails loudly when the shared
library has not been built: there is no CPU fallback behind any call.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libopflow_gpu.so")

# ---- enums (include/opflow_gpu.h) --------------------------------------------------------------------
OK, E_INVALID, E_NOMEM, E_CUDA, E_TIMEOUT, E_NOT_CONVERGED, E_UNSUPPORTED, E_RANGE, E_NAN = range(9)
CORNER, CENTER = 0, 1
BC_UNDEFINED, BC_DIRC, BC_NEUM, BC_PERIODIC, BC_SYMM, BC_ASYMM = range(6)
ASSIGN_EQ, ASSIGN_ADD, ASSIGN_SUB, ASSIGN_MUL, ASSIGN_DIV = range(5)
(NODE_FIELD, NODE_CONST, NODE_ADD, NODE_SUB, NODE_MUL, NODE_DIV, NODE_NEG, NODE_D2, NODE_D1,
 NODE_WENO53_DOWN, NODE_WENO53_UP, NODE_INTP_C2C, NODE_INTP_COR2CEN, NODE_D1_BIASED_UP,
 NODE_D1_BIASED_DOWN, NODE_GT, NODE_GE, NODE_LT, NODE_LE, NODE_NE, NODE_AND, NODE_OR, NODE_NOT, NODE_COND,
 NODE_FUNC1, NODE_FUNC2, NODE_INTP_FL_CEN2COR, NODE_INTP_FL_COR2CEN) = range(1, 29)
# enum opflow_func1 / opflow_func2 / opflow_flux_limiter
FUNC1 = {name: i for i, name in enumerate(["abs", "sqrt", "ceil", "floor", "trunc", "round", "rint"])}
FUNC1.update({name: 16 + i for i, name in enumerate(
    ["exp", "exp2", "expm1", "log", "log10", "log2", "log1p", "cbrt", "sin", "cos", "tan", "asin", "acos", "atan",
     "sinh", "cosh", "tanh", "asinh", "acosh", "atanh", "erf", "erfc", "tgamma", "lgamma"])})
FUNC1_EXACT = {"abs", "sqrt", "ceil", "floor", "trunc", "round", "rint"}
FUNC2 = {"max": 0, "min": 1, "fdim": 2, "copysign": 3, "fmod": 4, "remainder": 5, "pow": 16, "hypot": 17, "atan2": 18}
FUNC2_EXACT = {"max", "min", "fdim", "copysign", "fmod", "remainder"}
(FL_CDS, FL_QUICK, FL_CUI, FL_FROMM, FL_LUI, FL_MINMOD, FL_SUPERBEE, FL_MUSCL, FL_HARMONIC, FL_VANALBADA, FL_UMIST,
 FL_SPL13, FL_SPLMAX12, FL_SPLMAX13, FL_KOREN, FL_SMART, FL_BSOU) = range(17)
EVAL_EXACT, EVAL_FAST = 0, 1
PREC_FP64, PREC_MIXED = 0, 1

STATUS_NAMES = {OK: "OK", E_INVALID: "E_INVALID", E_NOMEM: "E_NOMEM", E_CUDA: "E_CUDA", E_TIMEOUT: "E_TIMEOUT",
                E_NOT_CONVERGED: "E_NOT_CONVERGED", E_UNSUPPORTED: "E_UNSUPPORTED", E_RANGE: "E_RANGE", E_NAN: "E_NAN"}


class MeshDesc(C.Structure):
    _fields_ = [("ndim", C.c_int), ("dims", C.c_int * 3), ("start", C.c_int * 3), ("pad_width", C.c_int),
                ("x", C.POINTER(C.c_double) * 3), ("dx", C.POINTER(C.c_double) * 3)]


class FieldDesc(C.Structure):
    _fields_ = [("ndim", C.c_int), ("loc", C.c_int * 3), ("bc_type", (C.c_int * 2) * 3),
                ("bc_value", (C.c_double * 2) * 3), ("ext", (C.c_int * 2) * 3), ("padding", C.c_int)]


class FieldInfo(C.Structure):
    _fields_ = [("ndim", C.c_int), ("padding", C.c_int), ("data_dims", C.c_int * 3), ("data_offset", C.c_int * 3),
                ("logical", (C.c_int * 2) * 3), ("accessible", (C.c_int * 2) * 3),
                ("assignable", (C.c_int * 2) * 3), ("local", (C.c_int * 2) * 3), ("count", C.c_size_t)]


class Node(C.Structure):
    _fields_ = [("kind", C.c_int), ("a", C.c_int), ("b", C.c_int), ("dim", C.c_int), ("field", C.c_int),
                ("value", C.c_double), ("c", C.c_int)]


class SolveParams(C.Structure):
    _fields_ = [("tol", C.c_double), ("max_iter", C.c_int), ("static_mat", C.c_int), ("pin_value", C.c_int),
                ("precision", C.c_int), ("pre_sweeps", C.c_int), ("post_sweeps", C.c_int), ("coarse_max", C.c_int),
                ("zero_guess", C.c_int), ("krylov", C.c_int), ("precond", C.c_int), ("kdim", C.c_int), ("abs_tol", C.c_double)]


# enum opflow_krylov / opflow_precond
KRYLOV_PCG, KRYLOV_GMRES, KRYLOV_FGMRES, KRYLOV_LGMRES, KRYLOV_BICGSTAB, KRYLOV_NONE = range(6)
PRECOND_MG, PRECOND_JACOBI, PRECOND_NONE, PRECOND_AMG = range(4)


class SolveState(C.Structure):
    _fields_ = [("iterations", C.c_int), ("rel_residual", C.c_double), ("abs_residual", C.c_double),
                ("converged", C.c_int), ("setup_ms", C.c_double), ("solve_ms", C.c_double)]


class ProblemDesc(C.Structure):
    _fields_ = [("ndim", C.c_int), ("n", C.c_int * 3), ("loc", C.c_int), ("bc", C.c_int), ("h", C.c_double * 3),
                ("alpha", C.c_double), ("beta", C.c_double)]


class Equation(C.Structure):
    _fields_ = [("nodes", C.POINTER(Node)), ("n_nodes", C.c_int), ("leaves", C.POINTER(C.c_void_p)), ("n_leaves", C.c_int),
                ("unknown", C.c_int)]


class Request(C.Structure):
    _fields_ = [("problem", ProblemDesc), ("steps", C.c_int), ("f", C.POINTER(C.c_double)), ("x_out", C.POINTER(C.c_double)),
                ("x0", C.POINTER(C.c_double)), ("equation", C.POINTER(Equation))]


class RequestResult(C.Structure):
    _fields_ = [("id", C.c_longlong), ("status", C.c_int), ("iterations", C.c_int), ("solves", C.c_int), ("rel_residual", C.c_double),
                ("queue_ms", C.c_double), ("latency_ms", C.c_double)]


class ServeStats(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("completed", C.c_longlong), ("solves", C.c_longlong), ("p50_ms", C.c_double),
                ("p99_ms", C.c_double), ("mean_ms", C.c_double), ("max_ms", C.c_double), ("elapsed_s", C.c_double),
                ("solves_per_s", C.c_double), ("max_active_seen", C.c_int), ("graph_launches", C.c_longlong),
                ("compositions", C.c_longlong), ("setup_s", C.c_double), ("compose_s", C.c_double), ("iterate_s", C.c_double),
                ("retire_s", C.c_double)]


class OpflowError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (STATUS_NAMES.get(code, code), msg))
        self.code = code


_lib = None

_SIGS = {
    "opflow_ctx_create": [C.c_int, C.POINTER(C.c_void_p)],
    "opflow_ctx_destroy": [C.c_void_p],
    "opflow_ctx_set_stream": [C.c_void_p, C.c_void_p],
    "opflow_ctx_get_stream": [C.c_void_p, C.POINTER(C.c_void_p)],
    "opflow_ctx_synchronize": [C.c_void_p],
    "opflow_kernel_launch_count": [C.POINTER(C.c_uint64)],
    "opflow_mesh_uniform": [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)],
    "opflow_field_describe": [C.POINTER(MeshDesc), C.POINTER(FieldDesc), C.POINTER(FieldInfo)],
    "opflow_field_create": [C.c_void_p, C.POINTER(MeshDesc), C.POINTER(FieldDesc), C.POINTER(C.c_void_p)],
    "opflow_field_destroy": [C.c_void_p],
    "opflow_field_get_info": [C.c_void_p, C.POINTER(FieldInfo)],
    "opflow_field_upload": [C.c_void_p, C.POINTER(C.c_double), C.c_size_t],
    "opflow_field_download": [C.c_void_p, C.POINTER(C.c_double), C.c_size_t],
    "opflow_field_device_ptr": [C.c_void_p, C.POINTER(C.c_void_p)],
    "opflow_field_update_padding": [C.c_void_p],
    "opflow_field_write_raw": [C.c_void_p, C.c_char_p, C.c_char_p, C.c_int, C.c_double],
    "opflow_assign_batch": [C.c_void_p, C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_int), C.POINTER(C.c_void_p), C.POINTER(C.c_int),
                            C.POINTER(C.c_void_p), C.POINTER(C.c_int), C.c_int],
    "opflow_tune_set_cache": [C.c_char_p],
    "opflow_tune_lookup": [C.c_char_p, C.POINTER(C.c_int)],
    "opflow_tune_stats": [C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)],
    "opflow_tune_clear": [],
    "opflow_eqnset_create": [C.c_void_p, C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_int), C.POINTER(C.c_void_p),
                             C.c_int, C.POINTER(C.c_int), C.c_void_p, C.POINTER(C.c_void_p)],
    "opflow_eqnset_solve": [C.c_void_p, C.c_void_p],
    "opflow_eqnset_csr": [C.c_void_p, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p],
    "opflow_eqnset_destroy": [C.c_void_p],
    "opflow_field_read_raw": [C.c_void_p, C.c_char_p, C.c_char_p, C.c_int, C.POINTER(C.c_double)],
    "opflow_field_fill": [C.c_void_p, C.c_int, C.c_double],
    "opflow_field_copy": [C.c_void_p, C.c_void_p],
    "opflow_assign": [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(Node), C.c_int, C.POINTER(C.c_void_p), C.c_int, C.c_int],
    "opflow_assign_repeat": [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(Node), C.c_int, C.POINTER(C.c_void_p), C.c_int,
                             C.c_int, C.c_int],
    "opflow_weno_rk3": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_int],
    "opflow_weno_rk3_mode": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int],
    "opflow_assemble": [C.c_void_p, C.c_void_p, C.POINTER(Node), C.c_int, C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int,
                        C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_double),
                        C.POINTER(C.c_size_t)],
    "opflow_solve_params_default": [C.POINTER(SolveParams)],
    "opflow_solver_create": [C.c_void_p, C.c_void_p, C.POINTER(Node), C.c_int, C.POINTER(C.c_void_p), C.c_int, C.c_int,
                             C.POINTER(SolveParams), C.POINTER(C.c_void_p)],
    "opflow_solver_solve": [C.c_void_p, C.POINTER(SolveState)],
    "opflow_solver_destroy": [C.c_void_p],
    "opflow_batch_create": [C.c_void_p, C.POINTER(ProblemDesc), C.c_int, C.POINTER(SolveParams), C.POINTER(C.c_void_p)],
    "opflow_batch_create_eqns": [C.c_void_p, C.POINTER(Equation), C.c_int, C.POINTER(SolveParams), C.POINTER(C.c_void_p)],
    "opflow_batch_vectors": [C.c_void_p, C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_size_t)],
    "opflow_batch_solve": [C.c_void_p, C.POINTER(SolveState)],
    "opflow_batch_set": [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_size_t],
    "opflow_batch_get": [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.c_size_t],
    "opflow_batch_destroy": [C.c_void_p],
    "opflow_server_create": [C.c_void_p, C.POINTER(SolveParams), C.c_size_t, C.c_int, C.POINTER(C.c_void_p)],
    "opflow_server_submit": [C.c_void_p, C.POINTER(Request), C.POINTER(C.c_longlong)],
    "opflow_server_result": [C.c_void_p, C.c_longlong, C.c_int, C.POINTER(C.c_int), C.POINTER(RequestResult)],
    "opflow_server_drain": [C.c_void_p],
    "opflow_server_checkpoint": [C.c_void_p, C.c_longlong, C.POINTER(C.c_double), C.c_size_t, C.POINTER(C.c_int)],
    "opflow_server_stats": [C.c_void_p, C.POINTER(ServeStats)],
    "opflow_server_destroy": [C.c_void_p],
    "opflow_residual_norms_noalloc": [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_void_p],
}


def declared_symbols():
    """Every function declared in include/opflow_gpu.h (parsed from the header)."""
    import re
    hdr = os.path.join(HERE, "..", "include", "opflow_gpu.h")
    txt = open(hdr).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*)\s+(opflow_\w+)\s*\(", txt, flags=re.M)))


def lib():
    """The loaded library; raises if it was not built (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise OpflowError(E_CUDA, "libopflow_gpu.so is not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
    L = C.CDLL(LIB_PATH)
    for name, args in _SIGS.items():
        fn = getattr(L, name, None)
        if fn is None:
            continue
        fn.argtypes = args
        fn.restype = None if name == "opflow_solve_params_default" else C.c_int
    L.opflow_last_error.restype = C.c_char_p
    L.opflow_last_error.argtypes = []
    L.opflow_abi_version.restype = C.c_int
    _lib = L
    return L


def check(rc):
    if rc != OK:
        raise OpflowError(rc, lib().opflow_last_error().decode(errors="replace"))
    return rc


def launch_count():
    v = C.c_uint64(0)
    check(lib().opflow_kernel_launch_count(C.byref(v)))
    return v.value
