"""ctypes binding of libgh1.so (the C ABI declared in include/gh1.h).

The library is built in-tree (``ngsolve_gb300/libgh1.so``).  There is no CPU
fallback: if the library or a CUDA device is missing, every call raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgh1.so")

GH1_OK = 0
GH1_F64, GH1_F32 = 0, 1
GH1_MEM_HOST, GH1_MEM_DEVICE = 0, 1
GH1_OP_CSR, GH1_OP_MATFREE, GH1_OP_BLOCK = 0, 1, 2
GH1_CG_FP64, GH1_CG_MIXED = 0, 1
GH1_STOP_PRECOND, GH1_STOP_TRUE = 0, 1
STATUS_NAMES = {0: "OK", 1: "ERR_ARG", 2: "ERR_CUDA", 3: "ERR_NOMEM", 4: "ERR_UNSUPPORTED",
                5: "ERR_ILLEGAL_DNUMS", 6: "MAXITER", 7: "BREAKDOWN"}


class GH1Error(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (STATUS_NAMES.get(code, "?"), code, msg))
        self.code = code


class CGOpts(ctypes.Structure):
    _fields_ = [("tol", ctypes.c_double), ("maxit", ctypes.c_int), ("mode", ctypes.c_int),
                ("stop_rule", ctypes.c_int), ("initialize", ctypes.c_int), ("inner_tol", ctypes.c_double),
                ("max_outer", ctypes.c_int), ("check_every", ctypes.c_int), ("res_hist", ctypes.c_void_p)]


class CGResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("iterations", ctypes.c_int), ("outer", ctypes.c_int),
                ("applies64", ctypes.c_int), ("applies32", ctypes.c_int), ("first_res", ctypes.c_double),
                ("final_res", ctypes.c_double), ("true_relres", ctypes.c_double)]


# name -> argtypes (restype int unless noted)
_P, _I, _L, _D = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double
_PP = ctypes.POINTER(ctypes.c_void_p)
SIGNATURES = {
    "gh1_create": [_PP, _I],
    "gh1_destroy": [_P],
    "gh1_set_stream": [_P, _P],
    "gh1_last_error": [_P],
    "gh1_version": [],
    "gh1_mesh_upload": [_P, _I, _P, _I, _I, _P, _PP],
    "gh1_mesh_free": [_P],
    "gh1_mesh_set_deformation": [_P, _P, _P, _I],
    "gh1_space_h1": [_P, _I, _I, _PP],
    "gh1_space_h1_bnd": [_P, _I, _L, _P, _PP],
    "gh1_space_free": [_P],
    "gh1_space_info": [_P, _P],
    "gh1_space_get_dofs": [_P, _P],
    "gh1_space_get_freedofs": [_P, _P],
    "gh1_shape_eval": [_P, _I, _I, _P, _I, _P, _P, _P],
    "gh1_form_create": [_P, _P, _P, _I, _PP],
    "gh1_form_set_coefs": [_P, _P, _P, _I],
    "gh1_form_set_tensor": [_P, _P, _I],
    "gh1_form_set_bdb": [_P, _P, _I, _I],
    "gh1_space_qpoints": [_P, _P, _P, _I, _P],
    "gh1_form_free": [_P],
    "gh1_assemble_csr": [_P, _PP],
    "gh1_csr_info": [_P, _P],
    "gh1_csr_export": [_P, _P, _P, _P, _I],
    "gh1_csr_import": [_P, _L, _L, _P, _P, _P, _I, _PP],
    "gh1_matfree_create": [_P, _I, _PP],
    "gh1_op_apply": [_P, _D, _P, _P, _I, _I],
    "gh1_op_info": [_P, _P],
    "gh1_op_check": [_P],
    "gh1_op_free": [_P],
    "gh1_op_block_create": [_P, _I, _PP],
    "gh1_jacobi_create": [_P, _P, _I, _PP],
    "gh1_pre_apply": [_P, _D, _P, _P, _I, _I],
    "gh1_pre_free": [_P],
    "gh1_space_smoothing_blocks": [_P, _I, _P, _P, _P, _P],
    "gh1_blockjacobi_create": [_P, _L, _P, _P, _I, _PP],
    "gh1_coarse_create": [_P, _L, _P, _P, _I, _PP],
    "gh1_pre_sum": [_P, _P, _PP],
    "gh1_rhs_elementwise": [_P, _P, _I, _P],
    "gh1_cg": [_P, _P, _P, _P, ctypes.POINTER(CGOpts), ctypes.POINTER(CGResult)],
    "gh1_elem_grad_dot": [_P, _P, _P, _P],
    "gh1_adjoint_grad": [_P, _P, _P, _D, _P, _P, _P, _P],
    "gh1_batch_create": [_P, _I, _P, _P, _PP],
    "gh1_batch_solve": [_P, _P, _P, ctypes.POINTER(CGOpts), _P],
    "gh1_batch_free": [_P],
    "gh1_shape_eval_noalloc": [_P, _I, _I, _P, _I, _P, _P, _P],
    "gh1_projector_create": [_P, _L, _P, _I, _I, _PP],
    "gh1_projector_apply": [_P, _D, _P, _P, _I, _I],
    "gh1_projector_project": [_P, _P, _I],
    "gh1_projector_free": [_P],
}

_lib = None


def load(path=LIB_PATH):
    """Load libgh1.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise GH1Error(4, "libgh1.so not built: run `python -m ngsolve_gb300.build` (no CPU fallback exists)")
    L = ctypes.CDLL(path)
    for name, args in SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = ctypes.c_char_p if name == "gh1_last_error" else ctypes.c_int
    _lib = L
    return L


def check(rc, ctx):
    if rc != GH1_OK:
        msg = load().gh1_last_error(ctx)
        raise GH1Error(rc, msg.decode() if msg else "")
